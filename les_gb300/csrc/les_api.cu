// C ABI of the GB300 LES core: context set-up, state transfer and the
// per-routine entry points declared in include/les_gb300.h.
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <memory>
#include <vector>
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include "les_internal.h"

static thread_local char g_err[512] = "";
unsigned long long g_les_launches = 0;
namespace les {
ProfSession* g_prof = nullptr;
bool prof_mark(int family, cudaStream_t s) {
  ProfSession* p = g_prof;
  if (!p || p->family != family || p->stream != s || p->n >= p->cap) return false;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return false;
  return cudaEventRecord(p->ev[2 * p->n], s) == cudaSuccess;
}
void prof_done(cudaStream_t s, double bytes) {
  ProfSession* p = g_prof;
  if (!p) return;
  if (cudaEventRecord(p->ev[2 * p->n + 1], s) == cudaSuccess) {
    p->bytes += bytes;
    p->n += 1;
  }
}
}  // namespace les
void les_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

namespace les {

static bool is_2a3b(int n) {
  if (n <= 0) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  return n == 1;
}

// (re, im) as float-float pairs: hi = the nearest float, lo = the nearest
// float to the remainder
static float4 ff_pair(long double re, long double im) {
  const float rh = (float)re, ih = (float)im;
  return make_float4(rh, (float)(re - (long double)rh), ih, (float)(im - (long double)ih));
}
// Stockham plan for a complex FFT of length n: radix 4, then 2, then 3.
// Twiddles exp(-2 pi i k r / (Ns R)) are evaluated in long double.
static int make_plan(les_ctx* c, int n, HostPlan& hp) {
  FftPlanDev& P = hp.c;
  P.n = n;
  P.nst = 0;
  int m = n;
  while (m % 4 == 0) { P.radix[P.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { P.radix[P.nst++] = 2; m /= 2; }
  while (m % 3 == 0) { P.radix[P.nst++] = 3; m /= 3; }
  if (m != 1 || P.nst > FFT_MAX_STAGES) { les_set_error("FFT size %d is not 2^a 3^b", n); return LES_ERR_UNSUPPORTED; }
  if (n > 4096) { les_set_error("FFT size %d exceeds 4096", n); return LES_ERR_UNSUPPORTED; }
  std::vector<double2> tw;
  std::vector<float4> twd;
  int Ns = 1;
  for (int s = 0; s < P.nst; ++s) {
    const int R = P.radix[s];
    P.dm[s] = FastDiv((unsigned)(n / R));
    P.dns[s] = FastDiv((unsigned)Ns);
    P.twoff[s] = (int)tw.size();
    for (int r = 1; r < R; ++r)
      for (int k = 0; k < Ns; ++k) {
        const long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)((long long)k * r) /
                                (long double)((long long)Ns * R);
        const long double cr = cosl(ang), ci = sinl(ang);
        tw.push_back(make_double2((double)cr, (double)ci));
        twd.push_back(ff_pair(cr, ci));
      }
    Ns *= R;
  }
  if (tw.empty()) {
    tw.push_back(make_double2(1.0, 0.0));
    twd.push_back(ff_pair(1.0L, 0.0L));
  }
  LES_CUDA_CHECK(cudaMalloc(&hp.devd, twd.size() * sizeof(float4)));
  c->allocs.push_back(hp.devd);
  LES_CUDA_CHECK(cudaMemcpy(hp.devd, twd.data(), twd.size() * sizeof(float4), cudaMemcpyHostToDevice));
  P.twd = static_cast<const float4*>(hp.devd);
  {  // unit-circle tables exp(-2 pi i m / n), m < n
    std::vector<float2> uf(n);
    std::vector<float4> ud(n);
    for (int mm = 0; mm < n; ++mm) {
      const long double ang = -2.0L * 3.14159265358979323846264338327950288L * mm / (long double)n;
      uf[mm] = make_float2((float)cosl(ang), (float)sinl(ang));
      ud[mm] = ff_pair(cosl(ang), sinl(ang));
    }
    LES_CUDA_CHECK(cudaMalloc(&hp.devuf, uf.size() * sizeof(float2)));
    c->allocs.push_back(hp.devuf);
    LES_CUDA_CHECK(cudaMemcpy(hp.devuf, uf.data(), uf.size() * sizeof(float2), cudaMemcpyHostToDevice));
    LES_CUDA_CHECK(cudaMalloc(&hp.devud, ud.size() * sizeof(float4)));
    c->allocs.push_back(hp.devud);
    LES_CUDA_CHECK(cudaMemcpy(hp.devud, ud.data(), ud.size() * sizeof(float4), cudaMemcpyHostToDevice));
    P.unitf = static_cast<const float2*>(hp.devuf);
    P.unitd = static_cast<const float4*>(hp.devud);
  }
  LES_CUDA_CHECK(cudaMalloc(&hp.dev, tw.size() * sizeof(double2)));
  c->allocs.push_back(hp.dev);
  LES_CUDA_CHECK(cudaMemcpy(hp.dev, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice));
  P.tw = hp.dev;
  std::vector<float2> twf(tw.size());
  for (size_t i = 0; i < tw.size(); ++i) twf[i] = make_float2((float)tw[i].x, (float)tw[i].y);
  LES_CUDA_CHECK(cudaMalloc(&hp.devf, twf.size() * sizeof(float2)));
  c->allocs.push_back(hp.devf);
  LES_CUDA_CHECK(cudaMemcpy(hp.devf, twf.data(), twf.size() * sizeof(float2), cudaMemcpyHostToDevice));
  P.twf = hp.devf;
  return 0;
}
static int make_real_plan(les_ctx* c, int nx, HostRealPlan& rp) {
  HostPlan hp;
  int st = make_plan(c, nx / 2, hp);
  if (st) return st;
  rp.r.c = hp.c;
  rp.r.nx = nx;
  const int m = nx / 2;
  rp.r.dm = FastDiv((unsigned)m);
  rp.r.dm1 = FastDiv((unsigned)(m + 1));
  std::vector<double2> w(m + 1);
  std::vector<float4> wd(m + 1);
  for (int k = 0; k <= m; ++k) {
    const long double ang = -2.0L * 3.14159265358979323846264338327950288L * k / (long double)nx;
    w[k] = make_double2((double)cosl(ang), (double)sinl(ang));
    wd[k] = ff_pair(cosl(ang), sinl(ang));
  }
  LES_CUDA_CHECK(cudaMalloc(&rp.devd, wd.size() * sizeof(float4)));
  c->allocs.push_back(rp.devd);
  LES_CUDA_CHECK(cudaMemcpy(rp.devd, wd.data(), wd.size() * sizeof(float4), cudaMemcpyHostToDevice));
  rp.r.wd = static_cast<const float4*>(rp.devd);
  LES_CUDA_CHECK(cudaMalloc(&rp.dev, w.size() * sizeof(double2)));
  c->allocs.push_back(rp.dev);
  LES_CUDA_CHECK(cudaMemcpy(rp.dev, w.data(), w.size() * sizeof(double2), cudaMemcpyHostToDevice));
  rp.r.w = rp.dev;
  std::vector<float2> wf(w.size());
  for (size_t i = 0; i < w.size(); ++i) wf[i] = make_float2((float)w[i].x, (float)w[i].y);
  LES_CUDA_CHECK(cudaMalloc(&rp.devf, wf.size() * sizeof(float2)));
  c->allocs.push_back(rp.devf);
  LES_CUDA_CHECK(cudaMemcpy(rp.devf, wf.data(), wf.size() * sizeof(float2), cudaMemcpyHostToDevice));
  rp.r.wf = rp.devf;
  return 0;
}

static int dalloc(les_ctx* c, void** p, size_t bytes) {
  if (bytes == 0) bytes = 256;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    les_set_error("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    return LES_ERR_OOM;
  }
  c->allocs.push_back(*p);
  c->bytes += bytes;
  LES_CUDA_CHECK(cudaMemset(*p, 0, bytes));
  return 0;
}

static void grid_of(const les_config& k, Grid& g) {
  g.nx = k.nx; g.ny = k.ny; g.nz = k.nz;
  g.nx2 = 3 * g.nx / 2; g.ny2 = 3 * g.ny / 2;          // param.f90:59
  g.lh = g.nx / 2 + 1; g.ld = 2 * g.lh;                 // param.f90:60
  g.lh_big = g.nx2 / 2 + 1; g.ld_big = 2 * g.lh_big;
  g.dz = (k.lz_over_zi * k.z_i) / k.z_i / (g.nz - 1);   // param.f90:64
  g.dx = k.l_x / g.nx; g.dy = k.l_y / g.ny;            // param.f90:65
  g.delta = 1.0 * std::pow(g.dx * g.dy, 1.0 / 2.0);     // sgs_stag.f90:43
  g.nplane = (size_t)g.ld * g.ny;
  g.nfield = g.nplane * g.nz;
  g.nplane_big = (size_t)g.ld_big * g.ny2;
  g.nfield_big = g.nplane_big * g.nz;
  g.C = (size_t)g.ny * g.lh;
  g.CB = (size_t)g.ny2 * (g.nx / 2);
}

struct Sizes {
  size_t wsA, wsB, wsP, big, tmp, fields, surf, spare, aux;
  int lag_chunk, ntmp;
};
static Sizes sizes_of(const Grid& g, bool q, bool m7) {
  Sizes s{};
  s.lag_chunk = std::min(32, g.nz);
  const size_t nz = g.nz, C = g.C, CB = g.CB, ch = s.lag_chunk;
  s.wsA = std::max({6 * nz * C, 21 * ch * C, 3 * nz * CB, (size_t)(g.nx2 / 2 + 1) * g.ny2 * 2}) * sizeof(double2);
  s.wsB = std::max({9 * nz * C, 6 * nz * CB, 42 * ch * C, (size_t)(g.nx2 / 2 + 1) * g.ny2 * 2}) * sizeof(double2);
  s.wsP = ((3 * (nz - 1) + 2 + (nz + 1)) * C) * sizeof(double2) + (nz + 1) * C * sizeof(double);
  s.big = 9 * g.nfield_big * sizeof(double);
  s.ntmp = (int)std::max<size_t>(63 * ch, 3 * nz + 2);
  s.tmp = (size_t)s.ntmp * g.nplane * sizeof(double);
  s.fields = 0;
  for (int f = 0; f < LES_ZO; ++f)
    if ((q || !is_q_field(f)) && (m7 || !is_m7_field(f)))
      s.fields += (f == LES_P ? g.nplane * (nz + 1) : g.nfield) * sizeof(double);
  s.surf = (size_t)(LES_NUM_FIELDS - LES_ZO + 1 - (q ? 0 : 2)) * g.nx * g.ny * sizeof(double);
  s.spare = 4 * g.nfield * sizeof(double) + (4 * nz + 4) * C * sizeof(double2) + 2 * (nz + 1) * C * sizeof(double);
  // saved spectra, wall-plane spectra, Thomas tables, reductions, wavenumber
  // and filter tables (FP64 + FP32)
  s.aux = 4 * nz * C * sizeof(double2) + 4 * C * sizeof(double2) + 2 * (nz + 1) * C * sizeof(double) +
          (36 * (nz + 8) + 64) * sizeof(double) + 5 * C * sizeof(double) + 4 * C * sizeof(float) +
          2 * C * sizeof(float2);
  return s;
}

static void wavenumbers(const les_config& k, const Grid& g, std::vector<double>& kx, std::vector<double>& ky,
                        std::vector<double>& k2) {
  // fft.f90:54-81
  const int lh = g.lh, ny = g.ny;
  kx.assign((size_t)lh * ny, 0.0); ky.assign((size_t)lh * ny, 0.0); k2.assign((size_t)lh * ny, 0.0);
  for (int jy = 0; jy < ny; ++jy)
    for (int jx = 0; jx < lh - 1; ++jx) kx[(size_t)jy * lh + jx] = (double)jx;
  for (int jy = 0; jy < ny; ++jy) {
    const int m = ((jy + ny / 2) % ny) - ny / 2;
    for (int jx = 0; jx < lh; ++jx) ky[(size_t)jy * lh + jx] = (double)m;
  }
  for (int jy = 0; jy < ny; ++jy) { kx[(size_t)jy * lh + lh - 1] = 0.0; ky[(size_t)jy * lh + lh - 1] = 0.0; }
  for (int jx = 0; jx < lh; ++jx) { kx[(size_t)(ny / 2) * lh + jx] = 0.0; ky[(size_t)(ny / 2) * lh + jx] = 0.0; }
  const double fx = 2.0 * LES_PI / k.l_x, fy = 2.0 * LES_PI / k.l_y;
  for (size_t i = 0; i < kx.size(); ++i) {
    kx[i] = fx * kx[i];
    ky[i] = fy * ky[i];
    k2[i] = kx[i] * kx[i] + ky[i] * ky[i];
  }
}
// test_filtermodule.f90:32-63 (ifilter = 1)
static void filter_G(const Grid& g, const std::vector<double>& k2, double alpha, std::vector<double>& G) {
  G.assign((size_t)g.lh * g.ny, 1.0 / (double)(g.nx * g.ny));
  const double delta = alpha * std::sqrt(g.dx * g.dy);
  const double q = LES_PI / delta;
  const double kc2 = q * q;
  for (size_t i = 0; i < G.size(); ++i)
    if (k2[i] >= kc2) G[i] = 0.0;
  for (int jy = 0; jy < g.ny; ++jy) G[(size_t)jy * g.lh + g.lh - 1] = 0.0;
  for (int jx = 0; jx < g.lh; ++jx) G[(size_t)(g.ny / 2) * g.lh + jx] = 0.0;
}

static size_t felems(const les_ctx* c, int f) {
  if (is_q_field(f) && !c->cfg.q_flag) return 0;  // humidity arrays exist only with q_flag
  if (is_m7_field(f) && c->cfg.model != 7) return 0;  // model-7 arrays exist only with model 7
  if (f >= LES_ZO) return (size_t)c->g.nx * c->g.ny;
  if (f == LES_P) return c->g.nplane * (c->g.nz + 1);
  return c->g.nfield;
}

}  // namespace les

using namespace les;

extern "C" {

const char* les_last_error(void) { return g_err; }
unsigned long long les_kernel_launch_count(void) { return g_les_launches; }

size_t les_estimate_device_bytes(const les_config* cfg) {
  if (!cfg) return 0;
  Grid g;
  grid_of(*cfg, g);
  Sizes s = sizes_of(g, cfg->q_flag != 0, cfg->model == 7);
  size_t mixed = 0;  // float-float Thomas tables of the FP32-mixed form
  if (cfg->precision == 1) mixed = 2 * (size_t)(g.nz + 1) * g.C * sizeof(float2) + 64 * sizeof(int);
  return s.wsA + s.wsB + s.wsP + s.big + s.tmp + s.fields + s.surf + s.spare + s.aux + mixed + (1u << 20);
}

int les_ctx_create(const les_config* cfg, les_ctx** out) {
  if (!cfg || !out) { les_set_error("null argument"); return LES_ERR_ARG; }
  *out = nullptr;
  const les_config& k = *cfg;
  if (k.nx < 8 || k.ny < 8 || k.nz < 4 || k.nx % 4 || k.ny % 2 || !is_2a3b(k.nx) || !is_2a3b(k.ny)) {
    les_set_error("unsupported grid %dx%dx%d: nx%%4 == 0, ny%%2 == 0, both 2^a 3^b, nz >= 4", k.nx, k.ny, k.nz);
    return LES_ERR_ARG;
  }
  if (k.cs_count < 1 || k.dt <= 0.0 || k.z_i <= 0.0 || k.u_star <= 0.0 || k.lz_over_zi <= 0.0) {
    les_set_error("invalid physical parameters");
    return LES_ERR_ARG;
  }
  if (k.precision < 0 || k.precision > 2) { les_set_error("precision must be 0, 1 or 2"); return LES_ERR_ARG; }
  if (k.q_flag != 0 && (k.q_flag != 1 || !k.s_flag || !(k.q_scale > 0.0))) {
    les_set_error("q_flag = 1 needs s_flag = 1 and q_scale > 0");
    return LES_ERR_ARG;
  }
  if (k.model == 7 && (k.precision == 1 || !k.s_flag)) {
    les_set_error("model 7 needs s_flag = 1 and precision 0 or 2");
    return LES_ERR_UNSUPPORTED;
  }
  if (k.model != 5 && k.model != 4 && k.model != 3 && k.model != 2 && k.model != 7) {
    les_set_error("model must be 7, 5, 4, 3 or 2");
    return LES_ERR_UNSUPPORTED;
  }
  if (k.precision == 1 && k.model != 5) {  // the plane-averaged models read S_ij in FP64
    les_set_error("the FP32-mixed form (precision 1) runs model 5");
    return LES_ERR_UNSUPPORTED;
  }
  les_ctx* c = new les_ctx();
  c->cfg = k;
  c->jt_total = k.jt_total0;
  grid_of(k, c->g);
  const Grid& g = c->g;
  int st = 0;
  auto fail = [&](int code) { les_ctx_destroy(c); return code; };
  if (cudaGetDevice(&c->device) != cudaSuccess) { les_set_error("no CUDA device"); delete c; return LES_ERR_CUDA; }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    les_set_error("stream creation failed"); delete c; return LES_ERR_CUDA;
  }
  c->own_stream = true;
  for (int f = 0; f < LES_NUM_FIELDS; ++f) {
    c->fsize[f] = felems(c, f);
    if (c->fsize[f] == 0) continue;  // not stored in this configuration (null pointer)
    if ((st = dalloc(c, (void**)&c->f[f], c->fsize[f] * sizeof(double)))) return fail(st);
  }
  if ((st = dalloc(c, (void**)&c->z_os, (size_t)g.nx * g.ny * sizeof(double)))) return fail(st);
  if (k.model == 7) {  // Pr_t starts at Pr (the reference reads it from the restart record)
    std::vector<double> pr(g.nfield, k.pr);
    cudaMemcpy(c->f[LES_PR_T], pr.data(), pr.size() * sizeof(double), cudaMemcpyHostToDevice);
  }
  {  // phi_m = phi_h = 1 (set by obukhov before first use in any case)
    std::vector<double> one((size_t)g.nx * g.ny, 1.0);
    cudaMemcpy(c->f[LES_PHI_M], one.data(), one.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(c->f[LES_PHI_H], one.data(), one.size() * sizeof(double), cudaMemcpyHostToDevice);
  }
  std::vector<double> kx, ky, k2, G, GG;
  wavenumbers(k, g, kx, ky, k2);
  filter_G(g, k2, 2.0 * 1.0, G);   // main.f90:166 (filter_size = 1)
  filter_G(g, k2, 4.0 * 1.0, GG);  // main.f90:169
  {  // the filters are cutoffs: columns beyond the last nonzero one are zero for every ky
    auto ncols = [&](const std::vector<double>& T) {
      int n = 0;
      for (int jy = 0; jy < g.ny; ++jy)
        for (int jx = 0; jx < g.lh; ++jx)
          if (T[(size_t)jy * g.lh + jx] != 0.0 && jx + 1 > n) n = jx + 1;
      return n;
    };
    c->ncG = ncols(G);
    c->ncGG = ncols(GG);
  }
  const size_t tb = (size_t)g.lh * g.ny * sizeof(double);
  if ((st = dalloc(c, (void**)&c->kx, tb)) || (st = dalloc(c, (void**)&c->ky, tb)) ||
      (st = dalloc(c, (void**)&c->G, tb)) || (st = dalloc(c, (void**)&c->GG, tb)))
    return fail(st);
  cudaMemcpy(c->kx, kx.data(), tb, cudaMemcpyHostToDevice);
  cudaMemcpy(c->ky, ky.data(), tb, cudaMemcpyHostToDevice);
  cudaMemcpy(c->G, G.data(), tb, cudaMemcpyHostToDevice);
  cudaMemcpy(c->GG, GG.data(), tb, cudaMemcpyHostToDevice);
  {
    const size_t tf = (size_t)g.lh * g.ny * sizeof(float);
    if ((st = dalloc(c, (void**)&c->kxf, tf)) || (st = dalloc(c, (void**)&c->kyf, tf)) ||
        (st = dalloc(c, (void**)&c->Gf, tf)) || (st = dalloc(c, (void**)&c->GGf, tf)))
      return fail(st);
    std::vector<float> a(kx.size());
    for (size_t i = 0; i < a.size(); ++i) a[i] = (float)kx[i];
    cudaMemcpy(c->kxf, a.data(), tf, cudaMemcpyHostToDevice);
    for (size_t i = 0; i < a.size(); ++i) a[i] = (float)ky[i];
    cudaMemcpy(c->kyf, a.data(), tf, cudaMemcpyHostToDevice);
    for (size_t i = 0; i < a.size(); ++i) a[i] = (float)G[i];
    cudaMemcpy(c->Gf, a.data(), tf, cudaMemcpyHostToDevice);
    for (size_t i = 0; i < a.size(); ++i) a[i] = (float)GG[i];
    cudaMemcpy(c->GGf, a.data(), tf, cudaMemcpyHostToDevice);
    const size_t td = kx.size() * sizeof(float2);
    if ((st = dalloc(c, (void**)&c->kxd, td)) || (st = dalloc(c, (void**)&c->kyd, td))) return fail(st);
    std::vector<float2> p2(kx.size());
    for (size_t i = 0; i < p2.size(); ++i) p2[i] = make_float2((float)kx[i], (float)(kx[i] - (double)(float)kx[i]));
    cudaMemcpy(c->kxd, p2.data(), td, cudaMemcpyHostToDevice);
    for (size_t i = 0; i < p2.size(); ++i) p2[i] = make_float2((float)ky[i], (float)(ky[i] - (double)(float)ky[i]));
    cudaMemcpy(c->kyd, p2.data(), td, cudaMemcpyHostToDevice);
  }
  if ((st = make_real_plan(c, g.nx, c->rx)) || (st = make_real_plan(c, g.nx2, c->rxb)) ||
      (st = make_plan(c, g.ny, c->cy)) || (st = make_plan(c, g.ny2, c->cyb)))
    return fail(st);
  Sizes s = sizes_of(g, k.q_flag != 0, k.model == 7);
  c->lag_chunk = s.lag_chunk;
  c->ntmp = s.ntmp;
  c->nbig = 9;
  if ((st = dalloc(c, &c->wsA, s.wsA)) || (st = dalloc(c, &c->wsB, s.wsB)) || (st = dalloc(c, &c->wsP, s.wsP)) ||
      (st = dalloc(c, (void**)&c->big, s.big)) || (st = dalloc(c, (void**)&c->tmp, s.tmp)) ||
      (st = dalloc(c, (void**)&c->spare, s.spare)) || (st = dalloc(c, (void**)&c->dscal, 64 * sizeof(double))) ||
      (st = dalloc(c, (void**)&c->dred, 36 * (size_t)(g.nz + 8) * sizeof(double))) ||
      (st = dalloc(c, (void**)&c->spec, 4 * (size_t)g.nz * g.C * sizeof(double2))) ||
      (st = dalloc(c, (void**)&c->wspec, 4 * g.C * sizeof(double2))) ||
      (st = dalloc(c, (void**)&c->ibet, (size_t)(g.nz + 1) * g.C * sizeof(double))) ||
      (st = dalloc(c, (void**)&c->gamt, (size_t)(g.nz + 1) * g.C * sizeof(double))))
    return fail(st);
  if (k.precision == 1) {  // the mixed form's float-float pressure solve
    c->nlow_cap = 64;
    if ((st = dalloc(c, (void**)&c->ibet_ff, (size_t)(g.nz + 1) * g.C * sizeof(float2))) ||
        (st = dalloc(c, (void**)&c->gamt_ff, (size_t)(g.nz + 1) * g.C * sizeof(float2))) ||
        (st = dalloc(c, (void**)&c->lowmodes, (size_t)c->nlow_cap * sizeof(int))))
      return fail(st);
  }
  if ((st = thomas_tables(c))) return fail(st);
  c->wsA_bytes = s.wsA; c->wsB_bytes = s.wsB; c->wsP_bytes = s.wsP;
  if (cudaMallocHost(&c->host_scal, 64 * sizeof(double)) != cudaSuccess) { les_set_error("pinned alloc failed"); return fail(LES_ERR_OOM); }
  if (cudaDeviceSynchronize() != cudaSuccess) { les_set_error("%s", cudaGetErrorString(cudaGetLastError())); return fail(LES_ERR_CUDA); }
  *out = c;
  return LES_OK;
}

int les_ctx_destroy(les_ctx* c) {
  if (!c) return LES_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int p = 0; p < 2; ++p)
        if (c->gexec[a][b][p]) cudaGraphExecDestroy(c->gexec[a][b][p]);
  for (void* p : c->allocs) cudaFree(p);
  if (c->host_scal) cudaFreeHost(c->host_scal);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return LES_OK;
}

int les_ctx_set_pointer_mode(les_ctx* c, int device_pointers) {
  if (!c) return LES_ERR_ARG;
  c->ptr_mode = device_pointers ? 1 : 0;
  return LES_OK;
}
void* les_ctx_stream(les_ctx* c) { return c ? (void*)c->stream : nullptr; }
int les_ctx_set_priority(les_ctx* c, int priority) {
  if (!c) return LES_ERR_ARG;
  if (!c->own_stream) { les_set_error("the context does not own its stream"); return LES_ERR_STATE; }
  int lo = 0, hi = 0;
  LES_CUDA_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));  // lo least urgent, hi most urgent
  const int p = std::max(hi, std::min(lo, priority));
  cudaStream_t s = nullptr;
  LES_CUDA_CHECK(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, p));
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    cudaStreamDestroy(s);
    les_set_error("%s", cudaGetErrorString(cudaGetLastError()));
    return LES_ERR_CUDA;
  }
  cudaStreamDestroy(c->stream);
  c->stream = s;
  return LES_OK;
}
size_t les_ctx_device_bytes(const les_ctx* c) { return c ? c->bytes : 0; }

int les_set_surface(les_ctx* c, const double* zo, const double* wt_s) {
  if (!c || !zo || !wt_s) return LES_ERR_ARG;
  const size_t n = (size_t)c->g.nx * c->g.ny;
  std::vector<double> zos(n);
  for (size_t i = 0; i < n; ++i) {
    if (!(zo[i] > 0.0)) { les_set_error("zo must be positive"); return LES_ERR_ARG; }
    zos[i] = zo[i] / 7.39;  // bottombc.f90:274 with zom/z_i = zo
  }
  LES_CUDA_CHECK(cudaMemcpyAsync(c->f[LES_ZO], zo, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  LES_CUDA_CHECK(cudaMemcpyAsync(c->f[LES_WT_S], wt_s, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  LES_CUDA_CHECK(cudaMemcpyAsync(c->z_os, zos.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  c->surface_set = true;
  return LES_OK;
}

// host <-> device copy of one field; the FP32-held fields of a mixed
// context are narrowed / widened on the host
static bool f32_held(const les_ctx* c, int f) { return c->cfg.precision == 1 && mixed_f32_field(f); }
static bool ff_held(const les_ctx* c, int f) { return c->cfg.precision == 1 && mixed_ff_field(f); }
static int field_in(les_ctx* c, int f, const double* host) {
  const size_t n = c->fsize[f];
  if (ff_held(c, f)) {  // hi = the value rounded to FP32, lo = the rest rounded to FP32
    std::vector<float> t(2 * n);
    for (size_t i = 0; i < n; ++i) {
      const float h = (float)host[i];
      t[2 * i] = h;
      t[2 * i + 1] = (float)(host[i] - (double)h);
    }
    LES_CUDA_CHECK(cudaMemcpyAsync(c->f[f], t.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return LES_OK;
  }
  if (f32_held(c, f)) {
    std::vector<float> t(n);
    for (size_t i = 0; i < n; ++i) t[i] = (float)host[i];
    LES_CUDA_CHECK(cudaMemcpyAsync(c->f[f], t.data(), n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return LES_OK;
  }
  LES_CUDA_CHECK(cudaMemcpyAsync(c->f[f], host, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return LES_OK;
}
static int field_out(les_ctx* c, int f, double* host) {
  const size_t n = c->fsize[f];
  if (ff_held(c, f)) {
    std::vector<float> t(2 * n);
    LES_CUDA_CHECK(cudaMemcpyAsync(t.data(), c->f[f], n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; ++i) host[i] = (double)t[2 * i] + (double)t[2 * i + 1];
    return LES_OK;
  }
  if (f32_held(c, f)) {
    std::vector<float> t(n);
    LES_CUDA_CHECK(cudaMemcpyAsync(t.data(), c->f[f], n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; ++i) host[i] = (double)t[i];
    return LES_OK;
  }
  LES_CUDA_CHECK(cudaMemcpyAsync(host, c->f[f], n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return LES_OK;
}
static int absent(const les_ctx* c, int f) {
  if (c->fsize[f]) return LES_OK;
  les_set_error("field %d is not stored in this context (humidity arrays need q_flag = 1)", f);
  return LES_ERR_STATE;
}
int les_set_field(les_ctx* c, les_field f, const double* host) {
  if (!c || !host || f < 0 || f >= LES_NUM_FIELDS) return LES_ERR_ARG;
  if (int a = absent(c, f)) return a;
  int st = field_in(c, f, host);
  if (st) return st;
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  return LES_OK;
}
int les_get_field(les_ctx* c, les_field f, double* host) {
  if (!c || !host || f < 0 || f >= LES_NUM_FIELDS) return LES_ERR_ARG;
  if (int a = absent(c, f)) return a;
  int st = field_out(c, f, host);
  if (st) return st;
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  return LES_OK;
}
double* les_field_device_ptr(les_ctx* c, les_field f) {
  if (!c || f < 0 || f >= LES_NUM_FIELDS) return nullptr;
  return c->f[f];
}
size_t les_field_elems(const les_ctx* c, les_field f) {
  if (!c || f < 0 || f >= LES_NUM_FIELDS) return 0;
  return c->fsize[f];
}
int les_register_field(les_ctx* c, les_field f, double* host) {
  if (!c || f < 0 || f >= LES_NUM_FIELDS) return LES_ERR_ARG;
  c->reg[f] = host;
  return LES_OK;
}
int les_sync_from_host(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  for (int f = 0; f < LES_NUM_FIELDS; ++f)
    if (c->reg[f]) {
      int st = field_in(c, f, c->reg[f]);
      if (st) return st;
    }
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  return LES_OK;
}
int les_sync_to_host(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  for (int f = 0; f < LES_NUM_FIELDS; ++f)
    if (c->reg[f]) {
      int st = field_out(c, f, c->reg[f]);
      if (st) return st;
    }
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  return LES_OK;
}
int les_get_counters(les_ctx* c, int* jt, int* jt_total) {
  if (!c) return LES_ERR_ARG;
  if (jt) *jt = c->jt;
  if (jt_total) *jt_total = c->jt_total;
  return LES_OK;
}

// ---- whole-member state image (serving: spill an evicted member to host
// memory and resume it later exactly where it stopped) ----------------------
namespace {
struct StateHeader {
  char magic[8];            // "LESSTAT1"
  int nx, ny, nz, precision, model, s_flag;
  int jt, jt_total;
  unsigned long long bytes;  // total image size
};
}  // namespace
size_t les_state_bytes(const les_ctx* c) {
  if (!c) return 0;
  size_t n = sizeof(StateHeader);
  for (int f = 0; f < LES_NUM_FIELDS; ++f) n += c->fsize[f] * sizeof(double);
  return n;
}
int les_state_save(les_ctx* c, void* host, size_t bytes) {
  if (!c || !host) return LES_ERR_ARG;
  const size_t need = les_state_bytes(c);
  if (bytes < need) { les_set_error("state image needs %zu bytes, buffer has %zu", need, bytes); return LES_ERR_ARG; }
  StateHeader h{};
  std::memcpy(h.magic, "LESSTAT1", 8);
  h.nx = c->cfg.nx; h.ny = c->cfg.ny; h.nz = c->cfg.nz;
  h.precision = c->cfg.precision; h.model = c->cfg.model; h.s_flag = c->cfg.s_flag;
  h.jt = c->jt; h.jt_total = c->jt_total;
  h.bytes = need;
  unsigned char* p = static_cast<unsigned char*>(host);
  std::memcpy(p, &h, sizeof(h));
  size_t off = sizeof(h);
  for (int f = 0; f < LES_NUM_FIELDS; ++f) {  // device storage as it is (FP32-held fields included)
    const size_t nb = c->fsize[f] * sizeof(double);
    LES_CUDA_CHECK(cudaMemcpyAsync(p + off, c->f[f], nb, cudaMemcpyDeviceToHost, c->stream));
    off += nb;
  }
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  return LES_OK;
}
int les_state_restore(les_ctx* c, const void* host, size_t bytes) {
  if (!c || !host) return LES_ERR_ARG;
  const size_t need = les_state_bytes(c);
  StateHeader h{};
  if (bytes < sizeof(h)) { les_set_error("state image too short"); return LES_ERR_ARG; }
  std::memcpy(&h, host, sizeof(h));
  if (std::memcmp(h.magic, "LESSTAT1", 8) != 0 || h.bytes != need || bytes < need || h.nx != c->cfg.nx ||
      h.ny != c->cfg.ny || h.nz != c->cfg.nz || h.precision != c->cfg.precision || h.model != c->cfg.model ||
      h.s_flag != c->cfg.s_flag) {
    les_set_error("state image does not match this context's configuration");
    return LES_ERR_ARG;
  }
  const unsigned char* p = static_cast<const unsigned char*>(host);
  size_t off = sizeof(h);
  for (int f = 0; f < LES_NUM_FIELDS; ++f) {
    const size_t nb = c->fsize[f] * sizeof(double);
    LES_CUDA_CHECK(cudaMemcpyAsync(c->f[f], p + off, nb, cudaMemcpyHostToDevice, c->stream));
    off += nb;
  }
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  c->jt = h.jt;
  c->jt_total = h.jt_total;
  return LES_OK;
}

// output_loop's running statistics (io.f90:211-213) after a step, when
// les_stats_enable asked for them
static int run_step(les_ctx* c) {
  switch (c->cfg.precision) {
    case 1: return step_mixed(c);
    case 2: return step_ff(c);
    default: return step_fp64(c);
  }
}
static void stats_after_step(les_ctx* c) {
  if (c->stats && c->stats_auto && c->cfg.s_flag && c->jt % c->stats_c == 0) op_stats(c);
}

int les_step(les_ctx* c, int nsteps) {
  if (!c || nsteps < 0) return LES_ERR_ARG;
  if (!c->surface_set) { les_set_error("les_set_surface must be called before les_step"); return LES_ERR_STATE; }
  for (int i = 0; i < nsteps; ++i) {
    int st = run_step(c);
    if (st) return st;
    stats_after_step(c);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { les_set_error("%s", cudaGetErrorString(e)); return LES_ERR_CUDA; }
  return LES_OK;
}

// ---- graphs, autotuning, ensembles -------------------------------------------
static inline bool special_step(const les_ctx* c, int next_jt) {
  const les_config& k = c->cfg;
  return next_jt == 1 || (k.rmsdiv_every > 0 && next_jt % k.rmsdiv_every == 0);
}
static inline void step_key(const les_ctx* c, int next_jt, int next_total, int* lag, int* ov) {
  const les_config& k = c->cfg;
  *lag = (next_jt % k.cs_count == 0) ? 1 : 0;
  *ov = ((k.model == 5 || k.model == 6 || k.model == 7) && next_total < 500) ? 1 : 0;
}


// capture one step of c on stream `s` (c->stream must be s or joined to it);
// the host state (counters, RHS buffer exchange) is left as before the step
static int capture_step(les_ctx* c, cudaGraph_t* graph) {
  const int jt0 = c->jt, jtt0 = c->jt_total, par0 = c->rhs_par;
  LES_CUDA_CHECK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int st = run_step(c);
  cudaError_t e = cudaStreamEndCapture(c->stream, graph);
  c->jt = jt0;
  c->jt_total = jtt0;
  if (c->rhs_par != par0) rhs_swap(c);
  if (st) return st;
  if (e != cudaSuccess) { les_set_error("capture: %s", cudaGetErrorString(e)); return LES_ERR_CUDA; }
  return 0;
}

int les_step_graph(les_ctx* c, int nsteps) {
  if (!c || nsteps < 0) return LES_ERR_ARG;
  if (!c->surface_set) { les_set_error("les_set_surface must be called before les_step_graph"); return LES_ERR_STATE; }
  for (int i = 0; i < nsteps; ++i) {
    const int nj = c->jt + 1, nt = c->jt_total + 1;
    if (special_step(c, nj)) {
      int st = run_step(c);
      if (st) return st;
      stats_after_step(c);
      continue;
    }
    int lag, ov;
    step_key(c, nj, nt, &lag, &ov);
    const int par = c->rhs_par;
    if (!c->gexec[lag][ov][par]) {
      cudaGraph_t gr;
      int st = capture_step(c, &gr);
      if (st) return st;
      cudaError_t e = cudaGraphInstantiate(&c->gexec[lag][ov][par], gr, 0);
      cudaGraphDestroy(gr);
      if (e != cudaSuccess) { les_set_error("instantiate: %s", cudaGetErrorString(e)); return LES_ERR_CUDA; }
    }
    LES_CUDA_CHECK(cudaGraphLaunch(c->gexec[lag][ov][par], c->stream));
    rhs_swap(c);  // what the replayed step did
    c->jt = nj;
    c->jt_total = nt;
    stats_after_step(c);
  }
  return LES_OK;
}

// Capture and instantiate the step graphs that les_step_graph replays for the
// next non-special steps of both kinds (with and without the Lagrangian
// update) and both RHS buffer parities, without running a step: a serving
// loop moves the capture cost off its path.  Counters and buffers are left as
// they were.
int les_step_graph_prepare(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  if (!c->surface_set) { les_set_error("les_set_surface must be called before les_step_graph_prepare"); return LES_ERR_STATE; }
  const int jt0 = c->jt, jtt0 = c->jt_total, par0 = c->rhs_par;
  int st = LES_OK;
  for (int want = 0; want < 2 && st == LES_OK; ++want) {
    int nj = jt0 + 1, found = 0;
    for (int k = 0; k < 4 * c->cfg.cs_count + 8; ++k, ++nj) {
      int lag, ov;
      step_key(c, nj, jtt0 + (nj - jt0), &lag, &ov);
      if (lag == want && !special_step(c, nj)) { found = 1; break; }
    }
    if (!found) continue;  // every step of this kind runs eagerly
    for (int par = 0; par < 2 && st == LES_OK; ++par) {
      c->jt = nj - 1;
      c->jt_total = jtt0 + (nj - jt0) - 1;
      if (c->rhs_par != par) rhs_swap(c);
      int lag, ov;
      step_key(c, nj, c->jt_total + 1, &lag, &ov);
      if (c->gexec[lag][ov][par]) continue;
      cudaGraph_t gr;
      st = capture_step(c, &gr);
      if (st) break;
      cudaError_t e = cudaGraphInstantiate(&c->gexec[lag][ov][par], gr, 0);
      cudaGraphDestroy(gr);
      if (e != cudaSuccess) { les_set_error("instantiate: %s", cudaGetErrorString(e)); st = LES_ERR_CUDA; }
    }
  }
  c->jt = jt0;
  c->jt_total = jtt0;
  if (c->rhs_par != par0) rhs_swap(c);
  return st;
}

// process-wide cache of tuned launch shapes per (grid, precision)
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int>, std::tuple<int, int, int>> g_tune;

int les_autotune(les_ctx* c, int* tx64, int* tx32, int* rpc_scale) {
  if (!c) return LES_ERR_ARG;
  const auto key = std::make_tuple(c->g.nx, c->g.ny, c->g.nz, c->cfg.precision);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      c->tx64 = std::get<0>(it->second);
      c->tx32 = std::get<1>(it->second);
      c->rpc_scale = std::get<2>(it->second);
    } else {
      cudaEvent_t e0, e1;
      LES_CUDA_CHECK(cudaEventCreate(&e0));
      LES_CUDA_CHECK(cudaEventCreate(&e1));
      auto rpc_of = [](int nx, int sc) {
        int m = nx / 2, r = 1024 / (m / 4 > 0 ? m : 4);
        r = std::max(1, std::min(16, r));
        if (sc > 0) r = std::min(32, r * 2);
        if (sc < 0) r = std::max(1, r / 2);
        return r;
      };
      auto time_cfg = [&](int fp32, int tx, int sc) -> float {
        if (fp32) c->tx32 = tx; else c->tx64 = tx;
        const int r = rpc_of(c->g.nx, sc), rb = rpc_of(c->g.nx2, sc);
        if (fp32) { c->rpc32 = r; c->rpcb32 = rb; } else { c->rpc64 = r; c->rpcb64 = rb; }
        autotune_probe(c, fp32);  // warm-up (and smem opt-in)
        cudaEventRecord(e0, c->stream);
        for (int k = 0; k < 3; ++k) autotune_probe(c, fp32);
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms;
      };
      int best[2][2] = {{4, 0}, {8, 0}};
      const int txs[2][3] = {{2, 4, 8}, {4, 8, 16}};
      for (int fp32 = 0; fp32 < 2; ++fp32) {
        if (fp32 && c->cfg.precision != 1) continue;
        float bt = 1e30f;
        for (int a = 0; a < 3; ++a)
          for (int sc = -1; sc <= 1; ++sc) {
            const float t = time_cfg(fp32, txs[fp32][a], sc);
            if (t < bt) { bt = t; best[fp32][0] = txs[fp32][a]; best[fp32][1] = sc; }
          }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      LES_CUDA_CHECK(cudaGetLastError());
      c->tx64 = best[0][0];
      c->tx32 = best[1][0];
      c->rpc_scale = best[0][1];  // one scale for both precisions: the FP64 choice
      g_tune[key] = std::make_tuple(c->tx64, c->tx32, c->rpc_scale);
    }
  }
  auto rpc_of = [](int nx, int sc) {
    int m = nx / 2, r = 1024 / (m / 4 > 0 ? m : 4);
    r = std::max(1, std::min(16, r));
    if (sc > 0) r = std::min(32, r * 2);
    if (sc < 0) r = std::max(1, r / 2);
    return r;
  };
  c->rpc64 = c->rpc32 = rpc_of(c->g.nx, c->rpc_scale);
  c->rpcb64 = c->rpcb32 = rpc_of(c->g.nx2, c->rpc_scale);
  // graphs captured with the old shapes are stale
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int p = 0; p < 2; ++p)
        if (c->gexec[a][b][p]) { cudaGraphExecDestroy(c->gexec[a][b][p]); c->gexec[a][b][p] = nullptr; }
  if (tx64) *tx64 = c->tx64;
  if (tx32) *tx32 = c->tx32;
  if (rpc_scale) *rpc_scale = c->rpc_scale;
  return LES_OK;
}

}  // extern "C"

struct les_ensemble {
  std::vector<les_ctx*> m;
  cudaStream_t root = nullptr;
  cudaEvent_t fork = nullptr;
  cudaEvent_t done = nullptr;  // end of the last graph launch, waited on by every member stream
  std::vector<cudaEvent_t> join;
  std::map<std::vector<int>, cudaGraphExec_t> graphs;
};

extern "C" {

int les_ensemble_create(les_ctx* const* members, int n, les_ensemble** out) {
  if (!members || n < 1 || !out) return LES_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    if (!members[i]) return LES_ERR_ARG;
    if (members[i]->cfg.cs_count != members[0]->cfg.cs_count || members[i]->jt != members[0]->jt) {
      les_set_error("ensemble members must share cs_count and the step counter");
      return LES_ERR_ARG;
    }
  }
  les_ensemble* e = new les_ensemble();
  e->m.assign(members, members + n);
  if (cudaStreamCreateWithFlags(&e->root, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming) != cudaSuccess) {
    delete e; les_set_error("ensemble stream/event creation failed"); return LES_ERR_CUDA;
  }
  e->join.resize(n);
  for (int i = 0; i < n; ++i)
    if (cudaEventCreateWithFlags(&e->join[i], cudaEventDisableTiming) != cudaSuccess) {
      les_set_error("ensemble event creation failed"); return LES_ERR_CUDA;
    }
  *out = e;
  return LES_OK;
}

void* les_ensemble_stream(les_ensemble* e) { return e ? (void*)e->root : nullptr; }

int les_ensemble_step(les_ensemble* e, int nsteps) {
  if (!e || nsteps < 0) return LES_ERR_ARG;
  const int n = (int)e->m.size();
  for (int s = 0; s < nsteps; ++s) {
    les_ctx* m0 = e->m[0];
    const int nj = m0->jt + 1;
    bool special = false;
    for (les_ctx* c : e->m) {
      if (!c->surface_set) { les_set_error("member without surface"); return LES_ERR_STATE; }
      if (c->jt + 1 != nj) { les_set_error("ensemble members out of step"); return LES_ERR_STATE; }
      special = special || special_step(c, nj);
    }
    if (special) {  // eager step on every member's stream, ordered after the root
      LES_CUDA_CHECK(cudaEventRecord(e->fork, e->root));
      for (int i = 0; i < n; ++i) {
        LES_CUDA_CHECK(cudaStreamWaitEvent(e->m[i]->stream, e->fork, 0));
        int st = run_step(e->m[i]);
        if (st) return st;
        LES_CUDA_CHECK(cudaEventRecord(e->join[i], e->m[i]->stream));
        LES_CUDA_CHECK(cudaStreamWaitEvent(e->root, e->join[i], 0));
      }
      continue;
    }
    std::vector<int> key(3 * n);
    for (int i = 0; i < n; ++i) {
      step_key(e->m[i], nj, e->m[i]->jt_total + 1, &key[3 * i], &key[3 * i + 1]);
      key[3 * i + 2] = e->m[i]->rhs_par;
    }
    auto it = e->graphs.find(key);
    if (it == e->graphs.end()) {
      // capture: root forks to every member stream and joins them back
      std::vector<int> jt0(n), jtt0(n), par0(n);
      for (int i = 0; i < n; ++i) { jt0[i] = e->m[i]->jt; jtt0[i] = e->m[i]->jt_total; par0[i] = e->m[i]->rhs_par; }
      LES_CUDA_CHECK(cudaStreamBeginCapture(e->root, cudaStreamCaptureModeThreadLocal));
      cudaEventRecord(e->fork, e->root);
      int st = 0;
      for (int i = 0; i < n && !st; ++i) {
        cudaStreamWaitEvent(e->m[i]->stream, e->fork, 0);
        st = run_step(e->m[i]);
        cudaEventRecord(e->join[i], e->m[i]->stream);
        cudaStreamWaitEvent(e->root, e->join[i], 0);
      }
      cudaGraph_t gr;
      cudaError_t ce = cudaStreamEndCapture(e->root, &gr);
      for (int i = 0; i < n; ++i) {
        e->m[i]->jt = jt0[i];
        e->m[i]->jt_total = jtt0[i];
        if (e->m[i]->rhs_par != par0[i]) rhs_swap(e->m[i]);
      }
      if (st) return st;
      if (ce != cudaSuccess) { les_set_error("ensemble capture: %s", cudaGetErrorString(ce)); return LES_ERR_CUDA; }
      cudaGraphExec_t ex;
      ce = cudaGraphInstantiate(&ex, gr, 0);
      cudaGraphDestroy(gr);
      if (ce != cudaSuccess) { les_set_error("ensemble instantiate: %s", cudaGetErrorString(ce)); return LES_ERR_CUDA; }
      it = e->graphs.emplace(key, ex).first;
    }
    // the graph runs on the root stream: it starts after work already queued
    // on the members' streams, and what is queued on them later (a field
    // read, a per-member step) starts after it
    for (int i = 0; i < n; ++i) {
      LES_CUDA_CHECK(cudaEventRecord(e->join[i], e->m[i]->stream));
      LES_CUDA_CHECK(cudaStreamWaitEvent(e->root, e->join[i], 0));
    }
    LES_CUDA_CHECK(cudaGraphLaunch(it->second, e->root));
    LES_CUDA_CHECK(cudaEventRecord(e->done, e->root));
    for (les_ctx* c : e->m) LES_CUDA_CHECK(cudaStreamWaitEvent(c->stream, e->done, 0));
    for (les_ctx* c : e->m) { c->jt += 1; c->jt_total += 1; rhs_swap(c); }
  }
  return LES_OK;
}

int les_ensemble_destroy(les_ensemble* e) {
  if (!e) return LES_OK;
  cudaStreamSynchronize(e->root);
  for (auto& kv : e->graphs) cudaGraphExecDestroy(kv.second);
  for (cudaEvent_t ev : e->join) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->done) cudaEventDestroy(e->done);
  if (e->root) cudaStreamDestroy(e->root);
  delete e;
  return LES_OK;
}

int les_profile_begin(les_ctx* c, int family, int max_launches) {
  if (!c || family < PROF_COLS64 || family > PROF_ROWS32 || max_launches < 1) return LES_ERR_ARG;
  if (g_prof) { les_set_error("a profiling session is already open"); return LES_ERR_STATE; }
  ProfSession* p = new ProfSession();
  p->family = family;
  p->stream = c->stream;
  p->cap = max_launches;
  p->ev = new cudaEvent_t[2 * (size_t)max_launches]();
  for (int i = 0; i < 2 * max_launches; ++i)
    if (cudaEventCreate(&p->ev[i]) != cudaSuccess) {
      for (int j = 0; j < i; ++j) cudaEventDestroy(p->ev[j]);
      delete[] p->ev;
      delete p;
      les_set_error("event creation failed");
      return LES_ERR_CUDA;
    }
  g_prof = p;
  return LES_OK;
}
int les_profile_end(les_ctx* c, int* launches, double* ms, double* bytes) {
  if (!c || !launches || !ms || !bytes) return LES_ERR_ARG;
  ProfSession* p = g_prof;
  if (!p || p->stream != c->stream) { les_set_error("no profiling session open on this context"); return LES_ERR_STATE; }
  g_prof = nullptr;
  int st = LES_OK;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) st = LES_ERR_CUDA;
  double tot = 0.0;
  for (int i = 0; i < p->n && !st; ++i) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, p->ev[2 * i], p->ev[2 * i + 1]) != cudaSuccess) st = LES_ERR_CUDA;
    tot += t;
  }
  *launches = p->n;
  *ms = tot;
  *bytes = p->bytes;
  for (int i = 0; i < 2 * p->cap; ++i) cudaEventDestroy(p->ev[i]);
  delete[] p->ev;
  delete p;
  if (st) les_set_error("profiling: %s", cudaGetErrorString(cudaGetLastError()));
  return st;
}
int les_selftest_conversions(size_t n, unsigned long long seed, unsigned long long* mismatches) {
  if (!mismatches) return LES_ERR_ARG;
  unsigned long long* d = nullptr;
  LES_CUDA_CHECK(cudaMalloc(&d, sizeof(*d)));
  cudaMemset(d, 0, sizeof(*d));
  op_cvt_selftest(n, seed, d, 0);
  cudaError_t e = cudaMemcpy(mismatches, d, sizeof(*d), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) { les_set_error("%s", cudaGetErrorString(e)); return LES_ERR_CUDA; }
  return LES_OK;
}
int les_rmsdiv(les_ctx* c, double* rms) {
  if (!c || !rms) return LES_ERR_ARG;
  if (c->cfg.precision == 1) op_rmsdiv_state(c, c->dscal + 1);
  else op_rmsdiv(c, c->dscal + 1);
  LES_CUDA_CHECK(cudaMemcpyAsync(c->host_scal + 1, c->dscal + 1, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  *rms = c->host_scal[1];
  return LES_OK;
}
int les_timestep_conditions(les_ctx* c, double* cflu, double* visc) {
  if (!c || !cflu || !visc) return LES_ERR_ARG;
  return op_tsc(c, cflu, visc);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// per-routine entry points: host or device array arguments
namespace {
struct Arg {
  les_ctx* c;
  const void* user;
  double* dev = nullptr;
  size_t n;
  bool owned = false;
  Arg(les_ctx* c_, const void* u, size_t n_) : c(c_), user(u), n(n_) {}
  Arg(const Arg&) = delete;
  Arg& operator=(const Arg&) = delete;
  // caller device arrays are read and written as pairs of doubles (16 bytes)
  int take_user() {
    if (reinterpret_cast<uintptr_t>(user) & 15u) {
      les_set_error("device array %p is not 16-byte aligned", user);
      return LES_ERR_ARG;
    }
    dev = (double*)user;
    return 0;
  }
  int in() {
    if (c->ptr_mode) return take_user();
    if (cudaMalloc(&dev, n * sizeof(double)) != cudaSuccess) { les_set_error("staging alloc failed"); return LES_ERR_OOM; }
    owned = true;
    if (cudaMemcpyAsync(dev, user, n * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) return LES_ERR_CUDA;
    return 0;
  }
  int alloc() {
    if (c->ptr_mode) return take_user();
    if (cudaMalloc(&dev, n * sizeof(double)) != cudaSuccess) { les_set_error("staging alloc failed"); return LES_ERR_OOM; }
    owned = true;
    if (cudaMemsetAsync(dev, 0, n * sizeof(double), c->stream) != cudaSuccess) {
      les_set_error("staging clear failed");
      return LES_ERR_CUDA;
    }
    return 0;
  }
  int out() {
    if (c->ptr_mode) return 0;
    if (cudaMemcpyAsync((void*)user, dev, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return LES_ERR_CUDA;
    return 0;
  }
  ~Arg() {
    if (owned) { cudaStreamSynchronize(c->stream); cudaFree(dev); }
  }
};
int finish(les_ctx* c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) { les_set_error("%s", cudaGetErrorString(e)); return LES_ERR_CUDA; }
  return LES_OK;
}
}  // namespace

#define CHK(x) do { int _s = (x); if (_s) return _s; } while (0)

extern "C" {

int les_ddx(les_ctx* c, double* dfdx, const double* f, int nlev) {
  if (!c || !dfdx || !f || nlev < 1 || nlev > c->g.nz + 1) return LES_ERR_ARG;
  const size_t n = c->g.nplane * nlev;
  Arg A(c, f, n), B(c, dfdx, n);
  CHK(A.in()); CHK(B.alloc());
  op_ddxy(c, B.dev, nullptr, A.dev, nlev);
  CHK(B.out());
  return finish(c);
}
int les_ddy(les_ctx* c, double* dfdy, const double* f, int nlev) {
  if (!c || !dfdy || !f || nlev < 1 || nlev > c->g.nz + 1) return LES_ERR_ARG;
  const size_t n = c->g.nplane * nlev;
  Arg A(c, f, n), B(c, dfdy, n);
  CHK(A.in()); CHK(B.alloc());
  op_ddxy(c, nullptr, B.dev, A.dev, nlev);
  CHK(B.out());
  return finish(c);
}
int les_ddxy(les_ctx* c, double* dfdx, double* dfdy, const double* f, int nlev) {
  if (!c || !dfdx || !dfdy || !f || nlev < 1 || nlev > c->g.nz + 1) return LES_ERR_ARG;
  const size_t n = c->g.nplane * nlev;
  Arg A(c, f, n), B(c, dfdx, n), D(c, dfdy, n);
  CHK(A.in()); CHK(B.alloc()); CHK(D.alloc());
  op_ddxy(c, B.dev, D.dev, A.dev, nlev);
  CHK(B.out()); CHK(D.out());
  return finish(c);
}
int les_filt_da(les_ctx* c, double* f, double* dfdx, double* dfdy, int nlev) {
  if (!c || !f || !dfdx || !dfdy || nlev < 1 || nlev > c->g.nz + 1) return LES_ERR_ARG;
  const size_t n = c->g.nplane * nlev;
  Arg A(c, f, n), B(c, dfdx, n), D(c, dfdy, n);
  CHK(A.in()); CHK(B.alloc()); CHK(D.alloc());
  op_filt_da(c, A.dev, B.dev, D.dev, nlev);
  CHK(A.out()); CHK(B.out()); CHK(D.out());
  return finish(c);
}
int les_ddz_uv(les_ctx* c, double* dfdz, const double* f) {
  if (!c || !dfdz || !f) return LES_ERR_ARG;
  Arg A(c, f, c->g.nfield), B(c, dfdz, c->g.nfield);
  CHK(A.in()); CHK(B.in());
  op_ddz(c, B.dev, A.dev, 1);
  CHK(B.out());
  return finish(c);
}
int les_ddz_w(les_ctx* c, double* dfdz, const double* f) {
  if (!c || !dfdz || !f) return LES_ERR_ARG;
  Arg A(c, f, c->g.nfield), B(c, dfdz, c->g.nfield);
  CHK(A.in()); CHK(B.in());
  op_ddz(c, B.dev, A.dev, 0);
  CHK(B.out());
  return finish(c);
}
int les_dealias1(les_ctx* c, const double* u, double* u_big, int nlev) {
  if (!c || !u || !u_big || nlev < 1 || nlev > c->g.nz) return LES_ERR_ARG;
  Arg A(c, u, c->g.nplane * nlev), B(c, u_big, c->g.nplane_big * nlev);
  CHK(A.in()); CHK(B.alloc());
  const double* in[1] = {A.dev};
  double* out[1] = {B.dev};
  op_dealias1(c, in, out, 1, nlev);
  CHK(B.out());
  return finish(c);
}
int les_dealias2(les_ctx* c, double* u, double* u_big, int nlev) {
  if (!c || !u || !u_big || nlev < 1 || nlev > c->g.nz) return LES_ERR_ARG;
  Arg A(c, u, c->g.nplane * nlev), B(c, u_big, c->g.nplane_big * nlev);
  CHK(A.alloc()); CHK(B.in());
  const double* in[1] = {B.dev};
  double* out[1] = {A.dev};
  op_dealias2(c, out, in, 1, nlev, 1.0 / (double)(c->g.nx2 * c->g.ny2));
  CHK(A.out());
  return finish(c);
}
int les_fft_r2c(les_ctx* c, double* planes, int nplanes, int big) {
  if (!c || !planes || nplanes < 1) return LES_ERR_ARG;
  const size_t np = big ? c->g.nplane_big : c->g.nplane;
  const size_t per = (big ? (size_t)c->g.lh_big * c->g.ny2 : c->g.C) * sizeof(double2);
  const int chunk = (int)std::max<size_t>(1, std::min(c->wsA_bytes, c->wsB_bytes) / per);
  Arg A(c, planes, np * nplanes);
  CHK(A.in());
  for (int p0 = 0; p0 < nplanes; p0 += chunk) op_fft(c, A.dev + (size_t)p0 * np, std::min(chunk, nplanes - p0), big, 0);
  CHK(A.out());
  return finish(c);
}
int les_fft_c2r(les_ctx* c, double* planes, int nplanes, int big) {
  if (!c || !planes || nplanes < 1) return LES_ERR_ARG;
  const size_t np = big ? c->g.nplane_big : c->g.nplane;
  const size_t per = (big ? (size_t)c->g.lh_big * c->g.ny2 : c->g.C) * sizeof(double2);
  const int chunk = (int)std::max<size_t>(1, std::min(c->wsA_bytes, c->wsB_bytes) / per);
  Arg A(c, planes, np * nplanes);
  CHK(A.in());
  for (int p0 = 0; p0 < nplanes; p0 += chunk) op_fft(c, A.dev + (size_t)p0 * np, std::min(chunk, nplanes - p0), big, 1);
  CHK(A.out());
  return finish(c);
}
int les_tridag_array(les_ctx* c, const double* a, const double* b, const double* cc, const double* r, double* u) {
  if (!c || !a || !b || !cc || !r || !u) return LES_ERR_ARG;
  const size_t nk = (size_t)c->g.lh * c->g.ny * (c->g.nz + 1);
  Arg A(c, a, nk), B(c, b, nk), Cc(c, cc, nk), R(c, r, 2 * nk), U(c, u, 2 * nk);
  CHK(A.in()); CHK(B.in()); CHK(Cc.in()); CHK(R.in()); CHK(U.in());
  int* flag = reinterpret_cast<int*>(c->dscal + 8);
  cudaMemsetAsync(flag, 0, sizeof(int), c->stream);
  // zero-pivot check on row 1 (tridag_array.f90:32-39)
  std::vector<double> b1((size_t)c->g.lh * c->g.ny);
  if (c->ptr_mode) cudaMemcpy(b1.data(), b, b1.size() * sizeof(double), cudaMemcpyDeviceToHost);
  else std::memcpy(b1.data(), b, b1.size() * sizeof(double));
  for (int jy = 0; jy < c->g.ny; ++jy)
    for (int jx = 0; jx < c->g.lh - 1; ++jx)
      if (b1[(size_t)jy * c->g.lh + jx] == 0.0) { les_set_error("tridag_array: rewrite eqs, jx, jy= %d %d", jx + 1, jy + 1); return LES_ERR_PIVOT; }
  op_tridag(c, A.dev, B.dev, Cc.dev, R.dev, U.dev);
  CHK(U.out());
  int st = finish(c);
  if (st) return st;
  int fl = 0;
  cudaMemcpy(&fl, flag, sizeof(int), cudaMemcpyDeviceToHost);
  if (fl) { les_set_error("tridag_array failed: zero pivot"); return LES_ERR_PIVOT; }
  return LES_OK;
}
static int need_fp64(const les_ctx* c, const char* name);
int les_convec(les_ctx* c, double* cx, double* cy, double* cz) {
  if (!c || !cx || !cy || !cz) return LES_ERR_ARG;
  if (int st = need_fp64(c, "les_convec")) return st;
  const size_t n = c->g.nfield;
  Arg X(c, cx, n), Y(c, cy, n), Z(c, cz, n);
  CHK(X.alloc()); CHK(Y.alloc()); CHK(Z.alloc());
  op_convec(c, X.dev, Y.dev, Z.dev);
  CHK(X.out()); CHK(Y.out()); CHK(Z.out());
  return finish(c);
}
int les_divstress_uv(les_ctx* c, double* divt, const double* tx, const double* ty, const double* tz) {
  if (!c || !divt || !tx || !ty || !tz) return LES_ERR_ARG;
  const size_t n = c->g.nfield;
  Arg D(c, divt, n), X(c, tx, n), Y(c, ty, n), Z(c, tz, n);
  CHK(D.alloc()); CHK(X.in()); CHK(Y.in()); CHK(Z.in());
  op_divstress_one(c, D.dev, X.dev, Y.dev, Z.dev, 0);
  CHK(D.out());
  return finish(c);
}
int les_divstress_w(les_ctx* c, double* divt, const double* tx, const double* ty, const double* tz) {
  if (!c || !divt || !tx || !ty || !tz) return LES_ERR_ARG;
  const size_t n = c->g.nfield;
  Arg D(c, divt, n), X(c, tx, n), Y(c, ty, n), Z(c, tz, n);
  CHK(D.alloc()); CHK(X.in()); CHK(Y.in()); CHK(Z.in());
  op_divstress_one(c, D.dev, X.dev, Y.dev, Z.dev, 1);
  CHK(D.out());
  return finish(c);
}
int les_press_stag_array(les_ctx* c, double* p_hat, double* dfdx, double* dfdy) {
  if (!c || !p_hat || !dfdx || !dfdy) return LES_ERR_ARG;
  Arg P(c, p_hat, c->g.nplane * (c->g.nz + 1)), X(c, dfdx, c->g.nfield), Y(c, dfdy, c->g.nfield);
  CHK(P.alloc()); CHK(X.alloc()); CHK(Y.alloc());
  int* flag = reinterpret_cast<int*>(c->dscal + 8);
  cudaMemsetAsync(flag, 0, sizeof(int), c->stream);
  op_press(c, P.dev, X.dev, Y.dev);
  CHK(P.out()); CHK(X.out()); CHK(Y.out());
  int st = finish(c);
  if (st) return st;
  int fl = 0;
  cudaMemcpy(&fl, flag, sizeof(int), cudaMemcpyDeviceToHost);
  if (fl) { les_set_error("tridag_array failed: zero pivot"); return LES_ERR_PIVOT; }
  return LES_OK;
}
int les_sgs_stag(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  if (int st = need_fp64(c, "les_sgs_stag")) return st;
  op_sgs_stag(c);
  return finish(c);
}
int les_lagrange_sdep(les_ctx* c, const double* S11, const double* S12, const double* S13, const double* S22,
                      const double* S23, const double* S33) {
  if (!c || !S11 || !S12 || !S13 || !S22 || !S23 || !S33) return LES_ERR_ARG;
  const size_t n = c->g.nfield;
  Arg a(c, S11, n), b(c, S12, n), d(c, S13, n), e(c, S22, n), f(c, S23, n), h(c, S33, n);
  CHK(a.in()); CHK(b.in()); CHK(d.in()); CHK(e.in()); CHK(f.in()); CHK(h.in());
  const double* S[6] = {a.dev, b.dev, d.dev, e.dev, f.dev, h.dev};
  op_lagrange(c, S);
  return finish(c);
}
int les_lagrange_ssim(les_ctx* c, const double* S11, const double* S12, const double* S13, const double* S22,
                      const double* S23, const double* S33) {
  if (!c || !S11 || !S12 || !S13 || !S22 || !S23 || !S33) return LES_ERR_ARG;
  const size_t n = c->g.nfield;
  Arg a(c, S11, n), b(c, S12, n), d(c, S13, n), e(c, S22, n), f(c, S23, n), h(c, S33, n);
  CHK(a.in()); CHK(b.in()); CHK(d.in()); CHK(e.in()); CHK(f.in()); CHK(h.in());
  const double* S[6] = {a.dev, b.dev, d.dev, e.dev, f.dev, h.dev};
  op_lagrange_ssim(c, S);
  return finish(c);
}
int les_interpolag_ssim(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  op_interpolag_n(c, 2);
  return finish(c);
}
int les_interpolag_sdep(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  op_interpolag(c);
  return finish(c);
}
int les_lagrange_scalar_sdep(les_ctx* c, double* cs2_pr, const double* S11, const double* S12, const double* S13,
                             const double* S22, const double* S23, const double* S33) {
  if (!c || !cs2_pr || !S11 || !S12 || !S13 || !S22 || !S23 || !S33) return LES_ERR_ARG;
  if (!c->f[LES_G_LM]) { les_set_error("les_lagrange_scalar_sdep needs a model-7 context"); return LES_ERR_STATE; }
  const size_t n = c->g.nfield;
  Arg a(c, S11, n), b(c, S12, n), d(c, S13, n), e(c, S22, n), f(c, S23, n), h(c, S33, n), o(c, cs2_pr, n);
  CHK(a.in()); CHK(b.in()); CHK(d.in()); CHK(e.in()); CHK(f.in()); CHK(h.in()); CHK(o.alloc());
  const double* S[6] = {a.dev, b.dev, d.dev, e.dev, f.dev, h.dev};
  op_lagrange_scalar(c, S, o.dev);
  CHK(o.out());
  return finish(c);
}
int les_interpolag_scalar_sdep(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  if (!c->f[LES_G_LM]) { les_set_error("les_interpolag_scalar_sdep needs a model-7 context"); return LES_ERR_STATE; }
  op_interpolag_scalar(c);
  return finish(c);
}
int les_scaledep_dynamic(les_ctx* c, double* cs_opt2, const double* S11, const double* S12, const double* S13,
                         const double* S22, const double* S23, const double* S33) {
  if (!c || !cs_opt2 || !S11 || !S12 || !S13 || !S22 || !S23 || !S33) return LES_ERR_ARG;
  const size_t n = c->g.nfield;
  Arg a(c, S11, n), b(c, S12, n), d(c, S13, n), e(c, S22, n), f(c, S23, n), h(c, S33, n), o(c, cs_opt2, c->g.nz);
  CHK(a.in()); CHK(b.in()); CHK(d.in()); CHK(e.in()); CHK(f.in()); CHK(h.in()); CHK(o.alloc());
  const double* S[6] = {a.dev, b.dev, d.dev, e.dev, f.dev, h.dev};
  op_scaledep(c, o.dev, S);
  CHK(o.out());
  return finish(c);
}
int les_std_dynamic(les_ctx* c, double* cs_opt2, const double* S11, const double* S12, const double* S13,
                    const double* S22, const double* S23, const double* S33) {
  if (!c || !cs_opt2 || !S11 || !S12 || !S13 || !S22 || !S23 || !S33) return LES_ERR_ARG;
  const size_t n = c->g.nfield;
  Arg a(c, S11, n), b(c, S12, n), d(c, S13, n), e(c, S22, n), f(c, S23, n), h(c, S33, n), o(c, cs_opt2, c->g.nz);
  CHK(a.in()); CHK(b.in()); CHK(d.in()); CHK(e.in()); CHK(f.in()); CHK(h.in()); CHK(o.alloc());
  const double* S[6] = {a.dev, b.dev, d.dev, e.dev, f.dev, h.dev};
  op_stddyn(c, o.dev, S);
  CHK(o.out());
  return finish(c);
}
// The per-routine module operations below read or write S_ij, Nu_t, tau_ij or
// the velocity gradients in FP64; on an FP32-mixed context those are held in
// FP32, so these entries need a precision-0 or precision-2 context.
static int need_fp64(const les_ctx* c, const char* name) {
  if (c->cfg.precision != 1) return LES_OK;
  les_set_error("%s: needs a precision-0 or -2 context (the mixed form holds S_ij, Nu_t, tau_ij in FP32)", name);
  return LES_ERR_ARG;
}
int les_wallstress(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  if (int st = need_fp64(c, "les_wallstress")) return st;
  op_wallstress(c);
  return finish(c);
}
int les_obukhov(les_ctx* c) { if (!c) return LES_ERR_ARG; op_obukhov(c); return finish(c); }
int les_project(les_ctx* c) { if (!c) return LES_ERR_ARG; op_project(c); return finish(c); }
int les_theta_all_in_one(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  if (int st = need_fp64(c, "les_theta_all_in_one")) return st;
  op_theta(c);
  return finish(c);
}
int les_q_all_in_one(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  if (!c->cfg.q_flag) { les_set_error("les_q_all_in_one: the context has no humidity (q_flag = 0)"); return LES_ERR_STATE; }
  if (int st = need_fp64(c, "les_q_all_in_one")) return st;
  op_q(c);
  return finish(c);
}
int les_atm_thermodynamics(les_ctx* c, double* actual_T, double* actual_Tv, double* sat_vapor_pr, double* pr_atm,
                           double* vapor_pr, double* sat_qmix, double* rel_hum, double* rel_hum_q, double* zlcl_all) {
  double* o[9] = {actual_T, actual_Tv, sat_vapor_pr, pr_atm, vapor_pr, sat_qmix, rel_hum, rel_hum_q, zlcl_all};
  if (!c) return LES_ERR_ARG;
  for (double* p : o)
    if (!p) return LES_ERR_ARG;
  if (!c->cfg.q_flag) {
    les_set_error("les_atm_thermodynamics: the context has no humidity (q_flag = 0)");
    return LES_ERR_STATE;
  }
  const size_t n = c->g.nfield;
  std::unique_ptr<Arg> a[9];
  double* dev[9];
  for (int i = 0; i < 9; ++i) {
    a[i].reset(new Arg(c, o[i], n));
    CHK(a[i]->alloc());
    dev[i] = a[i]->dev;
  }
  op_thermo(c, dev);
  for (int i = 0; i < 9; ++i) CHK(a[i]->out());
  return finish(c);
}

int les_test_filter(les_ctx* c, double* f, const double* G, int nplanes) {
  if (!c || !f || !G || nplanes < 1) return LES_ERR_ARG;
  // the transfer function must be one of the context's two filters
  const size_t nk = (size_t)c->g.lh * c->g.ny;
  std::vector<double> hg(nk), t0(nk), t1(nk);
  if (c->ptr_mode) cudaMemcpy(hg.data(), G, nk * sizeof(double), cudaMemcpyDeviceToHost);
  else std::memcpy(hg.data(), G, nk * sizeof(double));
  cudaMemcpy(t0.data(), c->G, nk * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(t1.data(), c->GG, nk * sizeof(double), cudaMemcpyDeviceToHost);
  int which = -1;
  if (std::memcmp(hg.data(), t0.data(), nk * sizeof(double)) == 0) which = 0;
  else if (std::memcmp(hg.data(), t1.data(), nk * sizeof(double)) == 0) which = 1;
  if (which < 0) { les_set_error("les_test_filter: G must be G_test or G_test_test of this context"); return LES_ERR_UNSUPPORTED; }
  Arg A(c, f, c->g.nplane * nplanes);
  CHK(A.in());
  op_test_filter(c, A.dev, A.dev, nplanes, which, (long)c->g.nplane);
  CHK(A.out());
  return finish(c);
}
int les_test_filter_init(les_ctx* c, double alpha, double* G) {
  if (!c || !G || !(alpha > 0.0)) return LES_ERR_ARG;
  std::vector<double> kx, ky, k2, g;
  wavenumbers(c->cfg, c->g, kx, ky, k2);
  filter_G(c->g, k2, alpha, g);
  if (c->ptr_mode) LES_CUDA_CHECK(cudaMemcpy(G, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice));
  else std::memcpy(G, g.data(), g.size() * sizeof(double));
  return LES_OK;
}

// padd.f90 / unpadd.f90 on complex planes
}  // extern "C"

namespace les {
__global__ void k_padd(double2* ub, const double2* us, int lh, int ny, int lhb, int ny2, int nx, int np) {
  const size_t tot = (size_t)lhb * ny2 * np;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const int p = (int)(i / ((size_t)lhb * ny2));
    const size_t r = i - (size_t)p * lhb * ny2;
    const int jy = (int)(r / lhb), jx = (int)(r % lhb);
    double2 v = make_double2(0.0, 0.0);
    if (jx < nx / 2) {
      int js = -1;
      if (jy < ny / 2) js = jy;
      else if (jy > ny2 - ny / 2) js = jy - (ny2 - ny);
      if (js >= 0) v = us[(size_t)p * lh * ny + (size_t)js * lh + jx];
    }
    ub[i] = v;
  }
}
__global__ void k_unpadd(double2* cc, const double2* cb, int lh, int ny, int lhb, int ny2, int nx, int np) {
  const size_t tot = (size_t)lh * ny * np;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const int p = (int)(i / ((size_t)lh * ny));
    const size_t r = i - (size_t)p * lh * ny;
    const int jy = (int)(r / lh), jx = (int)(r % lh);
    double2 v = make_double2(0.0, 0.0);
    if (jx < nx / 2 && jy != ny / 2) {
      const int jb = (jy < ny / 2) ? jy : jy + (ny2 - ny);
      v = cb[(size_t)p * lhb * ny2 + (size_t)jb * lhb + jx];
    }
    cc[i] = v;
  }
}
}  // namespace les

extern "C" {
int les_padd(les_ctx* c, double* u_big, const double* u, int nplanes) {
  if (!c || !u_big || !u || nplanes < 1) return LES_ERR_ARG;
  const Grid& g = c->g;
  Arg B(c, u_big, g.nplane_big * nplanes), S(c, u, g.nplane * nplanes);
  CHK(B.alloc()); CHK(S.in());
  k_padd<<<256, 256, 0, c->stream>>>((double2*)B.dev, (const double2*)S.dev, g.lh, g.ny, g.lh_big, g.ny2, g.nx, nplanes); LES_COUNT_LAUNCH();
  CHK(B.out());
  return finish(c);
}
int les_unpadd(les_ctx* c, double* cc, const double* cc_big, int nplanes) {
  if (!c || !cc || !cc_big || nplanes < 1) return LES_ERR_ARG;
  const Grid& g = c->g;
  Arg S(c, cc, g.nplane * nplanes), B(c, cc_big, g.nplane_big * nplanes);
  CHK(S.alloc()); CHK(B.in());
  k_unpadd<<<256, 256, 0, c->stream>>>((double2*)S.dev, (const double2*)B.dev, g.lh, g.ny, g.lh_big, g.ny2, g.nx, nplanes); LES_COUNT_LAUNCH();
  CHK(S.out());
  return finish(c);
}
}  // extern "C"
