// Per-routine device operations and the fused FP64 time step.
// Every kernel cites the reference routine it restates (file:line).
#include <algorithm>
#include <type_traits>
#include <cmath>
#include "les_internal.h"

namespace les {

typedef double2 C2;
struct Ptr6 { const double* p[6]; };

// ---------------------------------------------------------------------------
// self-test of the integer-pipe conversions against the hardware ones:
// n doubles built from SplitMix64 bit patterns (all exponents, both signs),
// halfway cases between adjacent floats, and every float rebuilt from the
// same patterns; counts results whose bits differ
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
__global__ void k_cvt_selftest(size_t n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long nb = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long r = splitmix64(seed + i);
    double x = __longlong_as_double((long long)r);
    if ((i & 3) == 1) {  // a double near the float range
      x = __longlong_as_double((long long)((r & 0x800fffffffffffffull) | ((0x380ull + (r >> 40) % 0x100ull) << 52)));
    } else if ((i & 3) == 2) {  // exactly halfway between two floats
      const unsigned fb = (unsigned)(r >> 32) & 0x7f7fffffu;
      const double lo = (double)__uint_as_float(fb), hi = (double)__uint_as_float(fb + 1u);
      x = 0.5 * (lo + hi);
    }
    if (__float_as_uint(cvt_d2f(x)) != __float_as_uint((float)x) && !(x != x)) ++nb;
    const float f = __uint_as_float((unsigned)r);
    if (__double_as_longlong(cvt_f2d(f)) != __double_as_longlong((double)f) && !(f != f)) ++nb;
  }
  if (nb) atomicAdd(bad, nb);
}
int op_cvt_selftest(size_t n, unsigned long long seed, unsigned long long* bad_dev, cudaStream_t s) {
  k_cvt_selftest<<<152 * 4, 256, 0, s>>>(n, seed, bad_dev); LES_COUNT_LAUNCH();
  return 0;
}

// ---------------------------------------------------------------------------
// launch helpers
static inline dim3 grid1(size_t n, int bs = 256) {
  size_t b = (n + bs - 1) / bs;
  if (b > 152 * 64) b = 152 * 64;
  if (b == 0) b = 1;
  return dim3((unsigned)b);
}
#define GSTRIDE(i, n) for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (n); i += (size_t)gridDim.x * blockDim.x)

__global__ void k_fill(double* p, size_t n, double v) { GSTRIDE(i, n) p[i] = v; }
static void fill(les_ctx* c, double* p, size_t n, double v) {
  if (n) { k_fill<<<grid1(n), 256, 0, c->stream>>>(p, n, v); LES_COUNT_LAUNCH(); }
}

// ---------------------------------------------------------------------------
// spectral pipeline helpers (T: transform precision; TIn/TOut: physical storage)
template <typename T, typename TIn>
static int r2cT(les_ctx* c, int nf, int nlev, const TIn* const* in, long pstride, const double* scale,
                const double* div, void* ws, bool big, int ncols, const double* const* off = nullptr) {
  typedef typename CT<T>::type CX;
  const Grid& g = c->g;
  for (int f0 = 0; f0 < nf; f0 += JOB_MAXF) {
    const int n = std::min(JOB_MAXF, nf - f0);
    RowJob J{};
    J.nfield = n; J.nlev = nlev;
    J.ny = big ? g.ny2 : g.ny;
    J.ld = big ? g.ld_big : g.ld;
    J.wc = big ? g.nx / 2 : g.lh;
    J.ncols = ncols;
    J.pstride_phys = pstride;
    J.pstride_work = (long)J.ny * J.wc;
    J.rpc = sizeof(T) == 8 ? (big ? c->rpcb64 : c->rpc64) : (big ? c->rpcb32 : c->rpc32);
    for (int f = 0; f < n; ++f) {
      J.phys[f] = in[f0 + f];
      J.work[f] = (CX*)ws + (size_t)(f0 + f) * nlev * J.pstride_work;
      J.scale[f] = scale ? scale[f0 + f] : 1.0;
      J.div[f] = div ? div[f0 + f] : 0.0;
      J.off[f] = off ? off[f0 + f] : nullptr;
    }
    launch_rows_r2c<T, TIn>(J, big ? c->rxb.r : c->rx.r, c->stream);
  }
  return 0;
}
template <typename T, typename TOut>
static int c2rT(les_ctx* c, int nf, int nlev, void* ws, TOut* const* out, long pstride, bool big, int ncols,
                const double* const* off = nullptr) {
  typedef typename CT<T>::type CX;
  const Grid& g = c->g;
  for (int f0 = 0; f0 < nf; f0 += JOB_MAXF) {
    const int n = std::min(JOB_MAXF, nf - f0);
    RowJob J{};
    J.nfield = n; J.nlev = nlev;
    J.ny = big ? g.ny2 : g.ny;
    J.ld = big ? g.ld_big : g.ld;
    J.wc = big ? g.nx / 2 : g.lh;
    J.ncols = ncols;
    J.pstride_phys = pstride;
    J.pstride_work = (long)J.ny * J.wc;
    J.rpc = sizeof(T) == 8 ? (big ? c->rpcb64 : c->rpc64) : (big ? c->rpcb32 : c->rpc32);
    for (int f = 0; f < n; ++f) {
      J.phys[f] = out[f0 + f];
      J.work[f] = (CX*)ws + (size_t)(f0 + f) * nlev * J.pstride_work;
      J.scale[f] = 1.0;
      J.div[f] = 0.0;
      J.off[f] = off ? off[f0 + f] : nullptr;
    }
    launch_rows_c2r<T, TOut>(J, big ? c->rxb.r : c->rx.r, c->stream);
  }
  return 0;
}
static int r2c(les_ctx* c, int nf, int nlev, const double* const* in, long pstride,
               const double* scale, const double* div, void* ws, bool big, int ncols) {
  return r2cT<double, double>(c, nf, nlev, in, pstride, scale, div, ws, big, ncols);
}
static int c2r(les_ctx* c, int nf, int nlev, void* ws, double* const* out, long pstride, bool big,
               int ncols) {
  return c2rT<double, double>(c, nf, nlev, ws, out, pstride, big, ncols);
}
static ColJob coljob(les_ctx* c, int map, int dir, int nlev) {
  const Grid& g = c->g;
  ColJob J{};
  J.nlev = nlev; J.map = map; J.dir = dir; J.nf = 1;
  J.inv_mask = (dir & DIR_INV) ? 0xffffffffu : 0u;
  J.ny_small = g.ny;
  J.kx = c->kx; J.ky = c->ky; J.G = c->G; J.GG = c->GG; J.lh = g.lh;
  J.kxf = c->kxf; J.kyf = c->kyf; J.Gf = c->Gf; J.GGf = c->GGf;
  J.kxd = c->kxd; J.kyd = c->kyd;
  if (map == MAP_SAME) {
    J.ny_in = J.ny_out = g.ny; J.ncols = g.lh; J.wc_in = J.wc_out = g.lh;
  } else if (map == MAP_PAD) {
    J.ny_in = g.ny; J.ny_out = g.ny2; J.ncols = g.nx / 2; J.wc_in = g.lh; J.wc_out = g.nx / 2;
  } else {
    J.ny_in = g.ny2; J.ny_out = g.ny; J.ncols = g.nx / 2; J.wc_in = g.nx / 2; J.wc_out = g.lh;
  }
  J.ps_in = (long)J.ny_in * J.wc_in;
  J.ps_out = (long)J.ny_out * J.wc_out;
  return J;
}
template <typename T, typename CIn>
static int colsT(les_ctx* c, const ColJob& J0) {
  ColJob J = J0;
  J.tx = sizeof(T) == 8 ? c->tx64 : c->tx32;
  const FftPlanDev& Pin = (J.ny_in == c->g.ny) ? c->cy.c : c->cyb.c;
  const FftPlanDev& Pout = (J.ny_out == c->g.ny) ? c->cy.c : c->cyb.c;
  return launch_cols<T, CIn>(J, Pin, Pout, c->stream);
}
static int cols(les_ctx* c, const ColJob& J) { return colsT<double, double2>(c, J); }

// ---------------------------------------------------------------------------
// deterministic reductions (fixed order, fixed tree)
// Sum of f(1:nx, r0+1:r1) of one plane per block (512 threads): warp w takes
// rows r0+w, r0+w+16, ..; lane l the columns l, l+32, ..; four independent
// partial sums per thread, then a fixed-order tree, so the result is
// deterministic.
template <typename TI>
__device__ __forceinline__ double plane_sum_block(const TI* p, int ld, int nx, int r0, int r1, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  for (int jy = r0 + wid; jy < r1; jy += 16) {
    const TI* row = p + (size_t)jy * ld;
    int jx = lane;
    for (; jx + 96 < nx; jx += 128) {
      a0 += cvt<double>(row[jx]); a1 += cvt<double>(row[jx + 32]);
      a2 += cvt<double>(row[jx + 64]); a3 += cvt<double>(row[jx + 96]);
    }
    for (; jx < nx; jx += 32) a0 += cvt<double>(row[jx]);
  }
  sh[threadIdx.x] = (a0 + a1) + (a2 + a3);
  __syncthreads();
  for (int w = 256; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  return sh[0];
}
// Row-split plane sums: block (q, j) sums rows [q rows, (q+1) rows) of plane
// j into part[j nsplit + q]; k_plane_fin adds the nsplit partial sums of a
// plane in order and divides by div (1: sums; nx*ny: means).  Several blocks
// per plane keep more loads in flight than one block per plane; the order
// stays fixed, so the result is deterministic.
template <typename TI>
__global__ void __launch_bounds__(512) k_plane_part(const TI* f, long pstride, int ld, int nx, int ny, int rows,
                                                    double* part) {
  __shared__ double sh[512];
  const int r0 = blockIdx.x * rows, r1 = min(r0 + rows, ny);
  const double t = plane_sum_block(f + (size_t)blockIdx.y * pstride, ld, nx, r0, r1, sh);
  if (threadIdx.x == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
}
__global__ void k_plane_fin(const double* __restrict__ part, int nsplit, int nplanes, double div, double* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nplanes) {
    double s = 0.0;
    for (int q = 0; q < nsplit; ++q) s += part[(size_t)j * nsplit + q];
    out[j] = s / div;
  }
}
// sums (div 1) or means (div nx*ny) of f(1:nx,1:ny) over nplanes planes;
// nsplit * nplanes <= 4 (nz + 8)
template <typename TI>
static void plane_sums(les_ctx* c, const TI* f, long pstride, int nplanes, int nsplit, double div, double* out) {
  const Grid& g = c->g;
  double* part = c->dred + 24 * (size_t)(g.nz + 8);
  const int rows = (g.ny + nsplit - 1) / nsplit;
  k_plane_part<TI><<<dim3(nsplit, nplanes), 512, 0, c->stream>>>(f, pstride, g.ld, g.nx, g.ny, rows, part); LES_COUNT_LAUNCH();
  k_plane_fin<<<(nplanes + 127) / 128, 128, 0, c->stream>>>(part, nsplit, nplanes, div, out); LES_COUNT_LAUNCH();
}

// ---------------------------------------------------------------------------
// ddz_uv.f90:36-55 and ddz_w.f90:81-106 (non-MPI)
// grid (ceil(np/256), nz): no 64-bit index division
__global__ void __launch_bounds__(256) k_ddz(double* __restrict__ dfdz, const double* __restrict__ f, int ld,
                                             int nx, int ny, int nz, double cst, int uv) {
  const unsigned np = (unsigned)ld * ny;
  const unsigned r = blockIdx.x * 256u + threadIdx.x;
  if (r >= np) return;
  const int jz = blockIdx.y + 1;
  const size_t i = (size_t)(jz - 1) * np + r;
  if (jz == nz) { dfdz[i] = 0.0; return; }
  if ((int)(r % (unsigned)ld) >= nx) return;
  if (uv) {
    if (jz >= 2) dfdz[i] = cst * (f[i] - f[i - np]);
  } else {
    dfdz[i] = cst * (f[i + np] - f[i]);
  }
}
int op_ddz(les_ctx* c, double* dfdz, const double* f, int uv) {
  const Grid& g = c->g;
  k_ddz<<<dim3((unsigned)((g.nplane + 255) / 256), (unsigned)g.nz), 256, 0, c->stream>>>(dfdz, f, g.ld, g.nx, g.ny,
                                                                                      g.nz, 1.0 / g.dz, uv);
  LES_COUNT_LAUNCH();
  return 0;
}

// ---------------------------------------------------------------------------
// filt_da.f90:3-42 for nf fields at once
static int filt_da_multi(les_ctx* c, double* const* f, double* const* dx, double* const* dy, int nf,
                         int nlev) {
  const Grid& g = c->g;
  double sc[JOB_MAXF];
  for (int i = 0; i < nf; ++i) sc[i] = 1.0 / (double)(g.nx * g.ny);
  const double* in[JOB_MAXF];
  for (int i = 0; i < nf; ++i) in[i] = f[i];
  r2c(c, nf, nlev, in, (long)g.nplane, sc, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nlev);
  J.nin = 1; J.nout = 3; J.nf = nf;
  J.in[0] = c->wsA; J.fs_in = (long)nlev * g.C;
  J.out[0] = c->wsB;
  J.out[1] = (C2*)c->wsB + (size_t)nf * nlev * g.C;
  J.out[2] = (C2*)c->wsB + (size_t)2 * nf * nlev * g.C;
  J.fs_out = (long)nlev * g.C;
  J.coef[0][0] = CC_KILL; J.coef[1][0] = CC_IKX; J.coef[2][0] = CC_IKY;
  cols(c, J);
  double* out[3 * JOB_MAXF];
  for (int i = 0; i < nf; ++i) { out[i] = f[i]; out[nf + i] = dx[i]; out[2 * nf + i] = dy[i]; }
  c2r(c, 3 * nf, nlev, c->wsB, out, (long)g.nplane, false, g.lh);
  return 0;
}
// filt_da with the Nyquist-filtered spectra F(f/(nx*ny)) also stored in
// `spec` (field stride nlev*C) for reuse by the fused step
int filt_da_multi_spec(les_ctx* c, double* const* f, double* const* dx, double* const* dy, int nf, int nlev,
                       C2* spec) {
  const Grid& g = c->g;
  double sc[JOB_MAXF];
  for (int i = 0; i < nf; ++i) sc[i] = 1.0 / (double)(g.nx * g.ny);
  const double* in[JOB_MAXF];
  for (int i = 0; i < nf; ++i) in[i] = f[i];
  r2c(c, nf, nlev, in, (long)g.nplane, sc, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nlev);
  J.nin = 1; J.nout = 4; J.nf = nf;
  J.inv_mask = 7u;  // outputs 0..2 back to physical space, output 3 kept spectral
  J.in[0] = c->wsA; J.fs_in = (long)nlev * g.C;
  J.out[0] = c->wsB;
  J.out[1] = (C2*)c->wsB + (size_t)nf * nlev * g.C;
  J.out[2] = (C2*)c->wsB + (size_t)2 * nf * nlev * g.C;
  J.out[3] = spec;
  J.fs_out = (long)nlev * g.C;
  J.coef[0][0] = CC_KILL; J.coef[1][0] = CC_IKX; J.coef[2][0] = CC_IKY; J.coef[3][0] = CC_KILL;
  cols(c, J);
  double* out[3 * JOB_MAXF];
  for (int i = 0; i < nf; ++i) { out[i] = f[i]; out[nf + i] = dx[i]; out[2 * nf + i] = dy[i]; }
  c2r(c, 3 * nf, nlev, c->wsB, out, (long)g.nplane, false, g.lh);
  return 0;
}
// filt_da.f90:3-42 Nyquist removal done in physical space, in FP64.  With
// a(x) = (1/ny) sum_y (-1)^y f(x,y), b(y) = (1/nx) sum_x (-1)^x f(x,y) and
// c = (1/nx) sum_x (-1)^x a(x), the part of f on the modes ky = ny/2 (every
// kx) and kx = nx/2 (every ky) is (-1)^y a(x) + (-1)^x b(y) - (-1)^(x+y) c,
// which is what the forward transform, the zeroing of those modes and the
// inverse transform remove; here it is removed exactly, up to FP64
// rounding, with no transform.  Three kernels, every sum in a fixed order
// (deterministic), no FP64 work on idle lanes (the FP64 pipe is the scarce
// unit on this part):
//   k_nyq_part   per (16-row chunk, level, field): the chunk's partial
//                a(x) (unnormalised), b(y) of its rows, its plain sum;
//   k_nyq_comb   per (level, field): a(x) -/+ c for even/odd x, the mean;
//   k_nyq_apply  every point: f -= (-1)^y (a - (-1)^x c) + (-1)^x b.
constexpr int NYQ_ROWS = 16;
struct NyqScratch {
  double* apart;  // [field][level][chunk][nx]
  double* b;      // [field][level][ny]
  double* spart;  // [field][level][chunk]
  double* ac;     // [field][level][nx]  a(x) - c (x even), a(x) + c (x odd)
};
template <int K>
__global__ void k_nyq_part(const double* f0, const double* f1, const double* f2, NyqScratch S, int ld, int nx,
                           int ny, long ps, int nlev, int nch) {
  __shared__ double ws[8][NYQ_ROWS], wd[8][NYQ_ROWS];
  const int ch = blockIdx.x, lev = blockIdx.y, fld = blockIdx.z;
  const double* f = (fld == 0 ? f0 : fld == 1 ? f1 : f2) + (size_t)lev * ps;
  const int np = nx / 2, lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int y0 = ch * NYQ_ROWS, nr = min(NYQ_ROWS, ny - y0);
  double2 acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = make_double2(0.0, 0.0);
#pragma unroll 4
  for (int r = 0; r < nr; ++r) {
    const int y = y0 + r;
    const double2* row = reinterpret_cast<const double2*>(f + (size_t)y * ld);
    double se = 0.0, so = 0.0;  // sums over even / odd x
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int p = threadIdx.x + k * blockDim.x;
      if (p < np) {
        const double2 v = row[p];
        if (y & 1) { acc[k].x -= v.x; acc[k].y -= v.y; }
        else { acc[k].x += v.x; acc[k].y += v.y; }
        se += v.x;
        so += v.y;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      se += __shfl_xor_sync(0xffffffffu, se, o);
      so += __shfl_xor_sync(0xffffffffu, so, o);
    }
    if (lane == 0) { ws[wid][r] = se + so; wd[wid][r] = se - so; }
  }
  const size_t pl = (size_t)fld * nlev + lev;
  double* ap = S.apart + (pl * nch + ch) * nx;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int p = threadIdx.x + k * blockDim.x;
    if (p < np) reinterpret_cast<double2*>(ap)[p] = acc[k];
  }
  __syncthreads();
  if (threadIdx.x < nr) {
    double b = 0.0;
    for (int w = 0; w < nw; ++w) b += wd[w][threadIdx.x];
    S.b[pl * ny + y0 + threadIdx.x] = b / (double)nx;
  }
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int r = 0; r < nr; ++r)
      for (int w = 0; w < nw; ++w) t += ws[w][r];
    S.spart[pl * nch + ch] = t;
  }
}
// The same partial sums with whole rows per warp: 4 warps, warp w takes rows
// w, w+4, .. of the chunk; lane l the column pairs l + 32k, k < KP.  Each
// lane sums its pairs before one warp reduction per row, and the four warps'
// column partials are combined once per chunk (fewer FP64 adds per element
// than one warp reduction per row across all the columns).
template <int KP>
__global__ void __launch_bounds__(128) k_nyq_part_rows(const double* f0, const double* f1, const double* f2,
                                                      NyqScratch S, int ld, int nx, int ny, long ps, int nlev,
                                                      int nch) {
  // per-lane partial row sums over even / odd x, summed once per row below
  // (31 adds per row instead of a 5-step warp reduction on every lane)
  __shared__ double pse[NYQ_ROWS][33], pso[NYQ_ROWS][33], ws[NYQ_ROWS];
  extern __shared__ double2 wacc[];  // [4][np]
  const int ch = blockIdx.x, lev = blockIdx.y, fld = blockIdx.z;
  const double* f = (fld == 0 ? f0 : fld == 1 ? f1 : f2) + (size_t)lev * ps;
  const int np = nx / 2, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int y0 = ch * NYQ_ROWS, nr = min(NYQ_ROWS, ny - y0);
  double2 acc[KP];
#pragma unroll
  for (int k = 0; k < KP; ++k) acc[k] = make_double2(0.0, 0.0);
  for (int r = wid; r < nr; r += 4) {
    const int y = y0 + r;
    const double2* row = reinterpret_cast<const double2*>(f + (size_t)y * ld);
    const double sg = (y & 1) ? -1.0 : 1.0;  // one FMA per element, no predicated pair
    double se = 0.0, so = 0.0;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int p = lane + 32 * k;
      if (p < np) {
        const double2 v = row[p];
        acc[k].x = fma(sg, v.x, acc[k].x);
        acc[k].y = fma(sg, v.y, acc[k].y);
        se += v.x;
        so += v.y;
      }
    }
    pse[r][lane] = se;
    pso[r][lane] = so;
  }
#pragma unroll
  for (int k = 0; k < KP; ++k) {
    const int p = lane + 32 * k;
    if (p < np) wacc[wid * np + p] = acc[k];
  }
  __syncthreads();
  const size_t pl = (size_t)fld * nlev + lev;
  double2* ap = reinterpret_cast<double2*>(S.apart + (pl * nch + ch) * nx);
  for (int p = threadIdx.x; p < np; p += 128) {
    double2 a = wacc[p];
    for (int w = 1; w < 4; ++w) { a.x += wacc[w * np + p].x; a.y += wacc[w * np + p].y; }
    ap[p] = a;
  }
  if (threadIdx.x < nr) {
    double e = 0.0, o = 0.0;
    for (int l = 0; l < 32; ++l) { e += pse[threadIdx.x][l]; o += pso[threadIdx.x][l]; }
    ws[threadIdx.x] = e + o;
    S.b[pl * ny + y0 + threadIdx.x] = (e - o) / (double)nx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int r = 0; r < nr; ++r) t += ws[r];
    S.spart[pl * nch + ch] = t;
  }
}
__global__ void __launch_bounds__(256) k_nyq_comb(NyqScratch S, double* mean, int mstride, int nx, int ny, int nlev,
                                                  int nch) {
  __shared__ double red[256];
  const int lev = blockIdx.x, fld = blockIdx.y;
  const size_t pl = (size_t)fld * nlev + lev;
  const double iny = 1.0 / (double)ny;
  double cp = 0.0;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    double a = 0.0;
    for (int ch = 0; ch < nch; ++ch) a += S.apart[(pl * nch + ch) * nx + x];
    a *= iny;
    S.ac[pl * nx + x] = a;
    cp += (x & 1) ? -a : a;
  }
  red[threadIdx.x] = cp;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double c = red[0] / (double)nx;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) S.ac[pl * nx + x] += (x & 1) ? c : -c;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int ch = 0; ch < nch; ++ch) t += S.spart[pl * nch + ch];
    mean[(size_t)fld * mstride + lev] = t / ((double)nx * (double)ny);
  }
}
// f -= (-1)^y a(x) + (-1)^x b(y) in FP64 (an FP32 correction would leave
// rounding noise in every mode, divergence included).  grid (ceil(ny (nx/2+1)
// / 256), nf nlev).
__global__ void __launch_bounds__(256) k_nyq_apply(double* f0, double* f1, double* f2, NyqScratch S, int ld,
                                                   int nx, int ny, long ps, int nlev) {
  const int np1 = nx / 2 + 1;  // pairs per row, the last one the padding columns
  const unsigned r = blockIdx.x * 256u + threadIdx.x;
  if (r >= (unsigned)ny * np1) return;
  const int pl = blockIdx.y;
  const int y = (int)(r / (unsigned)np1), p = (int)(r - (unsigned)y * np1);
  const int fld = pl / nlev, lev = pl - fld * nlev;
  double* f = (fld == 0 ? f0 : fld == 1 ? f1 : f2) + (size_t)lev * ps + (size_t)y * ld;
  double2* q = reinterpret_cast<double2*>(f) + p;
  if (p == np1 - 1) { *q = make_double2(0.0, 0.0); return; }  // padding columns ld-1:ld
  const double2 ac = reinterpret_cast<const double2*>(S.ac + (size_t)pl * nx)[p];
  const double b = S.b[(size_t)pl * ny + y];
  const double sg = (y & 1) ? -1.0 : 1.0;
  double2 v = *q;
  v.x = v.x - fma(sg, ac.x, b);   // even x: (-1)^x = +1
  v.y = v.y - fma(sg, ac.y, -b);  // odd x
  *q = v;
}
// nf <= 3 fields of nlev levels, in place; plane means to mean[f*mstride+lev];
// scratch (a few MB) in the given work buffer
static void nyq_kill(les_ctx* c, double* const* f, int nf, int nlev, double* mean, int mstride, void* scratch) {
  const Grid& g = c->g;
  const int nch = (g.ny + NYQ_ROWS - 1) / NYQ_ROWS;
  const size_t npl = (size_t)nf * nlev;
  NyqScratch S;
  S.apart = static_cast<double*>(scratch);
  S.b = S.apart + npl * nch * g.nx;
  S.spart = S.b + npl * g.ny;
  S.ac = S.spart + npl * nch + 2;  // keeps ac 16-byte aligned (npl*nch even or padded)
  if ((reinterpret_cast<uintptr_t>(S.ac) & 15) != 0) S.ac += 1;
  double* f0 = f[0];
  double* f1 = nf > 1 ? f[1] : f[0];
  double* f2 = nf > 2 ? f[2] : f[0];
  const int np = g.nx / 2;
  const int bt = std::min(256, (np + 31) / 32 * 32);
  const int K = (np + bt - 1) / bt;  // <= 16: nx <= 8192 (the transforms allow less)
  const dim3 grid(nch, nlev, nf);
  const long ps = (long)g.nplane;
  const int KP = (np + 31) / 32;
  const size_t smr = (size_t)4 * np * sizeof(double2);
  if (KP <= 8) {
    switch (KP) {
      case 1: k_nyq_part_rows<1><<<grid, 128, smr, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
      case 2: k_nyq_part_rows<2><<<grid, 128, smr, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
      case 3: case 4: k_nyq_part_rows<4><<<grid, 128, smr, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
      default: k_nyq_part_rows<8><<<grid, 128, smr, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
    }
  } else switch (K) {
    case 1: k_nyq_part<1><<<grid, bt, 0, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
    case 2: k_nyq_part<2><<<grid, bt, 0, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
    case 3: case 4: k_nyq_part<4><<<grid, bt, 0, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
    case 5: case 6: case 7: case 8:
      k_nyq_part<8><<<grid, bt, 0, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
    default: k_nyq_part<16><<<grid, bt, 0, c->stream>>>(f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev, nch); break;
  }
  LES_COUNT_LAUNCH();
  k_nyq_comb<<<dim3(nlev, nf), 256, 0, c->stream>>>(S, mean, mstride, g.nx, g.ny, nlev, nch); LES_COUNT_LAUNCH();
  k_nyq_apply<<<dim3((unsigned)((g.ny * (np + 1) + 255) / 256), (unsigned)npl), 256, 0, c->stream>>>(
      f0, f1, f2, S, g.ld, g.nx, g.ny, ps, nlev);
  LES_COUNT_LAUNCH();
}

// FP32 spectra of f - mean(level) -> the FP64 spectra F(f/(nx*ny)) the fused
// step reads: the (0,0) mode is the FP64 plane mean itself
__global__ void k_spec_widen(const float2* __restrict__ s, double2* __restrict__ d, const double* __restrict__ mean,
                             int mstride, size_t fs, size_t nk, int nf) {
  GSTRIDE(t, fs * nf) {
    const size_t fld = t / fs, r = t - fld * fs;
    const size_t lev = r / nk, m = r - lev * nk;
    const float2 v = s[t];
    d[t] = m == 0 ? make_double2(mean[fld * mstride + lev], 0.0) : make_double2((double)v.x, (double)v.y);
  }
}

// Mixed-form filt_da of u, v, w: the Nyquist removal in FP64 in physical
// space (the velocities keep FP64 accuracy); the six horizontal
// derivatives, which feed only the SGS strain (S_ij), and the saved spectra,
// which feed the FP32 convective, SGS and padding transforms, from one FP32
// transform of f - plane mean.  rmsdiv's FP64 dudx + dvdy are formed on the
// steps that report it (step_rmsdiv_mixed).
static int filt_da_uvw_mixed(les_ctx* c) {
  const Grid& g = c->g;
  const int nz = g.nz;
  const long FS = (long)nz * g.C;
  double* f3[3] = {c->f[LES_U], c->f[LES_V], c->f[LES_W]};
  const int ms = nz + 8;
  double* mean = c->dred + 16 * (size_t)ms;  // u, v, w plane means
  nyq_kill(c, f3, 3, nz, mean, ms, c->wsB);
  const double sc = 1.0 / (double)(g.nx * g.ny);
  const double* in[3] = {f3[0], f3[1], f3[2]};
  const double scs[3] = {sc, sc, sc};
  const double* offs[3] = {mean, mean + ms, mean + 2 * ms};
  r2cT<float, double>(c, 3, nz, in, (long)g.nplane, scs, nullptr, c->wsA, false, g.lh, offs);
  float2* ob = (float2*)c->wsB;
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nz);
  J.nin = 1; J.nout = 3; J.nf = 3; J.inv_mask = 6u;  // output 0 (the spectrum) stays spectral
  J.in[0] = c->wsA; J.fs_in = FS;
  J.out[0] = ob + 6 * FS; J.out[1] = ob; J.out[2] = ob + 3 * FS; J.fs_out = FS;
  J.coef[0][0] = CC_KILL; J.coef[1][0] = CC_IKX; J.coef[2][0] = CC_IKY;
  colsT<float, float2>(c, J);
  k_spec_widen<<<grid1(3 * (size_t)FS), 256, 0, c->stream>>>(ob + 6 * FS, c->spec, mean, ms, (size_t)FS, g.C, 3);
  LES_COUNT_LAUNCH();
  float* o6[6] = {f32(c, LES_DUDX), f32(c, LES_DVDX), f32(c, LES_DWDX), f32(c, LES_DUDY), f32(c, LES_DVDY),
                  f32(c, LES_DWDY)};  // FP32-held in the mixed form
  c2rT<float, float>(c, 6, nz, c->wsB, o6, (long)g.nplane, false, g.lh);
  return 0;
}

int op_filt_da(les_ctx* c, double* f, double* dfdx, double* dfdy, int nlev) {
  double* a[1] = {f}; double* b[1] = {dfdx}; double* d[1] = {dfdy};
  return filt_da_multi(c, a, b, d, 1, nlev);
}
// ddx.f90 / ddy.f90 / ddxy.f90 (dfdx or dfdy may be null)
int op_ddxy(les_ctx* c, double* dfdx, double* dfdy, const double* f, int nlev) {
  const Grid& g = c->g;
  double sc = 1.0 / (double)(g.nx * g.ny);
  r2c(c, 1, nlev, &f, (long)g.nplane, &sc, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nlev);
  J.nin = 1; J.nout = 0;
  J.in[0] = c->wsA;
  double* out[2]; int no = 0;
  if (dfdx) { J.out[J.nout] = (C2*)c->wsB + (size_t)J.nout * nlev * g.C; J.coef[J.nout][0] = CC_IKX; out[no++] = dfdx; J.nout++; }
  if (dfdy) { J.out[J.nout] = (C2*)c->wsB + (size_t)J.nout * nlev * g.C; J.coef[J.nout][0] = CC_IKY; out[no++] = dfdy; J.nout++; }
  cols(c, J);
  c2r(c, no, nlev, c->wsB, out, (long)g.nplane, false, g.lh);
  return 0;
}
// test_filtermodule.f90:13-30 on nplanes planes; which = 0 (G_test) / 1 (G_test_test)
int op_test_filter(les_ctx* c, double* out, const double* in, int nplanes, int which, long pstride) {
  const Grid& g = c->g;
  r2c(c, 1, nplanes, &in, pstride, nullptr, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nplanes);
  J.nin = 1; J.nout = 1; J.in[0] = c->wsA; J.out[0] = c->wsB;
  J.coef[0][0] = which == 0 ? CC_G : CC_GG;
  cols(c, J);
  c2r(c, 1, nplanes, c->wsB, &out, pstride, false, g.lh);
  return 0;
}
// plain transforms (rfftwnd_f77_one_*), in place on (ld,ny) planes
int op_fft(les_ctx* c, double* planes, int nplanes, int big, int inverse) {
  const Grid& g = c->g;
  const long ps = big ? (long)g.nplane_big : (long)g.nplane;
  const int lhh = big ? g.lh_big : g.lh;
  const int nyy = big ? g.ny2 : g.ny;
  // full-width work planes for these entry points
  RowJob J{};
  J.nfield = 1; J.nlev = nplanes; J.ny = nyy; J.ld = big ? g.ld_big : g.ld;
  J.wc = lhh; J.ncols = lhh; J.pstride_phys = ps; J.pstride_work = (long)nyy * lhh;
  J.phys[0] = planes; J.work[0] = c->wsA; J.scale[0] = 1.0; J.div[0] = 0.0;
  ColJob K{};
  K.nin = 1; K.nout = 1; K.nlev = nplanes; K.nf = 1; K.ny_in = K.ny_out = nyy; K.map = MAP_SAME;
  K.inv_mask = inverse ? 1u : 0u;
  K.ncols = lhh; K.ny_small = nyy; K.wc_in = K.wc_out = lhh; K.ps_in = K.ps_out = (long)nyy * lhh;
  K.coef[0][0] = CC_ONE; K.kx = c->kx; K.ky = c->ky; K.G = c->G; K.GG = c->GG; K.lh = g.lh;
  K.kxf = c->kxf; K.kyf = c->kyf; K.Gf = c->Gf; K.GGf = c->GGf;
  const HostRealPlan& rp = big ? c->rxb : c->rx;
  const HostPlan& cp = big ? c->cyb : c->cy;
  if (!inverse) {
    launch_rows_r2c<double, double>(J, rp.r, c->stream);
    K.dir = DIR_FWD; K.in[0] = c->wsA; K.out[0] = c->wsB;
    launch_cols<double, double2>(K, cp.c, cp.c, c->stream);
    // copy spectra back into the planes (complex view of (ld,ny))
    cudaMemcpy2DAsync(planes, (size_t)J.ld * sizeof(double), c->wsB, (size_t)lhh * sizeof(C2),
                      (size_t)lhh * sizeof(C2), (size_t)nyy * nplanes, cudaMemcpyDeviceToDevice, c->stream);
  } else {
    cudaMemcpy2DAsync(c->wsA, (size_t)lhh * sizeof(C2), planes, (size_t)J.ld * sizeof(double),
                      (size_t)lhh * sizeof(C2), (size_t)nyy * nplanes, cudaMemcpyDeviceToDevice, c->stream);
    K.dir = DIR_INV; K.in[0] = c->wsA; K.out[0] = c->wsB;
    launch_cols<double, double2>(K, cp.c, cp.c, c->stream);
    J.work[0] = c->wsB;
    launch_rows_c2r<double, double>(J, rp.r, c->stream);
  }
  return 0;
}

// dealias1.f90:1-31 for nf fields: small (ld,ny,nlev) -> big (ld_big,ny2,nlev)
int op_dealias1(les_ctx* c, const double* const* in, double* const* out, int nf, int nlev) {
  const Grid& g = c->g;
  double sc[JOB_MAXF];
  for (int i = 0; i < nf; ++i) sc[i] = 1.0 / (double)(g.nx * g.ny);
  r2c(c, nf, nlev, in, (long)g.nplane, sc, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_PAD, DIR_BOTH, nlev);
  J.nin = 1; J.nout = 1; J.nf = nf;
  J.in[0] = c->wsA; J.fs_in = (long)nlev * g.C;
  J.out[0] = c->wsB; J.fs_out = (long)nlev * g.CB;
  J.coef[0][0] = CC_ONE;
  cols(c, J);
  c2r(c, nf, nlev, c->wsB, out, (long)g.nplane_big, true, g.nx / 2);
  return 0;
}
// dealias2.f90:1-33 for nf fields: big -> small; the big input is multiplied
// by `scale` (1/(nx2*ny2) in dealias2, 1 when the caller folded it in)
int op_dealias2(les_ctx* c, double* const* out, const double* const* in, int nf, int nlev, double scale) {
  const Grid& g = c->g;
  double sc[JOB_MAXF];
  for (int i = 0; i < nf; ++i) sc[i] = scale;
  r2c(c, nf, nlev, in, (long)g.nplane_big, sc, nullptr, c->wsA, true, g.nx / 2);
  ColJob J = coljob(c, MAP_UNPAD, DIR_BOTH, nlev);
  J.nin = 1; J.nout = 1; J.nf = nf;
  J.in[0] = c->wsA; J.fs_in = (long)nlev * g.CB;
  J.out[0] = c->wsB; J.fs_out = (long)nlev * g.C;
  J.coef[0][0] = CC_ONE;
  cols(c, J);
  c2r(c, nf, nlev, c->wsB, out, (long)g.nplane, false, g.nx / 2);
  return 0;
}

// ---------------------------------------------------------------------------
// scalars_module.f90:508-690 obukhov (patch_flag = 1); u1, v1 are the
// 4-delta filtered first-level velocities, theta_sum the plane sum of theta(1);
// sgs_q3 the surface moisture flux (null without humidity: qmix = 0)
__global__ void k_obukhov(const double* __restrict__ u1, const double* __restrict__ v1,
                          const double* __restrict__ theta, const double* __restrict__ zo,
                          const double* __restrict__ z_os, double* __restrict__ sgs_t3,
                          double* ustar_avg, double* psi_m, double* psi_m0, double* psi_h,
                          double* psi_h0, double* phi_m, double* phi_h, const double* theta_sum,
                          const double* __restrict__ sgs_q3, double q_scale,
                          int nx, int ny, int ld, double dz, double vonk, double g_, double nxny_f) {
  GSTRIDE(s, (size_t)nx * ny) {
    const int jy = (int)(s / nx), jx = (int)(s - (size_t)jy * nx);
    const size_t i = (size_t)jy * ld + jx;
    const double theta_ = theta_sum[0] / nxny_f;
    const double u_avg = sqrt(u1[i] * u1[i] + v1[i] * v1[i]);
    const double us = u_avg * vonk / (log(0.5 * dz / zo[s]) - psi_m[s] + psi_m0[s]);
    ustar_avg[s] = us;
    const double wt_avg = sgs_t3[s];
    // virtual buoyancy flux (scalars_module.f90:549-550)
    const double wtv_avg = sgs_q3 ? sgs_t3[s] + 0.61 * theta[i] * (0.001 * q_scale * sgs_q3[s])
                                  : sgs_t3[s] + 0.61 * theta[i] * (0.001 * 100.0 * 0.0);
    const double L = -(us * us * us) / (vonk * (g_ / theta_) * wtv_avg);
    double zeta = 0.5 * dz / L, zeta0 = zo[s] / L, zeta0s = z_os[s] / L;
    if (zeta < -30.0) zeta = -30.0;
    if (zeta > 2.0) zeta = 2.0;
    if (zeta0 < -30.0) zeta0 = -30.0;
    if (zeta0 > 2.0) zeta0 = 2.0;
    if (zeta0s < -30.0) zeta0s = -30.0;
    if (zeta0s > 2.0) zeta0s = 2.0;
    if (L < 0.0 && wt_avg != 0.0) {
      const double x = pow(1.0 - 16.0 * zeta, 0.25);
      psi_m[s] = 2.0 * log((1.0 + x) / 2.0) + log((1.0 + x * x) / 2.0) - 2.0 * atan(x) + LES_PI / 2.0;
      psi_h[s] = 2.0 * log((1.0 + x * x) / 2.0);
      phi_m[s] = 1.0 / x;
      phi_h[s] = 1.0 / (x * x);
      const double x0 = pow(1.0 - 16.0 * zeta0, 0.25);
      const double x0s = pow(1.0 - 16.0 * zeta0s, 0.25);
      psi_m0[s] = 2.0 * log((1.0 + x0) / 2.0) + log((1.0 + x0 * x0) / 2.0) - 2.0 * atan(x0) + LES_PI / 2.0;
      psi_h0[s] = 2.0 * log((1.0 + x0s * x0s) / 2.0);
    } else if (L > 0.0 && wt_avg != 0.0) {
      phi_m[s] = 1.0 + 5.0 * zeta;
      phi_h[s] = 1.0 + 5.0 * zeta;
      psi_m[s] = -1.0 * 5.0 * zeta;
      psi_h[s] = -1.0 * 5.0 * zeta;
      psi_m0[s] = -1.0 * 5.0 * zeta0;
      psi_h0[s] = -1.0 * 5.0 * zeta0s;
    } else {
      psi_m[s] = 0.0; psi_m0[s] = 0.0; psi_h[s] = 0.0; psi_h0[s] = 0.0;
      phi_m[s] = 1.0; phi_h[s] = 1.0;
    }
  }
}
__global__ void k_obukhov_init(double* psi_m, double* psi_m0, double* psi_h, double* psi_h0,
                               double* sgs_t3, const double* wt_s, double* sgs_q3, const double* wq_s,
                               size_t n, int initsc, double div, double divq) {
  GSTRIDE(s, n) {
    psi_m[s] = 0.0; psi_m0[s] = 0.0; psi_h[s] = 0.0; psi_h0[s] = 0.0;
    if (!initsc) {
      sgs_t3[s] = wt_s[s] / div;
      if (sgs_q3) sgs_q3[s] = wq_s[s] / divq;
    }
  }
}
// G_test_test-filtered surface u, v (test_filtermodule.f90:13-30 on the
// first level; obukhov and wallstress filter the same planes) as one
// two-field job: u1 at uv1, v1 at uv1 + nplane
static void surface_uv_filtered(les_ctx* c, double* uv1) {
  const Grid& g = c->g;
  const double* in[2] = {c->f[LES_U], c->f[LES_V]};
  r2c(c, 2, 1, in, (long)g.nplane, nullptr, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, 1);
  J.nin = 1; J.nout = 1; J.nf = 2;
  J.in[0] = c->wsA; J.fs_in = (long)g.C;
  J.out[0] = c->wsB; J.fs_out = (long)g.C;
  J.coef[0][0] = CC_GG;
  cols(c, J);
  double* out[2] = {uv1, uv1 + g.nplane};
  c2r(c, 2, 1, c->wsB, out, (long)g.nplane, false, g.lh);
}
// uv1: the filtered surface planes when the caller already has them, else
// null (filtered here into the first two temp planes)
int op_obukhov(les_ctx* c, const double* uv1) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  const size_t ns = (size_t)g.nx * g.ny;
  if (c->jt == 1) {  // SCAL_init = 1 (scalars_module.f90:525-542)
    k_obukhov_init<<<grid1(ns), 256, 0, c->stream>>>(c->f[LES_PSI_M], c->f[LES_PSI_M0], c->f[LES_PSI_H],
                                                     c->f[LES_PSI_H0], c->f[LES_SGS_T3_SFC], c->f[LES_WT_S],
                                                     c->f[LES_SGS_Q3_SFC], c->f[LES_WQ_S], ns, k.initsc,
                                                     k.u_star * k.t_scale, k.u_star * k.q_scale); LES_COUNT_LAUNCH();
  }
  plane_sums(c, c->f[LES_THETA], 0, 1, 16, 1.0, c->dscal + 0);
  if (!uv1) {
    surface_uv_filtered(c, c->tmp);
    uv1 = c->tmp;
  }
  const double* u1 = uv1;
  const double* v1 = uv1 + g.nplane;
  const double g_ = (k.g * k.z_i) / (k.u_star * k.u_star);
  k_obukhov<<<grid1(ns), 256, 0, c->stream>>>(u1, v1, c->f[LES_THETA], c->f[LES_ZO], c->z_os,
                                              c->f[LES_SGS_T3_SFC], c->f[LES_USTAR_AVG], c->f[LES_PSI_M],
                                              c->f[LES_PSI_M0], c->f[LES_PSI_H], c->f[LES_PSI_H0],
                                              c->f[LES_PHI_M], c->f[LES_PHI_H], c->dscal + 0,
                                              c->f[LES_SGS_Q3_SFC], k.q_scale, g.nx, g.ny,
                                              g.ld, g.dz, k.vonk, g_, (double)(float)(g.nx * g.ny)); LES_COUNT_LAUNCH();
  return 0;
}

// wallstress.f90:5-69 ('wall')
template <typename TT>  // storage of txz, tyz (FP32 in the mixed form)
__global__ void k_wallstress(const double* __restrict__ u, const double* __restrict__ v,
                             const double* __restrict__ u1, const double* __restrict__ v1,
                             const double* __restrict__ zo, const double* __restrict__ psi_m,
                             const double* __restrict__ psi_m0, const double* __restrict__ phi_m,
                             double* ustar_avg, TT* txz, TT* tyz, double* dudz, double* dvdz,
                             int nx, int ny, int ld, double dz, double vonk) {
  GSTRIDE(s, (size_t)nx * ny) {
    const int jy = (int)(s / nx), jx = (int)(s - (size_t)jy * nx);
    const size_t i = (size_t)jy * ld + jx;
    const double denom = log(0.5 * dz / zo[s]) - psi_m[s] + psi_m0[s];
    const double u_avg = sqrt(u1[i] * u1[i] + v1[i] * v1[i]);
    const double us = u_avg * vonk / denom;
    ustar_avg[s] = us;
    const double cst = -(us * us) / u_avg;
    txz[i] = cvt<TT, double>(cst * u1[i]);
    tyz[i] = cvt<TT, double>(cst * v1[i]);
    const double a = us / (0.5 * dz * vonk) * u1[i] / u_avg * phi_m[s];
    const double b = us / (0.5 * dz * vonk) * v1[i] / u_avg * phi_m[s];
    dudz[i] = (u[i] == 0.0) ? 0.0 : a;
    dvdz[i] = (v[i] == 0.0) ? 0.0 : b;
  }
}
int op_wallstress(les_ctx* c, const double* uv1) {
  const Grid& g = c->g;
  if (!uv1) {
    surface_uv_filtered(c, c->tmp);
    uv1 = c->tmp;
  }
  const double* u1 = uv1;
  const double* v1 = uv1 + g.nplane;
  if (c->cfg.precision == 1)
    k_wallstress<float><<<grid1((size_t)g.nx * g.ny), 256, 0, c->stream>>>(
        c->f[LES_U], c->f[LES_V], u1, v1, c->f[LES_ZO], c->f[LES_PSI_M], c->f[LES_PSI_M0], c->f[LES_PHI_M],
        c->f[LES_USTAR_AVG], f32(c, LES_TXZ), f32(c, LES_TYZ), c->f[LES_DUDZ], c->f[LES_DVDZ], g.nx, g.ny, g.ld,
        g.dz, c->cfg.vonk);
  else
    k_wallstress<double><<<grid1((size_t)g.nx * g.ny), 256, 0, c->stream>>>(
        c->f[LES_U], c->f[LES_V], u1, v1, c->f[LES_ZO], c->f[LES_PSI_M], c->f[LES_PSI_M0], c->f[LES_PHI_M],
        c->f[LES_USTAR_AVG], c->f[LES_TXZ], c->f[LES_TYZ], c->f[LES_DUDZ], c->f[LES_DVDZ], g.nx, g.ny, g.ld,
        g.dz, c->cfg.vonk);
  LES_COUNT_LAUNCH();
  return 0;
}

// ---------------------------------------------------------------------------
// sgs_stag.f90:371-498 calc_Sij ('wall') fused with the Lagrangian velocity
// accumulation of sgs_stag.f90:59-69 (uls, vls, wls: the scalar model's
// second sum, u_lag_s, when it is carried, else null)
__global__ void k_calc_sij(const double* __restrict__ dudx, const double* __restrict__ dudy,
                           const double* __restrict__ dudz, const double* __restrict__ dvdx,
                           const double* __restrict__ dvdy, const double* __restrict__ dvdz,
                           const double* __restrict__ dwdx, const double* __restrict__ dwdy,
                           const double* __restrict__ dwdz, double* S11, double* S12, double* S13,
                           double* S22, double* S23, double* S33, const double* __restrict__ u,
                           const double* __restrict__ v, const double* __restrict__ w, double* ul,
                           double* vl, double* wl, double* uls, double* vls, double* wls, int ld, int nx,
                           int ny, int nz, int lag) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * nz) {
    const int jz = (int)(i / np) + 1;
    const int jx = (int)((i - (size_t)(jz - 1) * np) % ld);
    if (lag) { ul[i] += u[i]; vl[i] += v[i]; wl[i] += w[i]; }
    if (uls) { uls[i] += u[i]; vls[i] += v[i]; wls[i] += w[i]; }
    if (jx >= nx) continue;
    double ux, uy, uz, vx, vy, vz, wx, wy, wz;
    if (jz == 1) {
      ux = dudx[i]; uy = dudy[i]; uz = dudz[i];
      vx = dvdx[i]; vy = dvdy[i]; vz = dvdz[i];
      wx = 0.5 * (dwdx[i] + dwdx[i + np]);
      wy = 0.5 * (dwdy[i] + dwdy[i + np]);
      wz = dwdz[i];
    } else {
      ux = 0.5 * (dudx[i] + dudx[i - np]);
      uy = 0.5 * (dudy[i] + dudy[i - np]);
      uz = dudz[i];
      vx = 0.5 * (dvdx[i] + dvdx[i - np]);
      vy = 0.5 * (dvdy[i] + dvdy[i - np]);
      vz = dvdz[i];
      wx = dwdx[i];
      wy = dwdy[i];
      wz = 0.5 * (dwdz[i] + dwdz[i - np]);
    }
    S11[i] = ux; S12[i] = 0.5 * (uy + vx); S13[i] = 0.5 * (uz + wx);
    S22[i] = vy; S23[i] = 0.5 * (vz + wy); S33[i] = wz;
  }
}

// Mixed form: the same strain in FP32 from the FP32-held horizontal
// gradients (FP32 transforms) and the FP64 vertical ones, stored in FP32;
// the Lagrangian accumulation of u, v, w stays FP64.  grid (ceil(np/256),
// nz): no 64-bit index division.
__global__ void __launch_bounds__(256) k_calc_sij32(
    const float* __restrict__ dudx, const float* __restrict__ dudy, const double* __restrict__ dudz,
    const float* __restrict__ dvdx, const float* __restrict__ dvdy, const double* __restrict__ dvdz,
    const float* __restrict__ dwdx, const float* __restrict__ dwdy, const double* __restrict__ dwdz, float* S11,
    float* S12, float* S13, float* S22, float* S23, float* S33, const double* __restrict__ u,
    const double* __restrict__ v, const double* __restrict__ w, double* ul, double* vl, double* wl, int ld, int nx,
    int ny, int lag) {
  const unsigned np = (unsigned)ld * ny;
  const unsigned p = blockIdx.x * 256u + threadIdx.x;
  if (p >= np) return;
  const int jz = blockIdx.y + 1;
  const size_t i = (size_t)(jz - 1) * np + p;
  if (lag) { ul[i] += u[i]; vl[i] += v[i]; wl[i] += w[i]; }
  if ((int)(p % (unsigned)ld) >= nx) return;
  float ux, uy, uz, vx, vy, vz, wx, wy, wz;
  if (jz == 1) {
    ux = dudx[i]; uy = dudy[i]; uz = cvt_d2f(dudz[i]);
    vx = dvdx[i]; vy = dvdy[i]; vz = cvt_d2f(dvdz[i]);
    wx = 0.5f * (dwdx[i] + dwdx[i + np]);
    wy = 0.5f * (dwdy[i] + dwdy[i + np]);
    wz = cvt_d2f(dwdz[i]);
  } else {
    ux = 0.5f * (dudx[i] + dudx[i - np]);
    uy = 0.5f * (dudy[i] + dudy[i - np]);
    uz = cvt_d2f(dudz[i]);
    vx = 0.5f * (dvdx[i] + dvdx[i - np]);
    vy = 0.5f * (dvdy[i] + dvdy[i - np]);
    vz = cvt_d2f(dvdz[i]);
    wx = dwdx[i];
    wy = dwdy[i];
    wz = 0.5f * (cvt_d2f(dwdz[i]) + cvt_d2f(dwdz[i - np]));
  }
  S11[i] = ux; S12[i] = 0.5f * (uy + vx); S13[i] = 0.5f * (uz + wx);
  S22[i] = vy; S23[i] = 0.5f * (vz + wy); S33[i] = wz;
}

__device__ __forceinline__ double smag(double a11, double a22, double a33, double a12, double a13, double a23) {
  return sqrt(2.0 * (a11 * a11 + a22 * a22 + a33 * a33 + 2.0 * (a12 * a12 + a13 * a13 + a23 * a23)));
}

// sgs_stag.f90:166-211 (Cs override and Nu_t)
__global__ void k_nut(const double* __restrict__ S11, const double* __restrict__ S12,
                      const double* __restrict__ S13, const double* __restrict__ S22,
                      const double* __restrict__ S23, const double* __restrict__ S33, double* Cs,
                      double* Nu_t, int ld, int nx, int ny, int nz, double l2, int override_cs, double cs_ov) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * nz) {
    if (override_cs) Cs[i] = cs_ov;
    const int jx = (int)(i % ld);
    if (jx >= nx) continue;
    const double S = smag(S11[i], S22[i], S33[i], S12[i], S13[i], S23[i]);
    Nu_t[i] = S * Cs[i] * l2;
  }
}
// sgs_stag.f90:218-364 (tau_ij, 'wall', molec = .false.)
__global__ void k_tau(const double* __restrict__ S11, const double* __restrict__ S12,
                      const double* __restrict__ S13, const double* __restrict__ S22,
                      const double* __restrict__ S23, const double* __restrict__ S33,
                      const double* __restrict__ Nu_t, double* txx, double* txy, double* tyy, double* txz,
                      double* tyz, double* tzz, int ld, int nx, int ny, int nz) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * nz) {
    const int jz = (int)(i / np) + 1;
    const int jx = (int)((i - (size_t)(jz - 1) * np) % ld);
    if (jz == nz) {
      txx[i] = LES_BOGUS; txy[i] = LES_BOGUS; tyy[i] = LES_BOGUS; tzz[i] = LES_BOGUS;
      txz[i] = 0.0; tyz[i] = 0.0;
      continue;
    }
    if (jx >= nx) continue;
    if (jz == 1) {
      const double cst = Nu_t[i], nu = 0.0;
      txx[i] = -2.0 * (cst + nu) * S11[i];
      txy[i] = -2.0 * (cst + nu) * S12[i];
      tyy[i] = -2.0 * (cst + nu) * S22[i];
      tzz[i] = -2.0 * (cst + nu) * S33[i];
      // txz, tyz at the wall come from wallstress
    } else {
      const size_t ip = i + np;
      const double cst = 0.5 * (Nu_t[i] + Nu_t[ip]), nu = 0.0;
      txx[i] = -2.0 * (cst + nu) * 0.5 * (S11[i] + S11[ip]);
      txy[i] = -2.0 * (cst + nu) * 0.5 * (S12[i] + S12[ip]);
      tyy[i] = -2.0 * (cst + nu) * 0.5 * (S22[i] + S22[ip]);
      tzz[i] = -2.0 * (cst + nu) * 0.5 * (S33[i] + S33[ip]);
      const double c2 = Nu_t[i];
      txz[i] = -2.0 * (c2 + nu) * S13[i];
      tyz[i] = -2.0 * (c2 + nu) * S23[i];
    }
  }
}

// Mixed form: the eddy viscosity (k_nut) and tau (k_tau) in one pass, FP32
// arithmetic on the FP32-held strain, Nu_t and tau stored in FP32.  The thread of level jz forms Nu_t at its own level (stored,
// as sgs_stag.f90:166-211) and again at level jz+1 for the staggered
// averages of tau (the strain of both levels is read anyway), so Nu_t is not
// re-read.  grid (ceil(np/256), nz).
__device__ __forceinline__ float nut32_at(const float* const* S, size_t i, float cs, float l2) {
  const float a11 = S[0][i], a12 = S[1][i], a13 = S[2][i];
  const float a22 = S[3][i], a23 = S[4][i], a33 = S[5][i];
  const float sm = sqrtf(2.0f * (a11 * a11 + a22 * a22 + a33 * a33 + 2.0f * (a12 * a12 + a13 * a13 + a23 * a23)));
  return sm * cs * l2;
}
struct Ptr6f { const float* p[6]; };
__global__ void __launch_bounds__(256) k_nut_tau32(Ptr6f Sp, double* Cs, float* Nu_t, float* txx, float* txy,
                                                   float* tyy, float* txz, float* tyz, float* tzz, int ld,
                                                   int nx, int ny, int nz, float l2, int override_cs, double cs_ov) {
  const unsigned np = (unsigned)ld * ny;
  const unsigned p = blockIdx.x * 256u + threadIdx.x;
  if (p >= np) return;
  const int jz = blockIdx.y + 1;
  const size_t i = (size_t)(jz - 1) * np + p;
  if (override_cs) Cs[i] = cs_ov;
  const bool inx = (int)(p % (unsigned)ld) < nx;
  const float csov = cvt_d2f(cs_ov);
  float nu = 0.0f;
  if (inx) {
    nu = nut32_at(Sp.p, i, override_cs ? csov : cvt_d2f(Cs[i]), l2);
    Nu_t[i] = nu;
  }
  if (jz == nz) {
    txx[i] = (float)LES_BOGUS; txy[i] = (float)LES_BOGUS; tyy[i] = (float)LES_BOGUS; tzz[i] = (float)LES_BOGUS;
    txz[i] = 0.0f; tyz[i] = 0.0f;
    return;
  }
  if (!inx) return;
  const float* const* S = Sp.p;
  if (jz == 1) {
    const float c = -2.0f * nu;
    txx[i] = c * S[0][i];
    txy[i] = c * S[1][i];
    tyy[i] = c * S[3][i];
    tzz[i] = c * S[5][i];
    // txz, tyz at the wall come from wallstress
  } else {
    const size_t ip = i + np;
    const float nup = nut32_at(S, ip, override_cs ? csov : cvt_d2f(Cs[ip]), l2);
    const float c = -2.0f * (0.5f * (nu + nup)) * 0.5f;
    txx[i] = c * (S[0][i] + S[0][ip]);
    txy[i] = c * (S[1][i] + S[1][ip]);
    tyy[i] = c * (S[3][i] + S[3][ip]);
    tzz[i] = c * (S[5][i] + S[5][ip]);
    txz[i] = -2.0f * nu * S[2][i];
    tyz[i] = -2.0f * nu * S[4][i];
  }
}

__global__ void k_bcast_levels(double* dst, const double* lev, size_t np, size_t n) {
  GSTRIDE(i, n) dst[i] = lev[i / np];
}

int op_sgs_stag(les_ctx* c) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  const bool lag = (k.model == 4 || k.model == 5 || k.model == 7);
  k_calc_sij<<<grid1(g.nfield), 256, 0, c->stream>>>(
      c->f[LES_DUDX], c->f[LES_DUDY], c->f[LES_DUDZ], c->f[LES_DVDX], c->f[LES_DVDY], c->f[LES_DVDZ],
      c->f[LES_DWDX], c->f[LES_DWDY], c->f[LES_DWDZ], c->f[LES_S11], c->f[LES_S12], c->f[LES_S13],
      c->f[LES_S22], c->f[LES_S23], c->f[LES_S33], c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[LES_U_LAG],
      c->f[LES_V_LAG], c->f[LES_W_LAG], c->f[LES_U_LAG_S], c->f[LES_V_LAG_S], c->f[LES_W_LAG_S], g.ld, g.nx, g.ny,
      g.nz, lag ? 1 : 0); LES_COUNT_LAUNCH();
  const double* S[6] = {c->f[LES_S11], c->f[LES_S12], c->f[LES_S13], c->f[LES_S22], c->f[LES_S23], c->f[LES_S33]};
  if ((c->jt >= 1 || k.initu) && (c->jt % k.cs_count == 0)) {  // sgs_stag.f90:120-160
    if (k.model == 2 || k.model == 3) {
      double* csz = c->dred;
      if (k.model == 2) op_stddyn(c, csz, S);
      else op_scaledep(c, csz, S);
      // Cs_opt2(:,:,jz) = ziko(jz)
      k_bcast_levels<<<grid1(g.nfield), 256, 0, c->stream>>>(c->f[LES_CS_OPT2], csz, g.nplane, g.nfield); LES_COUNT_LAUNCH();
    } else if (k.model == 4) {
      op_lagrange_ssim(c, S);
    } else if (k.model == 5) {
      op_lagrange(c, S);
    } else if (k.model == 7) {  // sgs_stag.f90:150-152
      op_lagrange(c, S);
      op_lagrange_scalar(c, S, nullptr);
    }
  }
  int ov = 0;
  double csov = 0.0;
  if ((k.model == 5 || k.model == 6 || k.model == 7) && c->jt_total < 500) {  // :166-173
    ov = 1;
    const float c016 = 0.16f;
    csov = (double)(c016 * c016);
    if (k.model == 7) fill(c, c->f[LES_PR_T], g.nfield, k.pr);  // Pr_t = Pr (:171)
  }
  const double delta = g.delta;
  k_nut<<<grid1(g.nfield), 256, 0, c->stream>>>(S[0], S[1], S[2], S[3], S[4], S[5], c->f[LES_CS_OPT2],
                                               c->f[LES_NU_T], g.ld, g.nx, g.ny, g.nz, delta * delta, ov, csov); LES_COUNT_LAUNCH();
  k_tau<<<grid1(g.nfield), 256, 0, c->stream>>>(S[0], S[1], S[2], S[3], S[4], S[5], c->f[LES_NU_T],
                                               c->f[LES_TXX], c->f[LES_TXY], c->f[LES_TYY], c->f[LES_TXZ],
                                               c->f[LES_TYZ], c->f[LES_TZZ], g.ld, g.nx, g.ny, g.nz); LES_COUNT_LAUNCH();
  return 0;
}

// ---------------------------------------------------------------------------
// interpolag_Sdep.f90:2-380 (non-MPI).  Reads the accumulated u/v/w_lag and
// the old F_*, writes the interpolated F_* into Fn.
__device__ __forceinline__ double lag_disp_u(const double* ul, size_t i, size_t np, int jz, double cs,
                                             double dt, double dxx) {
  const double a = ul[i] / cs;
  const double ua = (jz >= 2) ? 0.5 * (a + ul[i - np] / cs) : a;
  return -ua * dt * cs / dxx;
}
// NF: F_* fields carried (4: interpolag_Sdep, 2: interpolag_Ssim, which
// also lacks the near-wall clip of interpolag_Sdep.f90:290-293, so its level 1 keeps
// 0.25 w_lag(2), doubled when positive).
template <int NF, bool SDEP>
__global__ void k_interpolag(const double* __restrict__ ul, const double* __restrict__ vl,
                             const double* __restrict__ wl, const double* __restrict__ FLM,
                             const double* __restrict__ FMM, const double* __restrict__ FQN,
                             const double* __restrict__ FNN, double* oLM, double* oMM, double* oQN,
                             double* oNN, int ld, int nx, int ny, int nz, double cs, double dt, double dx,
                             double dy, double dz) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(t, (size_t)nx * ny * nz) {
    const int jx = (int)(t % nx);
    const int jy = (int)((t / nx) % ny);
    const int jz = (int)(t / ((size_t)nx * ny)) + 1;
    const size_t i = (size_t)jx + (size_t)ld * jy + np * (jz - 1);
    const double xp = lag_disp_u(ul, i, np, jz, cs, dt, dx);
    const double yp = lag_disp_u(vl, i, np, jz, cs, dt, dy);
    double zp;
    {
      // level 2 after the near-wall doubling and clipping (:285-293);
      // level 1 takes level 2's final value
      const size_t i2 = (size_t)jx + (size_t)ld * jy + np;
      if (SDEP && jz <= 2) {
        double z2 = -(wl[i2] / cs) * dt * cs / dz;
        z2 = z2 + fmin(z2, 0.0);
        z2 = fmin(1.0, z2);
        z2 = fmax(-1.0, z2);
        zp = z2;
      } else if (!SDEP && jz == 2) {
        const double z2 = -(wl[i2] / cs) * dt * cs / dz;
        zp = z2 + fmin(z2, 0.0);
      } else if (!SDEP && jz == 1) {
        const double z1 = -(0.25 * (wl[i2] / cs)) * dt * cs / dz;
        zp = z1 + fmax(z1, 0.0);
      } else {
        zp = -(wl[i] / cs) * dt * cs / dz;
      }
    }
    const int addx = (xp < 0.0) ? -1 : 1;  // int(sign(1,x)), sign(1,-0) = +1
    const int addy = (yp < 0.0) ? -1 : 1;
    const int addz = (zp < 0.0) ? -1 : 1;
    int xa = jx + addx; if (xa < 0) xa = nx - 1; if (xa >= nx) xa = 0;
    int ya = jy + addy; if (ya < 0) ya = ny - 1; if (ya >= ny) ya = 0;
    int za = (jz - 1) + addz; if (za < 0) za = 0; if (za >= nz) za = nz - 1;
    const double cx = fabs(xp), cy = fabs(yp), cz = fabs(zp);
    const double fx = 1.0 - cx, fy = 1.0 - cy, fz = 1.0 - cz;
    const size_t z0 = np * (jz - 1), z1 = np * za;
    const size_t a00 = (size_t)jx + (size_t)ld * jy, a01 = (size_t)jx + (size_t)ld * ya;
    const size_t a10 = (size_t)xa + (size_t)ld * jy, a11 = (size_t)xa + (size_t)ld * ya;
#define LAGI(F)                                                                      \
  (fx * fy * (F[a00 + z0] * fz + F[a00 + z1] * cz) + fx * cy * (F[a01 + z0] * fz + F[a01 + z1] * cz) + \
   cx * fy * (F[a10 + z0] * fz + F[a10 + z1] * cz) + cx * cy * (F[a11 + z0] * fz + F[a11 + z1] * cz))
    oLM[i] = LAGI(FLM);
    oMM[i] = LAGI(FMM);
    if constexpr (NF == 4) {
      oQN[i] = LAGI(FQN);
      oNN[i] = LAGI(FNN);
    }
#undef LAGI
  }
}
// Mixed form: the same back-trajectory interpolation in FP32, gathering from
// FP32 copies of F_LM, F_MM, F_QN, F_NN (the reference itself truncates
// F_LM and F_QN to FP32), results widened to the FP64 state.  The
// displacement -u_lag dt / dx is formed without the cs factor that the
// reference divides out and multiplies back (:260-262); u_lag is the sum
// over the cs_count steps, so the displacement is -u_lag dt / dx.
__global__ void k_to_f32x4(const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                           const double* __restrict__ d, float* o, size_t n) {
  GSTRIDE(i, n) {
    o[i] = cvt_d2f(a[i]);
    o[i + n] = cvt_d2f(b[i]);
    o[i + 2 * n] = cvt_d2f(c[i]);
    o[i + 3 * n] = cvt_d2f(d[i]);
  }
}
__global__ void k_interpolag32(const double* __restrict__ ul, const double* __restrict__ vl,
                               const double* __restrict__ wl, const float* __restrict__ F4, double* oLM,
                               double* oMM, double* oQN, double* oNN, int ld, int nx, int ny, int nz, size_t nf,
                               float sx, float sy, float sz) {
  const size_t np = (size_t)ld * ny;
  const float* FLM = F4;
  const float* FMM = F4 + nf;
  const float* FQN = F4 + 2 * nf;
  const float* FNN = F4 + 3 * nf;
  GSTRIDE(t, (size_t)nx * ny * nz) {
    const int jx = (int)(t % nx);
    const int jy = (int)((t / nx) % ny);
    const int jz = (int)(t / ((size_t)nx * ny)) + 1;
    const size_t i = (size_t)jx + (size_t)ld * jy + np * (jz - 1);
    float ua = cvt_d2f(ul[i]), va = cvt_d2f(vl[i]);
    if (jz >= 2) {
      ua = 0.5f * (ua + cvt_d2f(ul[i - np]));
      va = 0.5f * (va + cvt_d2f(vl[i - np]));
    }
    const float xp = -ua * sx, yp = -va * sy;
    float zp;
    {
      const size_t i2 = (size_t)jx + (size_t)ld * jy + np;
      if (jz <= 2) {
        float z2 = -cvt_d2f(wl[i2]) * sz;
        z2 = z2 + fminf(z2, 0.0f);
        z2 = fminf(1.0f, z2);
        z2 = fmaxf(-1.0f, z2);
        zp = z2;
      } else {
        zp = -cvt_d2f(wl[i]) * sz;
      }
    }
    const int addx = (xp < 0.0f) ? -1 : 1;
    const int addy = (yp < 0.0f) ? -1 : 1;
    const int addz = (zp < 0.0f) ? -1 : 1;
    int xa = jx + addx; if (xa < 0) xa = nx - 1; if (xa >= nx) xa = 0;
    int ya = jy + addy; if (ya < 0) ya = ny - 1; if (ya >= ny) ya = 0;
    int za = (jz - 1) + addz; if (za < 0) za = 0; if (za >= nz) za = nz - 1;
    const float cx = fabsf(xp), cy = fabsf(yp), cz = fabsf(zp);
    const float fx = 1.0f - cx, fy = 1.0f - cy, fz = 1.0f - cz;
    const size_t z0 = np * (jz - 1), z1 = np * za;
    const size_t a00 = (size_t)jx + (size_t)ld * jy, a01 = (size_t)jx + (size_t)ld * ya;
    const size_t a10 = (size_t)xa + (size_t)ld * jy, a11 = (size_t)xa + (size_t)ld * ya;
#define LAGI(F)                                                                      \
  (fx * fy * (F[a00 + z0] * fz + F[a00 + z1] * cz) + fx * cy * (F[a01 + z0] * fz + F[a01 + z1] * cz) + \
   cx * fy * (F[a10 + z0] * fz + F[a10 + z1] * cz) + cx * cy * (F[a11 + z0] * fz + F[a11 + z1] * cz))
    oLM[i] = cvt_f2d(LAGI(FLM));
    oMM[i] = cvt_f2d(LAGI(FMM));
    oQN[i] = cvt_f2d(LAGI(FQN));
    oNN[i] = cvt_f2d(LAGI(FNN));
#undef LAGI
  }
}
static int op_interpolag32(les_ctx* c) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  double* Fn[4];
  for (int q = 0; q < 4; ++q) Fn[q] = c->spare + (size_t)q * g.nfield;
  float* F4 = reinterpret_cast<float*>(c->tmp);  // 4 * nfield floats, free until the filtering below
  k_to_f32x4<<<grid1(g.nfield), 256, 0, c->stream>>>(c->f[LES_F_LM], c->f[LES_F_MM], c->f[LES_F_QN], c->f[LES_F_NN],
                                                     F4, g.nfield); LES_COUNT_LAUNCH();
  // u_lag holds the sum over cs_count steps: (sum / cs_count) * (dt * cs_count) / dx
  k_interpolag32<<<grid1((size_t)g.nx * g.ny * g.nz), 256, 0, c->stream>>>(
      c->f[LES_U_LAG], c->f[LES_V_LAG], c->f[LES_W_LAG], F4, Fn[0], Fn[1], Fn[2], Fn[3], g.ld, g.nx, g.ny, g.nz,
      g.nfield, (float)(k.dt / g.dx), (float)(k.dt / g.dy), (float)(k.dt / g.dz)); LES_COUNT_LAUNCH();
  for (int q = 0; q < 4; ++q)
    cudaMemcpyAsync(c->f[LES_F_LM + q], Fn[q], g.nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  cudaMemsetAsync(c->f[LES_U_LAG], 0, g.nfield * sizeof(double), c->stream);
  cudaMemsetAsync(c->f[LES_V_LAG], 0, g.nfield * sizeof(double), c->stream);
  cudaMemsetAsync(c->f[LES_W_LAG], 0, g.nfield * sizeof(double), c->stream);
  return 0;
}
int op_interpolag(les_ctx* c) { return op_interpolag_n(c, 4); }
// nf = 4: interpolag_Sdep.f90:2-380; nf = 2: interpolag_Ssim.f90:3-316
int op_interpolag_n(les_ctx* c, int nf) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  double* Fn[4];
  for (int q = 0; q < 4; ++q) Fn[q] = c->spare + (size_t)q * g.nfield;
  if (nf == 4)
    k_interpolag<4, true><<<grid1((size_t)g.nx * g.ny * g.nz), 256, 0, c->stream>>>(
        c->f[LES_U_LAG], c->f[LES_V_LAG], c->f[LES_W_LAG], c->f[LES_F_LM], c->f[LES_F_MM], c->f[LES_F_QN],
        c->f[LES_F_NN], Fn[0], Fn[1], Fn[2], Fn[3], g.ld, g.nx, g.ny, g.nz, (double)k.cs_count, k.dt, g.dx, g.dy,
        g.dz);
  else
    k_interpolag<2, false><<<grid1((size_t)g.nx * g.ny * g.nz), 256, 0, c->stream>>>(
        c->f[LES_U_LAG], c->f[LES_V_LAG], c->f[LES_W_LAG], c->f[LES_F_LM], c->f[LES_F_MM], nullptr, nullptr,
        Fn[0], Fn[1], nullptr, nullptr, g.ld, g.nx, g.ny, g.nz, (double)k.cs_count, k.dt, g.dx, g.dy, g.dz);
  LES_COUNT_LAUNCH();
  // interior values changed; padding columns are never read
  for (int q = 0; q < nf; ++q)
    cudaMemcpyAsync(c->f[LES_F_LM + q], Fn[q], g.nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  cudaMemsetAsync(c->f[LES_U_LAG], 0, g.nfield * sizeof(double), c->stream);
  cudaMemsetAsync(c->f[LES_V_LAG], 0, g.nfield * sizeof(double), c->stream);
  cudaMemsetAsync(c->f[LES_W_LAG], 0, g.nfield * sizeof(double), c->stream);
  return 0;
}

// lagrange_Sdep.f90:127-285 inputs: 21 planes per level of the chunk
__global__ void k_lag_prep(const double* __restrict__ u, const double* __restrict__ v,
                           const double* __restrict__ w, Ptr6 Sp,
                           double* out, int ld, int nx, int ny, int jz0, int nlev, size_t np) {
  const size_t tot = np * nlev;
  GSTRIDE(t, tot) {
    const int lc = (int)(t / np);
    const size_t r = t - (size_t)lc * np;
    const int jz = jz0 + lc;  // 1-based
    const size_t i = (size_t)(jz - 1) * np + r;
    double ub, vb, wb;
    if (jz == 1) { ub = u[i]; vb = v[i]; wb = 0.25 * w[i + np]; }
    else { ub = 0.5 * (u[i] + u[i - np]); vb = 0.5 * (v[i] + v[i - np]); wb = w[i]; }
    const size_t stride = np * nlev;
    double* o = out + t;
    o[0 * stride] = ub; o[1 * stride] = vb; o[2 * stride] = wb;
    o[3 * stride] = ub * ub; o[4 * stride] = ub * vb; o[5 * stride] = ub * wb;
    o[6 * stride] = vb * vb; o[7 * stride] = vb * wb; o[8 * stride] = wb * wb;
    const double s11 = Sp.p[0][i], s12 = Sp.p[1][i], s13 = Sp.p[2][i], s22 = Sp.p[3][i], s23 = Sp.p[4][i], s33 = Sp.p[5][i];
    const double S = smag(s11, s22, s33, s12, s13, s23);
    o[9 * stride] = s11; o[10 * stride] = s12; o[11 * stride] = s13;
    o[12 * stride] = s22; o[13 * stride] = s23; o[14 * stride] = s33;
    o[15 * stride] = S * s11; o[16 * stride] = S * s12; o[17 * stride] = S * s13;
    o[18 * stride] = S * s22; o[19 * stride] = S * s23; o[20 * stride] = S * s33;
  }
}

__device__ __forceinline__ double pow_m18(double x) { return 1.0 / sqrt(sqrt(sqrt(x))); }
__device__ __forceinline__ float pow_m18(float x) { return 1.0f / sqrtf(sqrtf(sqrtf(x))); }
// max(real(a), real(b)) of the reference: FP32 comparison, result widened
__device__ __forceinline__ double fmax32r(double a, double b) { return fmax32(a, b); }
__device__ __forceinline__ float fmax32r(float a, float b) { return a > b ? a : b; }
template <typename R>
__device__ __forceinline__ R smagR(R a11, R a22, R a33, R a12, R a13, R a23) {
  return sqrt((R)2 * (a11 * a11 + a22 * a22 + a33 * a33 + (R)2 * (a12 * a12 + a13 * a13 + a23 * a23)));
}

// lagrange_Sdep.f90:268-421 from the 42 filtered planes (G: q, GG: 21+q).
// S: storage of the filtered planes; R: arithmetic (double in the FP64
// form; float in the mixed form, where the planes are FP32 and the
// reference truncates F_LM, F_QN and Cs^2 to FP32 itself).  The module
// arrays stay FP64.
template <typename S, typename R>
__global__ void k_lag_final(const S* __restrict__ flt, double* F_LM, double* F_MM, double* F_QN,
                            double* F_NN, double* Beta, double* Cs, double* TnLM, double* TnQN, int ld, int nx,
                            int ny, int nz, int jz0, int nlev, size_t np, R cst, R opftdelta, R lagran_dt,
                            int bexp_one, R bexp) {
  const size_t tot = np * nlev;
  GSTRIDE(t, tot) {
    const int lc = (int)(t / np);
    const size_t r = t - (size_t)lc * np;
    const int jx = (int)(r % ld);
    const int jz = jz0 + lc;
    const size_t gi = (size_t)(jz - 1) * np + r;
    if (jx >= nx) { Cs[gi] = (double)1e-24f; continue; }
    const size_t st = np * nlev;
    const S* G = flt + t;
    const S* H = flt + t + 21 * st;
    const R ub = G[0], vb = G[st], wb = G[2 * st];
    const R uh = H[0], vh = H[st], wh = H[2 * st];
    const R Lq[6] = {(R)G[3 * st] - ub * ub, (R)G[4 * st] - ub * vb, (R)G[5 * st] - ub * wb,
                     (R)G[6 * st] - vb * vb, (R)G[7 * st] - vb * wb, (R)G[8 * st] - wb * wb};
    const R Qq[6] = {(R)H[3 * st] - uh * uh, (R)H[4 * st] - uh * vh, (R)H[5 * st] - uh * wh,
                     (R)H[6 * st] - vh * vh, (R)H[7 * st] - vh * wh, (R)H[8 * st] - wh * wh};
    R Sb_[6], Sh_[6], SSb[6], SSh[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      Sb_[q] = G[(9 + q) * st]; Sh_[q] = H[(9 + q) * st];
      SSb[q] = G[(15 + q) * st]; SSh[q] = H[(15 + q) * st];
    }
    const R Sb = smagR<R>(Sb_[0], Sb_[3], Sb_[5], Sb_[1], Sb_[2], Sb_[4]);
    const R Sh = smagR<R>(Sh_[0], Sh_[3], Sh_[5], Sh_[1], Sh_[2], Sh_[4]);
    R M[6], N[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      M[q] = cst * (SSb[q] - (R)4 * Sb * Sb_[q]);
      N[q] = cst * (SSh[q] - (R)16 * Sh * Sh_[q]);
    }
    const R LM = Lq[0] * M[0] + Lq[3] * M[3] + Lq[5] * M[5] + (R)2 * (Lq[1] * M[1] + Lq[2] * M[2] + Lq[4] * M[4]);
    const R MM = M[0] * M[0] + M[3] * M[3] + M[5] * M[5] + (R)2 * (M[1] * M[1] + M[2] * M[2] + M[4] * M[4]);
    const R QN = Qq[0] * N[0] + Qq[3] * N[3] + Qq[5] * N[5] + (R)2 * (Qq[1] * N[1] + Qq[2] * N[2] + Qq[4] * N[4]);
    const R NN = N[0] * N[0] + N[3] * N[3] + N[5] * N[5] + (R)2 * (N[1] * N[1] + N[2] * N[2] + N[4] * N[4]);
    const R e24 = (R)1e-24f;
    R flm = (R)F_LM[gi], fmm = (R)F_MM[gi];
    R Tn = fmax32r(flm * fmm, e24);
    if (TnLM) TnLM[gi] = (double)Tn;  // lagrange_Sdep.f90:322, read by lagrange_scalar_Sdep
    Tn = opftdelta * pow_m18(Tn);
    Tn = fmax32r(e24, Tn);
    R dumfac = lagran_dt / Tn;
    R epsi = dumfac / ((R)1 + dumfac);
    flm = (epsi * LM + ((R)1 - epsi) * flm);
    fmm = (epsi * MM + ((R)1 - epsi) * fmm);
    flm = fmax32r(e24, flm);
    R cs2d = fmax32r(e24, flm / fmm);
    F_LM[gi] = flm; F_MM[gi] = fmm;
    R fqn = (R)F_QN[gi], fnn = (R)F_NN[gi];
    Tn = fmax32r(fqn * fnn, e24);
    if (TnQN) TnQN[gi] = (double)Tn;  // :363
    Tn = opftdelta * pow_m18(Tn);
    Tn = fmax32r(e24, Tn);
    dumfac = lagran_dt / Tn;
    epsi = dumfac / ((R)1 + dumfac);
    fqn = (epsi * QN + ((R)1 - epsi) * fqn);
    fnn = (epsi * NN + ((R)1 - epsi) * fnn);
    fqn = fmax32r(e24, fqn);
    R cs4d = fmax32r(e24, fqn / fnn);
    F_QN[gi] = fqn; F_NN[gi] = fnn;
    R beta = bexp_one ? cs4d / cs2d : pow(cs4d / cs2d, bexp);
    if (jz == nz) beta = (R)1;
    Beta[gi] = beta;
    const R betaclip = fmax32r(beta, (R)1 / ((R)2 * (R)4));
    Cs[gi] = fmax32r(e24, cs2d / betaclip);
  }
}

// lagrange_Sdep.f90:4-478 ; S = S11,S12,S13,S22,S23,S33 (device)
int op_lagrange(les_ctx* c, const double* const* S) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  op_interpolag(c);
  const double delta = g.delta;
  const double cst = 2.0 * (delta * delta);
  const double opftdelta = 1.5 * delta;
  const double lagran_dt = k.dt * (double)k.cs_count;
  const double bexp = std::log(2.0) / (std::log(4.0) - std::log(2.0));
  const int bone = (bexp == 1.0) ? 1 : 0;
  Ptr6 Sp;
  for (int q = 0; q < 6; ++q) Sp.p[q] = S[q];
  const int nch = c->lag_chunk;
  for (int jz0 = 1; jz0 <= g.nz; jz0 += nch) {
    const int nl = std::min(nch, g.nz - jz0 + 1);
    double* prep = c->tmp;                              // 21 * nl planes
    double* flt = c->tmp + (size_t)21 * nch * g.nplane;  // 42 * nl planes
    k_lag_prep<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W],
                                                           Sp, prep, g.ld, g.nx,
                                                           g.ny, jz0, nl, g.nplane); LES_COUNT_LAUNCH();
    const double* in[21];
    for (int q = 0; q < 21; ++q) in[q] = prep + (size_t)q * nl * g.nplane;
    r2c(c, 21, nl, in, (long)g.nplane, nullptr, nullptr, c->wsA, false, g.lh);
    ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nl);
    J.nin = 1; J.nout = 2; J.nf = 21;
    J.in[0] = c->wsA; J.fs_in = (long)nl * g.C;
    J.out[0] = c->wsB; J.out[1] = (C2*)c->wsB + (size_t)21 * nl * g.C; J.fs_out = (long)nl * g.C;
    J.coef[0][0] = CC_G; J.coef[1][0] = CC_GG;
    cols(c, J);
    double* out[42];
    for (int q = 0; q < 42; ++q) out[q] = flt + (size_t)q * nl * g.nplane;
    c2r(c, 42, nl, c->wsB, out, (long)g.nplane, false, g.lh);
    k_lag_final<double, double><<<grid1(g.nplane * nl), 256, 0, c->stream>>>(
        flt, c->f[LES_F_LM], c->f[LES_F_MM], c->f[LES_F_QN], c->f[LES_F_NN], c->f[LES_BETA],
        c->f[LES_CS_OPT2], c->f[LES_TN_LMMM], c->f[LES_TN_QNNN], g.ld, g.nx, g.ny, g.nz, jz0, nl, g.nplane, cst,
        opftdelta, lagran_dt, bone, bexp); LES_COUNT_LAUNCH();
  }
  // the level loop's pointer table must outlive the launches
  return 0;
}

// ---------------------------------------------------------------------------
// Model 7: the scalar's Lagrangian scale-dependent SGS Prandtl number.
// interpolag_scalar_Sdep.f90:1-227: interpolag_Sdep's back-trajectory
// interpolation applied to G_LM, G_MM, G_QN, G_NN along u_lag_s, v_lag_s,
// w_lag_s, which it then resets.
int op_interpolag_scalar(les_ctx* c) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  if (!c->f[LES_G_LM]) return LES_ERR_STATE;
  double* Fn[4];
  for (int q = 0; q < 4; ++q) Fn[q] = c->spare + (size_t)q * g.nfield;
  k_interpolag<4, true><<<grid1((size_t)g.nx * g.ny * g.nz), 256, 0, c->stream>>>(
      c->f[LES_U_LAG_S], c->f[LES_V_LAG_S], c->f[LES_W_LAG_S], c->f[LES_G_LM], c->f[LES_G_MM], c->f[LES_G_QN],
      c->f[LES_G_NN], Fn[0], Fn[1], Fn[2], Fn[3], g.ld, g.nx, g.ny, g.nz, (double)k.cs_count, k.dt, g.dx, g.dy,
      g.dz); LES_COUNT_LAUNCH();
  for (int q = 0; q < 4; ++q)
    cudaMemcpyAsync(c->f[LES_G_LM + q], Fn[q], g.nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  cudaMemsetAsync(c->f[LES_U_LAG_S], 0, g.nfield * sizeof(double), c->stream);
  cudaMemsetAsync(c->f[LES_V_LAG_S], 0, g.nfield * sizeof(double), c->stream);
  cudaMemsetAsync(c->f[LES_W_LAG_S], 0, g.nfield * sizeof(double), c->stream);
  return 0;
}

// lagrange_scalar_Sdep.f90:96-131 (lbc = 1): the homogeneous surface flux
// and the plane-mean u* of the log law give dTdz at z = dz/2.  One CTA: the
// four plane sums, then the first level.
__global__ void __launch_bounds__(1024) k_lag_s_surface(const double* __restrict__ u, const double* __restrict__ v,
                                                        const double* __restrict__ zo,
                                                        const double* __restrict__ wt_s,
                                                        const double* __restrict__ psi_m,
                                                        const double* __restrict__ phi_h, double* dTdz, int nx,
                                                        int ny, int ld, double dz, double vonk, double t_scale,
                                                        double u_star) {
  __shared__ double red[4][32];
  const int ns = nx * ny;
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (int s = threadIdx.x; s < ns; s += blockDim.x) {
    const int jy = s / nx, jx = s - jy * nx;
    const size_t i = (size_t)jy * ld + jx;
    a[0] += log(zo[s]);
    a[1] += wt_s[s];
    a[2] += sqrt(u[i] * u[i] + v[i] * v[i]);
    a[3] += psi_m[s];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    for (int o = 16; o > 0; o >>= 1) a[q] += __shfl_down_sync(0xffffffffu, a[q], o);
    if (lane == 0) red[q][wid] = a[q];
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      a[q] = lane < nw ? red[q][lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) a[q] += __shfl_down_sync(0xffffffffu, a[q], o);
    }
    if (lane == 0) {
      red[0][0] = a[0]; red[1][0] = a[1]; red[2][0] = a[2]; red[3][0] = a[3];
    }
  }
  __syncthreads();
  const double nf = (double)(float)ns;  // float(nx*ny)
  const double zo_avg = exp(red[0][0] / nf);
  const double ustar_ = red[2][0] / nf * vonk / (log(0.5 * dz / zo_avg) - red[3][0] / nf);
  const double sflux = (red[1][0] / (double)ns) / t_scale / u_star;
  for (int s = threadIdx.x; s < ns; s += blockDim.x) {
    const int jy = s / nx, jx = s - jy * nx;
    dTdz[(size_t)jy * ld + jx] = -phi_h[s] * sflux / (ustar_ * vonk * dz / 2.0);
  }
}

// lagrange_scalar_Sdep.f90:140-262 inputs: 19 planes per level of the chunk
// (u, v, w, theta on the w-node; their products with theta; S_ij; |S| dT/dx_i
// and dT/dx_i on the w-node), each filtered at 2 delta and at 4 delta
__global__ void k_lag_s_prep(const double* __restrict__ u, const double* __restrict__ v,
                             const double* __restrict__ w, const double* __restrict__ th, Ptr6 Sp,
                             const double* __restrict__ dTx, const double* __restrict__ dTy,
                             const double* __restrict__ dTz, double* out, int jz0, int nlev, size_t np) {
  const size_t tot = np * nlev;
  GSTRIDE(t, tot) {
    const int lc = (int)(t / np);
    const size_t r = t - (size_t)lc * np;
    const int jz = jz0 + lc;
    const size_t i = (size_t)(jz - 1) * np + r;
    const double s11 = Sp.p[0][i], s12 = Sp.p[1][i], s13 = Sp.p[2][i], s22 = Sp.p[3][i], s23 = Sp.p[4][i],
                 s33 = Sp.p[5][i];
    const double S = smag(s11, s22, s33, s12, s13, s23);
    double ub, vb, wb, tb, gx, gy, gz, sx, sy, sz;
    if (jz == 1) {  // :140-145, :227-235, :253-262
      ub = u[i]; vb = v[i]; wb = 0.25 * w[i + np]; tb = th[i];
      sx = S * dTx[i];
      sy = S * dTy[i];
      sz = S * (dTz[i] + dTz[i + np]) / 2.0;
      gx = dTx[i]; gy = dTy[i]; gz = (dTz[i] + dTz[i + np]) / 2.0;
    } else {
      ub = 0.5 * (u[i] + u[i - np]); vb = 0.5 * (v[i] + v[i - np]); wb = w[i];
      tb = 0.5 * (th[i] + th[i - np]);
      sx = S * (dTx[i] + dTx[i - np]) / 2.0;
      sy = S * (dTy[i] + dTy[i - np]) / 2.0;
      sz = S * dTz[i];
      gx = (dTx[i] + dTx[i - np]) / 2.0; gy = (dTy[i] + dTy[i - np]) / 2.0; gz = dTz[i];
    }
    double* o = out + t;
    const size_t st = np * nlev;
    o[0] = ub; o[st] = vb; o[2 * st] = wb; o[3 * st] = tb;
    o[4 * st] = ub * tb; o[5 * st] = vb * tb; o[6 * st] = wb * tb;
    o[7 * st] = s11; o[8 * st] = s12; o[9 * st] = s13; o[10 * st] = s22; o[11 * st] = s23; o[12 * st] = s33;
    o[13 * st] = sx; o[14 * st] = sy; o[15 * st] = sz;
    o[16 * st] = gx; o[17 * st] = gy; o[18 * st] = gz;
  }
}

// lagrange_scalar_Sdep.f90:166-390 from the 38 filtered planes (G_test: q,
// G_test_test: 19 + q): L_i = bar(u_i T) - bar u_i bar T, Q_i at 4 delta,
// M_i, N_i, the relaxed G_*, Cs2_Pr at 2 and 4 delta, Beta, Cs2_Pr, Pr_t
__global__ void k_lag_s_final(const double* __restrict__ flt, double* G_LM, double* G_MM, double* G_QN, double* G_NN,
                              const double* __restrict__ TnLM, const double* __restrict__ TnQN,
                              const double* __restrict__ Cs, double* Beta, double* Pr_t, double* cs2_pr, int ld,
                              int nx, int nz, int jz0, int nlev, size_t np, double cst, double opftdelta,
                              double lagran_dt, int bexp_one, double bexp) {
  const size_t tot = np * nlev;
  const double e24 = (double)1e-24f;
  GSTRIDE(t, tot) {
    const int lc = (int)(t / np);
    const size_t r = t - (size_t)lc * np;
    const int jx = (int)(r % ld);
    const int jz = jz0 + lc;
    const size_t gi = (size_t)(jz - 1) * np + r;
    if (jx >= nx) {  // padding: Cs2_Pr = Cs_opt2 = 1e-24 (:334-336, :384-386)
      Pr_t[gi] = 1.0;
      if (cs2_pr) cs2_pr[gi] = e24;
      continue;
    }
    const size_t st = np * nlev;
    const double* G = flt + t;
    const double* H = flt + t + 19 * st;
    double L[3], Q[3], M[3], N[3];
    const double Sb = smag(G[7 * st], G[10 * st], G[12 * st], G[8 * st], G[9 * st], G[11 * st]);
    const double Sh = smag(H[7 * st], H[10 * st], H[12 * st], H[8 * st], H[9 * st], H[11 * st]);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      L[q] = G[(4 + q) * st] - G[q * st] * G[3 * st];
      Q[q] = H[(4 + q) * st] - H[q * st] * H[3 * st];
      M[q] = cst * (G[(13 + q) * st] - 4.0 * Sb * G[(16 + q) * st]);
      N[q] = cst * (H[(13 + q) * st] - 16.0 * Sh * H[(16 + q) * st]);
    }
    const double LM = L[0] * M[0] + L[1] * M[1] + L[2] * M[2];
    const double MM = M[0] * M[0] + M[1] * M[1] + M[2] * M[2];
    const double QN = Q[0] * N[0] + Q[1] * N[1] + Q[2] * N[2];
    const double NN = N[0] * N[0] + N[1] * N[1] + N[2] * N[2];
    double Tn = opftdelta * pow_m18(TnLM[gi]);
    Tn = fmax32(e24, Tn);
    double dumfac = lagran_dt / Tn;
    double epsi = dumfac / (1.0 + dumfac);
    double glm = (epsi * LM + (1.0 - epsi) * G_LM[gi]);
    const double gmm = (epsi * MM + (1.0 - epsi) * G_MM[gi]);
    glm = fmax32(e24, glm);
    const double c2 = fmax32(e24, glm / gmm);
    G_LM[gi] = glm; G_MM[gi] = gmm;
    Tn = opftdelta * pow_m18(TnQN[gi]);
    Tn = fmax32(e24, Tn);
    dumfac = lagran_dt / Tn;
    epsi = dumfac / (1.0 + dumfac);
    double gqn = (epsi * QN + (1.0 - epsi) * G_QN[gi]);
    const double gnn = (epsi * NN + (1.0 - epsi) * G_NN[gi]);
    gqn = fmax32(e24, gqn);
    const double c4 = fmax32(e24, gqn / gnn);
    G_QN[gi] = gqn; G_NN[gi] = gnn;
    double beta = bexp_one ? c4 / c2 : pow(c4 / c2, bexp);
    if (jz == nz) beta = 1.0;
    Beta[gi] = beta;
    const double betaclip = fmax32(beta, 1.0 / (2.0 * 4.0));
    const double cp = fmax32(e24, c2 / betaclip);
    if (cs2_pr) cs2_pr[gi] = cp;
    Pr_t[gi] = Cs[gi] / cp;  // :390
  }
}

// lagrange_scalar_Sdep.f90:1-467 (inilag = .false., inflow = .false.,
// lbc = 1); S = S11..S33 (device).  theta is Nyquist-filtered in place
// (filt_da, :83) as in the reference; cs2_pr may be null.
int op_lagrange_scalar(les_ctx* c, const double* const* S, double* cs2_pr) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  if (!c->f[LES_G_LM]) return LES_ERR_STATE;
  op_interpolag_scalar(c);  // :76 (reads nothing the copies below change)
  double* th0 = c->spare;  // theta_temp (:74): theta before the filter
  double* dTx = c->spare + g.nfield;
  double* dTy = c->spare + 2 * g.nfield;
  double* dTz = c->spare + 3 * g.nfield;
  double* theta = c->f[LES_THETA];
  cudaMemcpyAsync(th0, theta, g.nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  op_filt_da(c, theta, dTx, dTy, g.nz);  // :83-84
  op_ddz(c, dTz, theta, 1);
  fill(c, dTz + (size_t)(g.nz - 1) * g.nplane, g.nplane, k.dtdz_top / k.t_scale * k.z_i);  // :86
  k_lag_s_surface<<<1, 1024, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_ZO], c->f[LES_WT_S],
                                             c->f[LES_PSI_M], c->f[LES_PHI_H], dTz, g.nx, g.ny, g.ld, g.dz, k.vonk,
                                             k.t_scale, k.u_star); LES_COUNT_LAUNCH();
  const double delta = g.delta;
  const double cst = delta * delta;  // :81
  const double opftdelta = 1.5 * delta;
  const double lagran_dt = k.dt * (double)k.cs_count;
  const double bexp = std::log(2.0) / (std::log(4.0) - std::log(2.0));
  const int bone = (bexp == 1.0) ? 1 : 0;
  Ptr6 Sp;
  for (int q = 0; q < 6; ++q) Sp.p[q] = S[q];
  const int nch = c->lag_chunk;
  for (int jz0 = 1; jz0 <= g.nz; jz0 += nch) {
    const int nl = std::min(nch, g.nz - jz0 + 1);
    double* prep = c->tmp;                               // 19 * nl planes
    double* flt = c->tmp + (size_t)19 * nch * g.nplane;  // 38 * nl planes
    k_lag_s_prep<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W], th0, Sp, dTx,
                                                             dTy, dTz, prep, jz0, nl, g.nplane); LES_COUNT_LAUNCH();
    const double* in[19];
    for (int q = 0; q < 19; ++q) in[q] = prep + (size_t)q * nl * g.nplane;
    r2c(c, 19, nl, in, (long)g.nplane, nullptr, nullptr, c->wsA, false, g.lh);
    ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nl);
    J.nin = 1; J.nout = 2; J.nf = 19;
    J.in[0] = c->wsA; J.fs_in = (long)nl * g.C;
    J.out[0] = c->wsB; J.out[1] = (C2*)c->wsB + (size_t)19 * nl * g.C; J.fs_out = (long)nl * g.C;
    J.coef[0][0] = CC_G; J.coef[1][0] = CC_GG;
    cols(c, J);
    double* out[38];
    for (int q = 0; q < 38; ++q) out[q] = flt + (size_t)q * nl * g.nplane;
    c2r(c, 38, nl, c->wsB, out, (long)g.nplane, false, g.lh);
    k_lag_s_final<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(
        flt, c->f[LES_G_LM], c->f[LES_G_MM], c->f[LES_G_QN], c->f[LES_G_NN], c->f[LES_TN_LMMM], c->f[LES_TN_QNNN],
        c->f[LES_CS_OPT2], c->f[LES_BETA], c->f[LES_PR_T], cs2_pr, g.ld, g.nx, g.nz, jz0, nl, g.nplane, cst,
        opftdelta, lagran_dt, bone, bexp); LES_COUNT_LAUNCH();
  }
  return 0;
}

// scaledep_dynamic.f90:4-255 (plane sums over 1:nx) -> cs_z (device, nz)
__global__ void k_sd_prep(const double* __restrict__ u, const double* __restrict__ v,
                          const double* __restrict__ w, Ptr6 Sp, double* out,
                          int ld, int nx, int ny, int jz0, int nlev, size_t np) {
  const size_t tot = np * nlev;
  GSTRIDE(t, tot) {
    const int lc = (int)(t / np);
    const size_t r = t - (size_t)lc * np;
    const int jz = jz0 + lc;
    const size_t i = (size_t)(jz - 1) * np + r;
    double ub, vb, wb, L11, L12, L13, L22, L23, L33;
    if (jz == 1) {
      ub = u[i]; vb = v[i]; wb = 0.25 * w[i + np];
      L11 = u[i] * u[i]; L12 = u[i] * v[i]; L13 = u[i] * 0.25 * w[i + np];
      L22 = v[i] * v[i]; L23 = v[i] * 0.25 * w[i + np];
      const double tt = 0.25 * w[i + np]; L33 = tt * tt;
    } else {
      ub = 0.5 * (u[i] + u[i - np]); vb = 0.5 * (v[i] + v[i - np]); wb = w[i];
      L11 = 0.5 * (u[i] + u[i - np]) * 0.5 * (u[i] + u[i - np]);
      L12 = 0.5 * (u[i] + u[i - np]) * 0.5 * (v[i] + v[i - np]);
      L13 = 0.5 * (u[i] + u[i - np]) * w[i];
      L22 = 0.5 * (v[i] + v[i - np]) * 0.5 * (v[i] + v[i - np]);
      L23 = 0.5 * (v[i] + v[i - np]) * w[i];
      L33 = w[i] * w[i];
    }
    const size_t stride = np * nlev;
    double* o = out + t;
    o[0] = ub; o[stride] = vb; o[2 * stride] = wb;
    o[3 * stride] = L11; o[4 * stride] = L12; o[5 * stride] = L13;
    o[6 * stride] = L22; o[7 * stride] = L23; o[8 * stride] = L33;
    const double s11 = Sp.p[0][i], s12 = Sp.p[1][i], s13 = Sp.p[2][i], s22 = Sp.p[3][i], s23 = Sp.p[4][i], s33 = Sp.p[5][i];
    const double S = smag(s11, s22, s33, s12, s13, s23);
    o[9 * stride] = s11; o[10 * stride] = s12; o[11 * stride] = s13;
    o[12 * stride] = s22; o[13 * stride] = s23; o[14 * stride] = s33;
    o[15 * stride] = S * s11; o[16 * stride] = S * s12; o[17 * stride] = S * s13;
    o[18 * stride] = S * s22; o[19 * stride] = S * s23; o[20 * stride] = S * s33;
  }
}
// Second filtered set: Q_ij inputs are products of the G-filtered velocities.
__global__ void k_sd_qprep(const double* __restrict__ flt, double* qin, int nlev, size_t np) {
  const size_t st = np * nlev;
  GSTRIDE(t, st) {
    const double ub = flt[t], vb = flt[t + st], wb = flt[t + 2 * st];
    qin[t] = ub * ub; qin[t + st] = ub * vb; qin[t + 2 * st] = ub * wb;
    qin[t + 3 * st] = vb * vb; qin[t + 4 * st] = vb * wb; qin[t + 5 * st] = wb * wb;
  }
}
// per-level sums a1..e2 (10 sums) -> sums[lev*10 + q]; one CTA per level, fixed order
__global__ void __launch_bounds__(256) k_sd_sums(const double* __restrict__ flt, const double* __restrict__ qf,
                                                 double* sums, int ld, int nx, int ny, int nlev, size_t np, int jz0) {
  __shared__ double sh[10][256];
  const int lc = blockIdx.x;
  const size_t st = np * nlev;
  double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int e = threadIdx.x; e < nx * ny; e += blockDim.x) {
    const int jy = e / nx, jx = e - jy * nx;
    const size_t t = (size_t)lc * np + (size_t)jy * ld + jx;
    // G outputs q (0..20), GG outputs 21+q ; Q from qf (6 planes GG-filtered)
    const double* G = flt + t;
    const double* H = flt + t + 21 * st;
    const double ub = G[0], vb = G[st], wb = G[2 * st];
    const double uh = H[0], vh = H[st], wh = H[2 * st];
    const double L[6] = {G[3 * st] - ub * ub, G[4 * st] - ub * vb, G[5 * st] - ub * wb,
                         G[6 * st] - vb * vb, G[7 * st] - vb * wb, G[8 * st] - wb * wb};
    const double Q[6] = {qf[t] - uh * uh, qf[t + st] - uh * vh, qf[t + 2 * st] - uh * wh,
                         qf[t + 3 * st] - vh * vh, qf[t + 4 * st] - vh * wh, qf[t + 5 * st] - wh * wh};
    double b[6], h[6], sb[6], sh_[6];
    for (int q = 0; q < 6; ++q) { b[q] = G[(9 + q) * st]; h[q] = H[(9 + q) * st]; sb[q] = G[(15 + q) * st]; sh_[q] = H[(15 + q) * st]; }
    const double Sb = smag(b[0], b[3], b[5], b[1], b[2], b[4]);
    const double Sh = smag(h[0], h[3], h[5], h[1], h[2], h[4]);
    acc[0] += Sb * (b[0] * L[0] + b[3] * L[3] + b[5] * L[5] + 2.0 * (b[1] * L[1] + b[2] * L[2] + b[4] * L[4]));
    acc[1] += sb[0] * L[0] + sb[3] * L[3] + sb[5] * L[5] + 2.0 * (sb[1] * L[1] + sb[2] * L[2] + sb[4] * L[4]);
    acc[2] += sb[0] * sb[0] + sb[3] * sb[3] + sb[5] * sb[5] + 2.0 * (sb[1] * sb[1] + sb[2] * sb[2] + sb[4] * sb[4]);
    acc[3] += 0.5 * (Sb * Sb * Sb * Sb);
    acc[4] += Sb * (b[0] * sb[0] + b[3] * sb[3] + b[5] * sb[5] + 2.0 * (b[1] * sb[1] + b[2] * sb[2] + b[4] * sb[4]));
    acc[5] += Sh * (h[0] * Q[0] + h[3] * Q[3] + h[5] * Q[5] + 2.0 * (h[1] * Q[1] + h[2] * Q[2] + h[4] * Q[4]));
    acc[6] += sh_[0] * Q[0] + sh_[3] * Q[3] + sh_[5] * Q[5] + 2.0 * (sh_[1] * Q[1] + sh_[2] * Q[2] + sh_[4] * Q[4]);
    acc[7] += sh_[0] * sh_[0] + sh_[3] * sh_[3] + sh_[5] * sh_[5] + 2.0 * (sh_[1] * sh_[1] + sh_[2] * sh_[2] + sh_[4] * sh_[4]);
    acc[8] += 0.5 * (Sh * Sh * Sh * Sh);
    acc[9] += Sh * (h[0] * sh_[0] + h[3] * sh_[3] + h[5] * sh_[5] + 2.0 * (h[1] * sh_[1] + h[2] * sh_[2] + h[4] * sh_[4]));
  }
  for (int q = 0; q < 10; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 10; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 10) sums[(size_t)(jz0 - 1 + lc) * 10 + threadIdx.x] = sh[threadIdx.x][0];
}
// sgsmodule.f90:37-59 rtnewt and scaledep_dynamic.f90:187-244 second pass
__device__ double rtnewt_d(const double* A) {
  double r = 0.5 * (0.0 + 15.0);
  for (int j = 1; j <= 100; ++j) {
    const double f = A[0] + r * (A[1] + r * (A[2] + r * (A[3] + r * (A[4] + r * A[5]))));
    const double df = A[1] + r * (2.0 * A[2] + r * (3.0 * A[3] + r * (4.0 * A[4] + r * (5.0 * A[5]))));
    const double d = f / df;
    r = r - d;
    if (fabs(d) < 0.001) return r;
  }
  return 1.0;
}
__global__ void __launch_bounds__(256) k_sd_final(const double* __restrict__ flt, const double* __restrict__ sums,
                                                  double* cs_z, int ld, int nx, int ny, int nlev, size_t np,
                                                  int jz0, double delta) {
  __shared__ double sn[256], sd[256];
  __shared__ double beta_s;
  const int lc = blockIdx.x;
  const int jz = jz0 + lc;
  const size_t st = np * nlev;
  if (threadIdx.x == 0 && !sums) beta_s = 1.0;  // std_dynamic.f90:120-127: no scale dependence
  if (threadIdx.x == 0 && sums) {
    const double* s = sums + (size_t)(jz - 1) * 10;
    const double N2 = (double)(nx * ny);
    const double d2 = delta * delta, t2 = (2.0 * d2) * (2.0 * d2);
    const double a1 = -2.0 * d2 * 4.0 * s[0] / N2, b1 = -2.0 * d2 * s[1] / N2, c1 = t2 * s[2] / N2;
    const double d1 = t2 * 16.0 * s[3] / N2, e1 = 2.0 * t2 * 4.0 * s[4] / N2;
    const double a2 = -2.0 * d2 * 16.0 * s[5] / N2, b2 = -2.0 * d2 * s[6] / N2, c2 = t2 * s[7] / N2;
    const double dd2 = t2 * 256.0 * s[8] / N2, e2 = 2.0 * t2 * 16.0 * s[9] / N2;
    double A[6];
    A[0] = b2 * c1 - b1 * c2;
    A[1] = a1 * c2 - b2 * e1;
    A[2] = b2 * d1 + b1 * e2 - a2 * c1;
    A[3] = a2 * e1 - a1 * e2;
    A[4] = -a2 * d1 - b1 * dd2;
    A[5] = a1 * dd2;
    beta_s = rtnewt_d(A);
  }
  __syncthreads();
  const double beta = beta_s;
  const double cst = 2.0 * (delta * delta);
  double num = 0.0, den = 0.0;
  for (int e = threadIdx.x; e < nx * ny; e += blockDim.x) {
    const int jy = e / nx, jx = e - jy * nx;
    const size_t t = (size_t)lc * np + (size_t)jy * ld + jx;
    const double* G = flt + t;
    const double ub = G[0], vb = G[st], wb = G[2 * st];
    const double L[6] = {G[3 * st] - ub * ub, G[4 * st] - ub * vb, G[5 * st] - ub * wb,
                         G[6 * st] - vb * vb, G[7 * st] - vb * wb, G[8 * st] - wb * wb};
    double b[6], sb[6];
    for (int q = 0; q < 6; ++q) { b[q] = G[(9 + q) * st]; sb[q] = G[(15 + q) * st]; }
    const double Sb = smag(b[0], b[3], b[5], b[1], b[2], b[4]);
    double M[6];
    for (int q = 0; q < 6; ++q) M[q] = cst * (sb[q] - 4.0 * beta * Sb * b[q]);
    num += L[0] * M[0] + L[3] * M[3] + L[5] * M[5] + 2.0 * (L[1] * M[1] + L[2] * M[2] + L[4] * M[4]);
    den += M[0] * M[0] + M[3] * M[3] + M[5] * M[5] + 2.0 * (M[1] * M[1] + M[2] * M[2] + M[4] * M[4]);
  }
  sn[threadIdx.x] = num; sd[threadIdx.x] = den;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) { sn[threadIdx.x] += sn[threadIdx.x + w]; sd[threadIdx.x] += sd[threadIdx.x + w]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) cs_z[jz - 1] = fmax(0.0, sn[0] / sd[0]);
}
// lagrange_Ssim.f90:140-269 (model 4) on one chunk of levels: L_ij and M_ij
// (fourbeta = 4 Beta = 4) from the 21 G_test-filtered planes, LM and MM per
// point, the Lagrangian relaxation of F_LM, F_MM and Cs^2 = F_LM / F_MM.
// Every column of (ld,ny) is relaxed as the reference does; LM = MM = 0 on
// the padding columns, where Cs^2 ends at eps.
__global__ void k_ssim_final(const double* __restrict__ flt, double* F_LM, double* F_MM, double* Cs,
                             int ld, int nx, int ny, int nlev, size_t np, int jz0, double cst, double opftdelta,
                             double lagran_dt) {
  const double eps = 1e-32;  // lagrange_Ssim.f90:25
  const size_t st = np * nlev;
  GSTRIDE(t, st) {
    const int lc = (int)(t / np);
    const size_t r = t - (size_t)lc * np;
    const int jx = (int)(r % ld);
    const size_t i = (size_t)(jz0 - 1 + lc) * np + r;
    double LM = 0.0, MM = 0.0;
    if (jx < nx) {
      const double* G = flt + t;
      const double ub = G[0], vb = G[st], wb = G[2 * st];
      const double L[6] = {G[3 * st] - ub * ub, G[4 * st] - ub * vb, G[5 * st] - ub * wb,
                           G[6 * st] - vb * vb, G[7 * st] - vb * wb, G[8 * st] - wb * wb};
      double b[6], sb[6], M[6];
      for (int q = 0; q < 6; ++q) { b[q] = G[(9 + q) * st]; sb[q] = G[(15 + q) * st]; }
      const double Sb = smag(b[0], b[3], b[5], b[1], b[2], b[4]);
      for (int q = 0; q < 6; ++q) M[q] = cst * (sb[q] - 4.0 * Sb * b[q]);
      LM = L[0] * M[0] + L[3] * M[3] + L[5] * M[5] + 2.0 * (L[1] * M[1] + L[2] * M[2] + L[4] * M[4]);
      MM = M[0] * M[0] + M[3] * M[3] + M[5] * M[5] + 2.0 * (M[1] * M[1] + M[2] * M[2] + M[4] * M[4]);
    }
    double flm = F_LM[i], fmm = F_MM[i];
    double Tn = fmax(flm * fmm, eps);
    Tn = opftdelta * pow_m18(Tn);
    const double dumfac = lagran_dt / Tn;
    const double epsi = dumfac / (1.0 + dumfac);
    flm = epsi * LM + (1.0 - epsi) * flm;
    fmm = epsi * MM + (1.0 - epsi) * fmm;
    flm = fmax(eps, flm);
    F_LM[i] = flm;
    F_MM[i] = fmm;
    Cs[i] = fmax(eps, jx < nx ? flm / fmm : 0.0);
  }
}
// lagrange_Ssim.f90:5-335 (model 4): Beta = 1, interpolag_Ssim, then per
// chunk of levels the 21 planes of k_sd_prep G_test-filtered and the
// relaxation of k_ssim_final
int op_lagrange_ssim(les_ctx* c, const double* const* S) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  fill(c, c->f[LES_BETA], g.nfield, 1.0);
  op_interpolag_n(c, 2);
  Ptr6 Sp;
  for (int q = 0; q < 6; ++q) Sp.p[q] = S[q];
  const double cst = 2.0 * (g.delta * g.delta), opftdelta = 1.5 * g.delta;
  const double lagran_dt = k.dt * (double)k.cs_count;
  const int nch = c->lag_chunk;
  for (int jz0 = 1; jz0 <= g.nz; jz0 += nch) {
    const int nl = std::min(nch, g.nz - jz0 + 1);
    double* prep = c->tmp;
    double* flt = c->tmp + (size_t)21 * nch * g.nplane;
    k_sd_prep<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W],
                                                          Sp, prep, g.ld, g.nx, g.ny,
                                                          jz0, nl, g.nplane); LES_COUNT_LAUNCH();
    const double* in[21];
    for (int q = 0; q < 21; ++q) in[q] = prep + (size_t)q * nl * g.nplane;
    r2c(c, 21, nl, in, (long)g.nplane, nullptr, nullptr, c->wsA, false, g.lh);
    ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nl);
    J.nin = 1; J.nout = 1; J.nf = 21;
    J.in[0] = c->wsA; J.fs_in = (long)nl * g.C;
    J.out[0] = c->wsB; J.fs_out = (long)nl * g.C;
    J.coef[0][0] = CC_G;
    cols(c, J);
    double* out[21];
    for (int q = 0; q < 21; ++q) out[q] = flt + (size_t)q * nl * g.nplane;
    c2r(c, 21, nl, c->wsB, out, (long)g.nplane, false, g.lh);
    k_ssim_final<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(flt, c->f[LES_F_LM], c->f[LES_F_MM],
                                                             c->f[LES_CS_OPT2], g.ld, g.nx, g.ny, nl, g.nplane,
                                                             jz0, cst, opftdelta, lagran_dt); LES_COUNT_LAUNCH();
  }
  return 0;
}

// std_dynamic.f90:1-136 (model 2) -> cs_z (device, nz): the 21 planes of
// k_sd_prep G_test-filtered, then k_sd_final with beta = 1 and
// delta = (dx dy dz)^(1/3) (std_dynamic.f90:28)
int op_stddyn(les_ctx* c, double* cs_z, const double* const* S) {
  const Grid& g = c->g;
  Ptr6 Sp;
  for (int q = 0; q < 6; ++q) Sp.p[q] = S[q];
  const double delta3 = std::pow(g.dx * g.dy * g.dz, 1.0 / 3.0);
  const int nch = c->lag_chunk;
  for (int jz0 = 1; jz0 <= g.nz; jz0 += nch) {
    const int nl = std::min(nch, g.nz - jz0 + 1);
    double* prep = c->tmp;
    double* flt = c->tmp + (size_t)21 * nch * g.nplane;
    k_sd_prep<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W],
                                                          Sp, prep, g.ld, g.nx, g.ny,
                                                          jz0, nl, g.nplane); LES_COUNT_LAUNCH();
    const double* in[21];
    for (int q = 0; q < 21; ++q) in[q] = prep + (size_t)q * nl * g.nplane;
    r2c(c, 21, nl, in, (long)g.nplane, nullptr, nullptr, c->wsA, false, g.lh);
    ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nl);
    J.nin = 1; J.nout = 1; J.nf = 21;
    J.in[0] = c->wsA; J.fs_in = (long)nl * g.C;
    J.out[0] = c->wsB; J.fs_out = (long)nl * g.C;
    J.coef[0][0] = CC_G;
    cols(c, J);
    double* out[21];
    for (int q = 0; q < 21; ++q) out[q] = flt + (size_t)q * nl * g.nplane;
    c2r(c, 21, nl, c->wsB, out, (long)g.nplane, false, g.lh);
    k_sd_final<<<nl, 256, 0, c->stream>>>(flt, nullptr, cs_z, g.ld, g.nx, g.ny, nl, g.nplane, jz0, delta3); LES_COUNT_LAUNCH();
  }
  return 0;
}
int op_scaledep(les_ctx* c, double* cs_z, const double* const* S) {
  const Grid& g = c->g;
  Ptr6 Sp;
  for (int q = 0; q < 6; ++q) Sp.p[q] = S[q];
  double* sums = c->dred + 2 * (size_t)(g.nz + 8);
  const int nch = c->lag_chunk;
  for (int jz0 = 1; jz0 <= g.nz; jz0 += nch) {
    const int nl = std::min(nch, g.nz - jz0 + 1);
    double* prep = c->tmp;
    double* flt = c->tmp + (size_t)21 * nch * g.nplane;
    k_sd_prep<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W],
                                                          Sp, prep, g.ld, g.nx, g.ny,
                                                          jz0, nl, g.nplane); LES_COUNT_LAUNCH();
    const double* in[21];
    for (int q = 0; q < 21; ++q) in[q] = prep + (size_t)q * nl * g.nplane;
    r2c(c, 21, nl, in, (long)g.nplane, nullptr, nullptr, c->wsA, false, g.lh);
    ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nl);
    J.nin = 1; J.nout = 2; J.nf = 21;
    J.in[0] = c->wsA; J.fs_in = (long)nl * g.C;
    J.out[0] = c->wsB; J.out[1] = (C2*)c->wsB + (size_t)21 * nl * g.C; J.fs_out = (long)nl * g.C;
    J.coef[0][0] = CC_G; J.coef[1][0] = CC_GG;
    cols(c, J);
    double* out[42];
    for (int q = 0; q < 42; ++q) out[q] = flt + (size_t)q * nl * g.nplane;
    c2r(c, 42, nl, c->wsB, out, (long)g.nplane, false, g.lh);
    // Q_ij inputs: products of the G-filtered velocities, then GG-filtered
    double* qin = prep;  // reuse: 6 * nl planes
    k_sd_qprep<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(flt, qin, nl, g.nplane); LES_COUNT_LAUNCH();
    const double* qi[6];
    double* qo[6];
    for (int q = 0; q < 6; ++q) { qi[q] = qin + (size_t)q * nl * g.nplane; qo[q] = prep + (size_t)(6 + q) * nl * g.nplane; }
    r2c(c, 6, nl, qi, (long)g.nplane, nullptr, nullptr, c->wsA, false, g.lh);
    ColJob K = coljob(c, MAP_SAME, DIR_BOTH, nl);
    K.nin = 1; K.nout = 1; K.nf = 6; K.in[0] = c->wsA; K.fs_in = (long)nl * g.C;
    K.out[0] = c->wsB; K.fs_out = (long)nl * g.C; K.coef[0][0] = CC_GG;
    cols(c, K);
    c2r(c, 6, nl, c->wsB, qo, (long)g.nplane, false, g.lh);
    k_sd_sums<<<nl, 256, 0, c->stream>>>(flt, prep + (size_t)6 * nl * g.nplane, sums, g.ld, g.nx, g.ny, nl,
                                         g.nplane, jz0); LES_COUNT_LAUNCH();
    k_sd_final<<<nl, 256, 0, c->stream>>>(flt, sums, cs_z, g.ld, g.nx, g.ny, nl, g.nplane, jz0, g.delta); LES_COUNT_LAUNCH();
  }
  return 0;
}

// ---------------------------------------------------------------------------
// divstress_uv.f90:1-63 and divstress_w.f90:4-86, with the horizontal
// derivatives summed in spectral space (one inverse transform per component).
__global__ void k_divstress_fin(double* __restrict__ divx, double* __restrict__ divy,
                                double* __restrict__ divz, const double* __restrict__ hx,
                                const double* __restrict__ hy, const double* __restrict__ hz,
                                const double* __restrict__ txz, const double* __restrict__ tyz,
                                const double* __restrict__ tzz, int ld, int nx, int ny, int nz, double cdz,
                                int want) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * nz) {
    const int jz = (int)(i / np) + 1;
    const int jx = (int)((i - (size_t)(jz - 1) * np) % ld);
    if (jz == nz) {
      if (want & 1) divx[i] = LES_BOGUS;
      if (want & 2) divy[i] = LES_BOGUS;
      if (want & 4) divz[i] = (jx >= nx) ? 0.0 : hz[i] + 0.0;
      continue;
    }
    if (jx >= nx) {
      if (want & 1) divx[i] = 0.0;
      if (want & 2) divy[i] = 0.0;
      if (want & 4) divz[i] = 0.0;
      continue;
    }
    if (want & 1) divx[i] = hx[i] + cdz * (txz[i + np] - txz[i]);
    if (want & 2) divy[i] = hy[i] + cdz * (tyz[i + np] - tyz[i]);
    if (want & 4) divz[i] = (jz == 1) ? hz[i] : hz[i] + cdz * (tzz[i] - tzz[i - np]);
  }
}
int op_divstress(les_ctx* c, double* divtx, double* divty, double* divtz) {
  const Grid& g = c->g;
  const double sc = 1.0 / (double)(g.nx * g.ny);
  const double* in[5] = {c->f[LES_TXX], c->f[LES_TXY], c->f[LES_TYY], c->f[LES_TXZ], c->f[LES_TYZ]};
  double scs[5] = {sc, sc, sc, sc, sc};
  r2c(c, 5, g.nz, in, (long)g.nplane, scs, nullptr, c->wsA, false, g.lh);
  const long FS = (long)g.nz * g.C;
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, g.nz);
  J.nin = 3; J.nout = 2;
  J.in[0] = c->wsA; J.in[1] = (C2*)c->wsA + FS; J.in[2] = (C2*)c->wsA + 2 * FS;
  J.out[0] = c->wsB; J.out[1] = (C2*)c->wsB + FS;
  J.coef[0][0] = CC_IKX; J.coef[0][1] = CC_IKY;   // d txx/dx + d txy/dy
  J.coef[1][1] = CC_IKX; J.coef[1][2] = CC_IKY;   // d txy/dx + d tyy/dy
  cols(c, J);
  ColJob K = coljob(c, MAP_SAME, DIR_BOTH, g.nz);
  K.nin = 2; K.nout = 1;
  K.in[0] = (C2*)c->wsA + 3 * FS; K.in[1] = (C2*)c->wsA + 4 * FS;
  K.out[0] = (C2*)c->wsB + 2 * FS;
  K.coef[0][0] = CC_IKX; K.coef[0][1] = CC_IKY;   // d txz/dx + d tyz/dy
  cols(c, K);
  double* h[3] = {c->tmp, c->tmp + g.nfield, c->tmp + 2 * g.nfield};
  c2r(c, 3, g.nz, c->wsB, h, (long)g.nplane, false, g.lh);
  k_divstress_fin<<<grid1(g.nfield), 256, 0, c->stream>>>(divtx, divty, divtz, h[0], h[1], h[2], c->f[LES_TXZ],
                                                         c->f[LES_TYZ], c->f[LES_TZZ], g.ld, g.nx, g.ny, g.nz,
                                                         1.0 / g.dz, 7); LES_COUNT_LAUNCH();
  return 0;
}
// single divstress call with caller-supplied stresses (per-routine entry point)
int op_divstress_one(les_ctx* c, double* divt, const double* tx, const double* ty, const double* tz,
                     int w_variant) {
  const Grid& g = c->g;
  const double sc = 1.0 / (double)(g.nx * g.ny);
  const double* in[2] = {tx, ty};
  double scs[2] = {sc, sc};
  r2c(c, 2, g.nz, in, (long)g.nplane, scs, nullptr, c->wsA, false, g.lh);
  const long FS = (long)g.nz * g.C;
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, g.nz);
  J.nin = 2; J.nout = 1;
  J.in[0] = c->wsA; J.in[1] = (C2*)c->wsA + FS; J.out[0] = c->wsB;
  J.coef[0][0] = CC_IKX; J.coef[0][1] = CC_IKY;
  cols(c, J);
  double* h = c->tmp;
  c2r(c, 1, g.nz, c->wsB, &h, (long)g.nplane, false, g.lh);
  if (!w_variant) {
    k_divstress_fin<<<grid1(g.nfield), 256, 0, c->stream>>>(divt, nullptr, nullptr, h, nullptr, nullptr, tz, nullptr,
                                                           nullptr, g.ld, g.nx, g.ny, g.nz, 1.0 / g.dz, 1); LES_COUNT_LAUNCH();
  } else {
    k_divstress_fin<<<grid1(g.nfield), 256, 0, c->stream>>>(nullptr, nullptr, divt, nullptr, nullptr, h, nullptr,
                                                           nullptr, tz, g.ld, g.nx, g.ny, g.nz, 1.0 / g.dz, 4); LES_COUNT_LAUNCH();
  }
  return 0;
}

// ---------------------------------------------------------------------------
// convec.f90:67-114 vorticity inputs (already multiplied by 1/(nx*ny))
__global__ void k_vort(const double* __restrict__ dudy, const double* __restrict__ dudz,
                       const double* __restrict__ dvdx, const double* __restrict__ dvdz,
                       const double* __restrict__ dwdx, const double* __restrict__ dwdy, double* o1,
                       double* o2, double* o3, int ld, int ny, int nz, double cst) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * nz) {
    const int jz = (int)(i / np) + 1;
    if (jz == 1) {  // lbc_mom = 'wall'
      o1[i] = cst * (0.5 * (dwdy[i] + dwdy[i + np]) - dvdz[i]);
      o2[i] = cst * (dudz[i] - 0.5 * (dwdx[i] + dwdx[i + np]));
    } else {
      o1[i] = cst * (dwdy[i] - dvdz[i]);
      o2[i] = cst * (dudz[i] - dwdx[i]);
    }
    o3[i] = cst * (dvdx[i] - dudy[i]);
  }
}
// convec.f90:117-217 products on the 3/2 grid, levels 1..nz-1
template <typename S>
__global__ void k_convec_prod(const S* __restrict__ u1, const S* __restrict__ u2,
                              const S* __restrict__ u3, const S* __restrict__ w1,
                              const S* __restrict__ w2, const S* __restrict__ w3, S* ccx,
                              S* ccy, S* ccz, int ldb, int nx2, int ny2, int nz, S cst) {
  const size_t np = (size_t)ldb * ny2;
  GSTRIDE(i, np * (nz - 1)) {
    const int jz = (int)(i / np) + 1;
    const int jx = (int)((i - (size_t)(jz - 1) * np) % ldb);
    if (jx >= nx2) continue;
    const size_t ip = i + np;
    const S h = (S)0.5;
    if (jz == 1) {
      ccx[i] = cst * (u2[i] * (-w3[i]) + h * u3[ip] * (w2[ip]));
      ccy[i] = cst * (u1[i] * (w3[i]) + h * u3[ip] * (-w1[ip]));
      ccz[i] = (S)0;
    } else {
      const size_t im = i - np;
      ccx[i] = cst * (u2[i] * (-w3[i]) + h * (u3[ip] * (w2[ip]) + u3[i] * (w2[i])));
      ccy[i] = cst * (u1[i] * (w3[i]) + h * (u3[ip] * (-w1[ip]) + u3[i] * (-w1[i])));
      ccz[i] = cst * h * ((u1[i] + u1[im]) * (-w2[i]) + (u2[i] + u2[im]) * (w1[i]));
    }
  }
}
int op_convec(les_ctx* c, double* cx, double* cy, double* cz) {
  const Grid& g = c->g;
  const double cst = 1.0 / (double)(g.nx * g.ny);
  double* vort[3] = {c->tmp, c->tmp + g.nfield, c->tmp + 2 * g.nfield};
  k_vort<<<grid1(g.nfield), 256, 0, c->stream>>>(c->f[LES_DUDY], c->f[LES_DUDZ], c->f[LES_DVDX], c->f[LES_DVDZ],
                                                c->f[LES_DWDX], c->f[LES_DWDY], vort[0], vort[1], vort[2], g.ld,
                                                g.ny, g.nz, cst); LES_COUNT_LAUNCH();
  const double* in[6] = {c->f[LES_U], c->f[LES_V], c->f[LES_W], vort[0], vort[1], vort[2]};
  double* bigf[9];
  for (int q = 0; q < 9; ++q) bigf[q] = c->big + (size_t)q * g.nfield_big;
  // dealias1 semantics: scale 1/(nx*ny) for the velocities, vorticity already scaled
  {
    double sc[6] = {cst, cst, cst, 1.0, 1.0, 1.0};
    r2c(c, 6, g.nz, in, (long)g.nplane, sc, nullptr, c->wsA, false, g.lh);
    ColJob J = coljob(c, MAP_PAD, DIR_BOTH, g.nz);
    J.nin = 1; J.nout = 1; J.nf = 6;
    J.in[0] = c->wsA; J.fs_in = (long)g.nz * g.C;
    J.out[0] = c->wsB; J.fs_out = (long)g.nz * g.CB;
    J.coef[0][0] = CC_ONE;
    cols(c, J);
    c2r(c, 6, g.nz, c->wsB, bigf, (long)g.nplane_big, true, g.nx / 2);
  }
  const double cst2 = 1.0 / (double)(g.nx2 * g.ny2);
  k_convec_prod<double><<<grid1(g.nplane_big * (g.nz - 1)), 256, 0, c->stream>>>(
      bigf[0], bigf[1], bigf[2], bigf[3], bigf[4], bigf[5], bigf[6], bigf[7], bigf[8], g.ld_big, g.nx2, g.ny2,
      g.nz, cst2); LES_COUNT_LAUNCH();
  double* outs[3] = {cx, cy, cz};
  const double* bins[3] = {bigf[6], bigf[7], bigf[8]};
  op_dealias2(c, outs, bins, 3, g.nz - 1, 1.0);
  const size_t top = (size_t)(g.nz - 1) * g.nplane;
  fill(c, cx + top, g.nplane, LES_BOGUS);
  fill(c, cy + top, g.nplane, LES_BOGUS);
  fill(c, cz + top, g.nplane, LES_BOGUS);
  return 0;
}

// ---------------------------------------------------------------------------
// main.f90:309-390 : RHS assembly, buoyancy, Euler/AB2 predictor, u(nz)=BOGUS
__global__ void k_rhs_ab2(double* u, double* v, double* w, double* Rx, double* Ry, double* Rz, double* Rxf,
                          double* Ryf, double* Rzf, const double* __restrict__ dx_, const double* __restrict__ dy_,
                          const double* __restrict__ dz_, const double* __restrict__ bs, size_t nv, size_t np,
                          double dt, int sflag, int euler) {
  GSTRIDE(i, nv + np) {
    if (i >= nv) { u[i] = LES_BOGUS; v[i] = LES_BOGUS; w[i] = LES_BOGUS; continue; }
    const double rx = -Rx[i] - dx_[i];
    const double ry = -Ry[i] - dy_[i];
    double rz = -Rz[i] - dz_[i];
    if (sflag) rz = rz + bs[i];
    Rx[i] = rx; Ry[i] = ry; Rz[i] = rz;
    double fx = Rxf[i], fy = Ryf[i], fz = Rzf[i];
    if (euler) { fx = rx; fy = ry; fz = rz; Rxf[i] = rx; Ryf[i] = ry; Rzf[i] = rz; }
    u[i] = u[i] + dt * (1.5 * rx + (1.0 - 1.5) * fx + 0.0);
    v[i] = v[i] + dt * (1.5 * ry + (1.0 - 1.5) * fy);
    w[i] = w[i] + dt * (1.5 * rz + (1.0 - 1.5) * fz);
  }
}

// ---------------------------------------------------------------------------
// Mixed form: the convective term split about the plane-mean wind.
// With u = U(z) + u', v = V(z) + v' (U, V the plane means of the uvp levels)
// and the w-level vorticity w_x = Ox(z) + w_x', w_y = Oy(z) + w_y' (Oy = dU/dz,
// Ox = -dV/dz; w_z has no plane mean), the products of convec.f90:117-217
//   cx = -v w_z + (w w_y)~      cy = u w_z - (w w_x)~
//   cz = ((u + u_m)(-w_y) + (v + v_m) w_x) / 2       (~: the two-level average)
// are the FP32 products of the fluctuations (k_convec_prod on u', v', w and
// w_x', w_y', w_z, 3/2-dealiased as before) plus terms linear in one
// fluctuating field with a plane-constant factor, plus a plane constant:
//   cx_lin = -V w_z + (Oy w)~          cy_lin = U w_z - (Ox w)~
//   cz_lin = (-(U + U_m) w_y' - Oy (u' + u'_m) + (V + V_m) w_x' + Ox (v' + v'_m)) / 2
//            + (-(U + U_m) Oy + (V + V_m) Ox) / 2
// A plane constant times a band-limited field is band-limited, so the 3/2
// dealiasing leaves the linear terms unchanged: they are formed on the
// small grid.  U w_z is of order U k |v'| (about 260 at 256^3), so w_z and
// dw/dx come from float-float transforms (k_rhs_ab2_mx reads them) and the
// linear terms and the right-hand-side sums run in float-float arithmetic.
// In FP32 they left a relative error of about 5e-8 per step in v and w.
// Per-level factors in float-float (entry jz, 1-based):
//   U, V at uvp level jz; Oy, Ox at w-level jz (zero at jz = 1 and nz:
//   level 1 vorticity is not read by the products, level nz is w = 0);
//   Cz = the plane constant of cz at w-level jz; UVf = (U, V) in FP32.
struct MeanTab {
  float2 *U, *V, *Oy, *Ox, *Cz, *UVf;
};
// d/dx of x-spectra with y still physical (rows [plane][ny][lh], float-float):
// out = i kx in (acc: out += i kx in), kx of the column (the kx = nx/2 column
// zeroed, as ddx.f90 zeroes it).  The fields this is used on carry no
// ky = ny/2 content (Nyquist-filtered state, or p-hat with its Nyquist modes
// zeroed), so skipping the y round trip that ddx would make loses nothing;
// the forward x pass that made `in` is scaled for an x round trip alone
// (1/nx, not 1/(nx ny)), or `in` is already the inverse y transform.
// The column's kx: row 0 of the (lh, ny) table, as a float-float pair or FP64.
template <typename CX> struct KxCol;
template <> struct KxCol<dcomplex> {
  static __device__ __forceinline__ dfloat get(const float2* __restrict__ kxd, const double*, int jx) {
    const float2 kv = kxd[jx];
    return dfloat(kv.x, kv.y);
  }
};
template <> struct KxCol<double2> {
  static __device__ __forceinline__ double get(const float2*, const double* __restrict__ kx, int jx) {
    return kx[jx];
  }
};
template <typename CX>
__global__ void k_ikx_rows(const CX* __restrict__ in, CX* out, const float2* __restrict__ kxd,
                           const double* __restrict__ kx, int lh, size_t n, int acc) {
  GSTRIDE(e, n) {
    const int jx = (int)(e % lh);
    const auto k = KxCol<CX>::get(kxd, kx, jx);
    const CX v = in[e];
    CX r;
    r.x = -(k * v.y);
    r.y = k * v.x;
    if (acc) {
      const CX o = out[e];
      r.x = r.x + o.x;
      r.y = r.y + o.y;
    }
    out[e] = r;
  }
}
static MeanTab mean_tab(les_ctx* c) {
  const size_t ms = (size_t)c->g.nz + 8;
  float2* b = reinterpret_cast<float2*>(c->dred + 28 * ms);  // slots 28..33
  return MeanTab{b, b + ms, b + 2 * ms, b + 3 * ms, b + 4 * ms, b + 5 * ms};
}
__device__ __forceinline__ float2 df2(double x) {
  const dfloat d = cvt<dfloat>(x);
  return make_float2(d.hi, d.lo);
}
__global__ void k_mean_tab(const double* __restrict__ mean, int ms, int nz, double dz, MeanTab T) {
  const int jz = blockIdx.x * blockDim.x + threadIdx.x + 1;  // 1..nz
  if (jz > nz) return;
  const double U = mean[jz - 1], V = mean[ms + jz - 1];
  double oy = 0.0, ox = 0.0, cz = 0.0;
  if (jz >= 2 && jz <= nz - 1) {
    const double Um = mean[jz - 2], Vm = mean[ms + jz - 2];
    oy = (U - Um) / dz;
    ox = -(V - Vm) / dz;
    cz = 0.5 * (-(U + Um) * oy + (V + Vm) * ox);
  }
  T.U[jz] = df2(U);
  T.V[jz] = df2(V);
  T.Oy[jz] = df2(oy);
  T.Ox[jz] = df2(ox);
  T.Cz[jz] = df2(cz);
  T.UVf[jz] = make_float2(cvt_d2f(U), cvt_d2f(V));
  if (jz == nz) {  // w-level nz + 1 is never a neighbour with a nonzero factor
    T.Oy[nz + 1] = make_float2(0.f, 0.f);
    T.Ox[nz + 1] = make_float2(0.f, 0.f);
  }
}
__device__ __forceinline__ dfloat ldt(const float2* p, int j) {
  const float2 v = p[j];
  return dfloat(v.x, v.y);
}
__device__ __forceinline__ dfloat dfs(float a) { return dfloat(a, 0.f); }
__device__ __forceinline__ dfloat ldf2(const float2* p, size_t i) {
  const float2 v = p[i];
  return dfloat(v.x, v.y);
}

// main.f90:309-390 for the mixed form: RHS = -(c_nl + c_lin) - divt
// (+ buoyancy on z), the AB2 predictor u* = u + dt (1.5 RHS - 0.5 RHS_f)
// (Euler on the first step), u*(nz) = BOGUS.  The linear terms read u and w
// at the neighbouring levels, so u*, v*, w* go to separate fields (us, vs,
// ws) and the state keeps its start-of-step values until the projection
// writes u = u* - 1.5 dt grad p.  c_nl (RHSx..z on entry: the FP64-stored
// dealiased FP32 products of the fluctuations) and divt are FP32-accurate;
// the linear terms, the sums and the AB2 increments are float-float.  The
// RHS (this step's, then next step's RHS_f) and u*, v*, w* are stored as
// float-float pairs (hi, lo floats in each 8-byte slot, about 48 bits): no
// FP64 operation joins them, which leaves this kernel five FP64 operations
// per point (splitting u and w into float-float) instead of seventeen; the
// projection forms the FP64 state from u* (k_dpdz_project32).  wz = w_z,
// wx = dw/dx on the uvp / w levels (float-float transforms), dwdy the
// FP32-held dw/dy.  grid (ceil(np/256), nz).
__global__ void __launch_bounds__(256) k_rhs_ab2_mx(
    const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ w, double* Rx,
    double* Ry, double* Rz, float2* Rxf, float2* Ryf, float2* Rzf,
    const double* __restrict__ dx_, const double* __restrict__ dy_, const double* __restrict__ dz_,
    const double* __restrict__ bs, const dfloat* __restrict__ wz, const dfloat* __restrict__ wx,
    const float* __restrict__ dwdy, MeanTab T, float2* __restrict__ us, float2* __restrict__ vs,
    float2* __restrict__ ws, int ld, int ny, int nz, float2 idz2, float2 dt2, int sflag, int euler) {
  const unsigned np = (unsigned)ld * ny;
  const unsigned p = blockIdx.x * 256u + threadIdx.x;
  if (p >= np) return;
  const int jz = blockIdx.y + 1;
  const size_t i = (size_t)(jz - 1) * np + p;
  if (jz == nz) {
    const float2 bog = make_float2((float)LES_BOGUS, 0.f);
    us[i] = bog; vs[i] = bog; ws[i] = bog;
    return;
  }
  const dfloat h(0.5f, 0.f);
  const dfloat idz(idz2.x, idz2.y);  // 1/dz and dt as float-float pairs formed on the host
  const dfloat U = ldt(T.U, jz), V = ldt(T.V, jz);
  const dfloat wi = cvt<dfloat>(w[i]), wp = cvt<dfloat>(w[i + np]);
  const dfloat s1 = wz[i];
  const dfloat oyp = ldt(T.Oy, jz + 1), oxp = ldt(T.Ox, jz + 1), oy = ldt(T.Oy, jz), ox = ldt(T.Ox, jz);
  const dfloat cxl = (-V) * s1 + h * (oyp * wp + oy * wi);
  const dfloat cyl = U * s1 - h * (oxp * wp + ox * wi);
  dfloat czl(0.f, 0.f);
  const dfloat uf = cvt<dfloat>(u[i]);
  if (jz >= 2) {
    const size_t im = i - np;
    const dfloat Um = ldt(T.U, jz - 1);
    const dfloat up = uf - U, upm = cvt<dfloat>(u[im]) - Um;
    const float vp = cvt_d2f(v[i]) - T.UVf[jz].y, vpm = cvt_d2f(v[im]) - T.UVf[jz - 1].y;
    const dfloat wyp = (up - upm) * idz - wx[i];                          // w_y' at w-level jz
    const float wxp = dwdy[i] - (vp - vpm) * idz2.x;                    // w_x' (FP32: its factor V is small)
    const dfloat Us = U + Um;
    const float Vs = T.UVf[jz].y + T.UVf[jz - 1].y;
    czl = h * ((-Us) * wyp - oy * (up + upm)) + dfs(0.5f * (Vs * wxp) + 0.5f * (ox.hi * (vp + vpm))) +
          ldt(T.Cz, jz);
  }
  const dfloat rx = -(dfs(cvt_d2f(Rx[i])) + cxl) - dfs(cvt_d2f(dx_[i]));
  const dfloat ry = -(dfs(cvt_d2f(Ry[i])) + cyl) - dfs(cvt_d2f(dy_[i]));
  dfloat rz = -(dfs(cvt_d2f(Rz[i])) + czl) - dfs(cvt_d2f(dz_[i]));
  if (sflag) rz = rz + cvt<dfloat>(bs[i]);
  const float2 rx2 = make_float2(rx.hi, rx.lo), ry2 = make_float2(ry.hi, ry.lo), rz2 = make_float2(rz.hi, rz.lo);
  reinterpret_cast<float2*>(Rx)[i] = rx2;  // the slot held c_nl in FP64 until now
  reinterpret_cast<float2*>(Ry)[i] = ry2;
  reinterpret_cast<float2*>(Rz)[i] = rz2;
  dfloat fx, fy, fz;
  if (euler) {
    fx = rx; fy = ry; fz = rz;
    Rxf[i] = rx2; Ryf[i] = ry2; Rzf[i] = rz2;
  } else {
    fx = ldf2(Rxf, i); fy = ldf2(Ryf, i); fz = ldf2(Rzf, i);
  }
  const dfloat dtf(dt2.x, dt2.y);
  const dfloat a15(1.5f, 0.f), a05(0.5f, 0.f);
  const dfloat ux = uf + dtf * (a15 * rx - a05 * fx);
  const dfloat vx = cvt<dfloat>(v[i]) + dtf * (a15 * ry - a05 * fy);
  const dfloat wx2 = wi + dtf * (a15 * rz - a05 * fz);
  us[i] = make_float2(ux.hi, ux.lo);
  vs[i] = make_float2(vx.hi, vx.lo);
  ws[i] = make_float2(wx2.hi, wx2.lo);
}

// main.f90:403-410 + forcing.f90:128-219 project, one thread per point of
// levels 1..nz-1; the thread of level nz-1 also sets the top level and the
// thread of level 1 the wall value of w.
__global__ void k_dpdz_project(double* u, double* v, double* w, double* Rx, double* Ry, double* Rz,
                               const double* __restrict__ p, const double* __restrict__ dpdx,
                               const double* __restrict__ dpdy, double* dpdz, int ld, int nx, int ny, int nz,
                               double dz, double dt) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * (nz - 1)) {
    const int jz = (int)(i / np) + 1;
    const size_t r = i - (size_t)(jz - 1) * np;
    const int jx = (int)(r % ld);
    double pz = 0.0;
    if (jx < nx) {
      const double dp = p[r + (size_t)jz * np] - p[r + (size_t)(jz - 1) * np];
      pz = dp / dz;
      dpdz[i] = pz;
    } else {
      pz = dpdz[i];
    }
    Rx[i] = Rx[i] - dpdx[i];
    Ry[i] = Ry[i] - dpdy[i];
    Rz[i] = Rz[i] - pz;
    double uu = u[i], vv = v[i], ww = w[i];
    if (jx < nx) {
      uu = (uu + dt * (-1.5 * dpdx[i] + 0.0));
      vv = (vv + dt * (-1.5 * dpdy[i] + 0.0));
      if (jz >= 2) ww = (ww + dt * (-1.5 * pz + 0.0));
      u[i] = uu; v[i] = vv;
      if (jz >= 2) w[i] = ww;
    }
    if (jz == nz - 1) {
      const size_t top = i + np;
      dpdz[top] = LES_BOGUS;
      u[top] = uu;
      v[top] = vv;
      w[top] = 0.0;
    }
    if (jz == 1) w[i] = 0.0;
  }
}
// Mixed form: dpdz and the projection in FP64 with the fused factor
// -1.5 dt (the pressure comes from float-float transforms and the projection
// sets the divergence): u = u* - 1.5 dt grad p from the float-float
// predictor u*, v*, w* (one FP64 addition joins each), and the RHS
// bookkeeping R -= grad p in float-float on the float-float RHS (it is next
// step's RHS_f; the horizontal RHS are of order U k |v'|, whose FP32
// rounding is 1e-5 of v's own scale).  grid (ceil(np/256), nz-1).
__global__ void __launch_bounds__(256) k_dpdz_project32(double* u, double* v, double* w, const float2* __restrict__ us,
                                                        const float2* __restrict__ vs,
                                                        const float2* __restrict__ ws, float2* Rx, float2* Ry,
                                                        float2* Rz, const double* __restrict__ p,
                                                        const double* __restrict__ dpdx,
                                                        const double* __restrict__ dpdy, double* dpdz, int ld,
                                                        int nx, int ny, int nz, double idz, double dt) {
  const unsigned np = (unsigned)ld * ny;
  const unsigned r = blockIdx.x * 256u + threadIdx.x;
  if (r >= np) return;
  const int jz = blockIdx.y + 1;
  const size_t i = (size_t)(jz - 1) * np + r;
  const bool inx = (int)(r % (unsigned)ld) < nx;
  const double c = -1.5 * dt;
  double pz;
  if (inx) {
    pz = (p[i + np] - p[i]) * idz;
    dpdz[i] = pz;
  } else {
    pz = dpdz[i];
  }
  const double gx = dpdx[i], gy = dpdy[i];
  const dfloat rx = ldf2(Rx, i) - cvt<dfloat>(gx), ry = ldf2(Ry, i) - cvt<dfloat>(gy);
  const dfloat rz = ldf2(Rz, i) - cvt<dfloat>(pz);
  Rx[i] = make_float2(rx.hi, rx.lo);
  Ry[i] = make_float2(ry.hi, ry.lo);
  Rz[i] = make_float2(rz.hi, rz.lo);
  double uu = cvt<double>(ldf2(us, i)), vv = cvt<double>(ldf2(vs, i)), ww = cvt<double>(ldf2(ws, i));
  if (inx) {
    uu = fma(c, gx, uu);
    vv = fma(c, gy, vv);
    if (jz >= 2) ww = fma(c, pz, ww);
  }
  u[i] = uu; v[i] = vv; w[i] = ww;
  if (jz == nz - 1) {
    const size_t top = i + np;
    dpdz[top] = LES_BOGUS;
    u[top] = uu;
    v[top] = vv;
    w[top] = 0.0;
  }
  if (jz == 1) w[i] = 0.0;
}

__global__ void k_project_only(double* u, double* v, double* w, const double* dpdx, const double* dpdy,
                               const double* dpdz, int ld, int nx, int ny, int nz, double dt) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(r, np) {
    const int jx = (int)(r % ld);
    for (int jz = 1; jz <= nz - 1; ++jz) {
      const size_t i = r + (size_t)(jz - 1) * np;
      if (jx < nx) {
        u[i] = (u[i] + dt * (-1.5 * dpdx[i] + 0.0));
        v[i] = (v[i] + dt * (-1.5 * dpdy[i] + 0.0));
        if (jz >= 2) w[i] = (w[i] + dt * (-1.5 * dpdz[i] + 0.0));
      }
    }
    const size_t top = r + (size_t)(nz - 1) * np, below = r + (size_t)(nz - 2) * np;
    u[top] = u[below];
    v[top] = v[below];
    w[top] = 0.0;
    w[r] = 0.0;
  }
}

int op_project(les_ctx* c) {
  // stand-alone project (forcing.f90:128-219): dpdz is taken as given
  const Grid& g = c->g;
  k_project_only<<<grid1(g.nplane), 256, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[LES_DPDX],
                                                        c->f[LES_DPDY], c->f[LES_DPDZ], g.ld, g.nx, g.ny, g.nz,
                                                        c->cfg.dt); LES_COUNT_LAUNCH();
  return 0;
}

// ---------------------------------------------------------------------------
// press_stag_array.f90:192-264 + tridag_array.f90:1-109: one thread per
// wavenumber pair solves its z-tridiagonal (Thomas), building the RHS rows
// from the spectra H on the fly.  Spectra are (level, ny, lh) complex.
// HC, PC: storage of the spectra H and p-hat (double2, or float-float in the
// mixed form); the solve itself is FP64.  One mode t.
template <typename HC, typename PC>
__device__ __forceinline__ void tridiag_mode(int t, const HC* __restrict__ Hx, const HC* __restrict__ Hy,
                                                 const HC* __restrict__ Hz, const C2* __restrict__ bot,
                                                 const C2* __restrict__ top, PC* P, const double* __restrict__ ibet,
                                                 const double* __restrict__ gam, const double* __restrict__ kx,
                                                 const double* __restrict__ ky, int lh, int ny, int nz, double dz) {
  const int nk = lh * ny;
  const int jx = t % lh, jy = t / lh;
  const size_t NK = (size_t)nk;
  if (jy == ny / 2 || jx == lh - 1) {  // Nyquist modes: zeroed (press_stag_array.f90:263-264)
    for (int j = 0; j <= nz; ++j) P[(size_t)j * NK + t] = from_d2<PC>(make_double2(0.0, 0.0));
    return;
  }
  if (t == 0) {  // kx = ky = 0 : direct integration (:238-247)
    C2 p = make_double2(0.0, 0.0);
    P[0] = from_d2<PC>(p);
    const C2 b = bot[0];
    C2 p1; p1.x = p.x - dz * b.x; p1.y = p.y - dz * b.y;
    P[NK] = from_d2<PC>(p1);
    p = p1;
    for (int jz = 2; jz <= nz; ++jz) {
      const C2 h = (jz <= nz - 1) ? to_d2(Hz[(size_t)(jz - 1) * NK]) : make_double2(0.0, 0.0);
      p.x = p.x + h.x * dz; p.y = p.y + h.y * dz;
      P[(size_t)jz * NK] = from_d2<PC>(p);
    }
    return;
  }
  const double k_x = kx[t], k_y = ky[t];
  const double idz2 = 1.0 / (dz * dz);
  const int n = nz + 1;
  // row 1: a = BOGUS, b = -1, c = 1, r = -dz * bottomw ; u = r / bet
  const C2 r1 = bot[t];
  C2 up; up.x = (-dz * r1.x) * ibet[t]; up.y = (-dz * r1.y) * ibet[t];
  P[t] = from_d2<PC>(up);
  C2 hz0 = to_d2(Hz[t]);
  for (int j = 2; j <= n; ++j) {
    double a;
    C2 r;
    if (j <= nz) {
      a = idz2;
      const C2 hx = to_d2(Hx[(size_t)(j - 2) * NK + t]);
      const C2 hy = to_d2(Hy[(size_t)(j - 2) * NK + t]);
      const C2 hz1 = (j <= nz - 1) ? to_d2(Hz[(size_t)(j - 1) * NK + t]) : make_double2(0.0, 0.0);
      const double sr = k_x * hx.x + k_y * hy.x;
      const double si = k_x * hx.y + k_y * hy.y;
      r.x = -si + (hz1.x - hz0.x) / dz;
      r.y = sr + (hz1.y - hz0.y) / dz;
      hz0 = hz1;
    } else {
      a = -1.0;
      const C2 tp = top[t];
      r.x = -tp.x * dz; r.y = -tp.y * dz;
    }
    const double ib = ibet[(size_t)(j - 1) * NK + t];
    C2 u; u.x = (r.x - a * up.x) * ib; u.y = (r.y - a * up.y) * ib;
    P[(size_t)(j - 1) * NK + t] = from_d2<PC>(u);
    up = u;
  }
  for (int j = n - 1; j >= 1; --j) {
    const double gm = gam[(size_t)j * NK + t];
    C2 u = to_d2(P[(size_t)(j - 1) * NK + t]);
    u.x = u.x - gm * up.x; u.y = u.y - gm * up.y;
    P[(size_t)(j - 1) * NK + t] = from_d2<PC>(u);
    up = u;
  }
}

// The same solve with two threads per mode: part 0 the real, part 1 the
// imaginary part of p-hat (a, b, c are real, so the two recurrences are
// independent), each load issued four levels ahead; the arithmetic and its
// order are those of tridiag_mode.  The kx = ky = 0 and Nyquist modes run
// tridiag_mode on part 0.
// Mixed form (float-float spectra): the right-hand side
// -(kx Hx + ky Hy) + (Hz(k) - Hz(k-1))/dz is formed in float-float on the
// FP32 pipe (the inputs carry float-float precision), the recurrences run in
// FP64, and the forward sweep parks its FP64 value in the 8-byte float-float
// slot of p-hat that the back sweep reads and overwrites, so each level
// costs five FP64 instructions instead of fourteen.
template <typename HC> __device__ __forceinline__ double ld1(const HC* p, size_t i, int comp);
template <> __device__ __forceinline__ double ld1<double2>(const double2* p, size_t i, int comp) {
  return reinterpret_cast<const double*>(p)[2 * i + comp];
}
template <> __device__ __forceinline__ double ld1<dcomplex>(const dcomplex* p, size_t i, int comp) {
  return cvt<double>(reinterpret_cast<const dfloat*>(p)[2 * i + comp]);
}
__device__ __forceinline__ void st1(double2* p, size_t i, int comp, double v) {
  reinterpret_cast<double*>(p)[2 * i + comp] = v;
}
__device__ __forceinline__ void st1(dcomplex* p, size_t i, int comp, double v) {
  reinterpret_cast<dfloat*>(p)[2 * i + comp] = cvt<dfloat>(v);
}
__device__ __forceinline__ dfloat ldf(const dcomplex* p, size_t i, int comp) {
  return reinterpret_cast<const dfloat*>(p)[2 * i + comp];
}
// an FP64 value parked in the 8-byte slot of one component
template <typename PC> __device__ __forceinline__ void st_park(PC* p, size_t i, int comp, double v) {
  reinterpret_cast<double*>(p)[2 * i + comp] = v;
}
template <typename PC> __device__ __forceinline__ double ld_park(const PC* p, size_t i, int comp) {
  return reinterpret_cast<const double*>(p)[2 * i + comp];
}
template <typename HC, typename PC>
__global__ void __launch_bounds__(128) k_tridiag2(const HC* __restrict__ Hx, const HC* __restrict__ Hy,
                                                  const HC* __restrict__ Hz, const C2* __restrict__ bot,
                                                  const C2* __restrict__ top, PC* P, const double* __restrict__ ibet,
                                                  const double* __restrict__ gam, const double* __restrict__ kx,
                                                  const double* __restrict__ ky, const float2* __restrict__ kxd,
                                                  const float2* __restrict__ kyd, int lh, int ny, int nz, double dz,
                                                  const int* __restrict__ modes, int nmodes) {
  const int nk = lh * ny;
  const int g2 = blockIdx.x * blockDim.x + threadIdx.x;
  int t = g2 >> 1;
  const int part = g2 & 1;
  if (modes) {  // a list of modes (the mixed form's lowest |k|)
    if (t >= nmodes) return;
    t = modes[t];
  } else if (t >= nk) {
    return;
  }
  const int jx = t % lh, jy = t / lh;
  if (t == 0 || jy == ny / 2 || jx == lh - 1) {
    if (part == 0) tridiag_mode<HC, PC>(t, Hx, Hy, Hz, bot, top, P, ibet, gam, kx, ky, lh, ny, nz, dz);
    return;
  }
  const size_t NK = (size_t)nk;
  const int ch = part == 0 ? 1 : 0;  // component of Hx, Hy feeding this part
  const int n = nz + 1;
  const C2 b1 = bot[t];
  double up = (-dz * (part == 0 ? b1.x : b1.y)) * ibet[t];
  constexpr int D = 4;
  if constexpr (std::is_same<HC, dcomplex>::value) {
    const dfloat k_x(kxd[t].x, kxd[t].y), k_y(kyd[t].x, kyd[t].y);
    const dfloat idzf(1.0 / dz);
    const double idz2 = 1.0 / (dz * dz);
    st_park(P, t, part, up);
    dfloat hz0 = ldf(Hz, t, part);
    const dfloat zero(0.f, 0.f);
    // level j's inputs in ring slot (j - 2) % 4, loaded four levels ahead
    dfloat bx[D], by[D], bz[D];
    double bi[D];
    auto load = [&](int j, dfloat& x, dfloat& y, dfloat& z, double& ib) {
      if (j <= n) ib = ibet[(size_t)(j - 1) * NK + t];
      if (j <= nz) {
        x = ldf(Hx, (size_t)(j - 2) * NK + t, ch);
        y = ldf(Hy, (size_t)(j - 2) * NK + t, ch);
      }
      z = (j <= nz - 1) ? ldf(Hz, (size_t)(j - 1) * NK + t, part) : zero;
    };
#pragma unroll
    for (int q = 0; q < D; ++q) load(2 + q, bx[q], by[q], bz[q], bi[q]);
    for (int jb = 2; jb <= n; jb += D) {
#pragma unroll
      for (int q = 0; q < D; ++q) {
        const int j = jb + q;
        if (j <= n) {
          const dfloat hx = bx[q], hy = by[q], hz1 = bz[q];
          const double ib = bi[q];
          load(j + D, bx[q], by[q], bz[q], bi[q]);
          double u;
          if (j <= nz) {
            const dfloat sxy = k_x * hx + k_y * hy;
            const dfloat dh = (hz1 - hz0) * idzf;
            const double r = cvt<double>(part == 0 ? dh - sxy : sxy + dh);
            hz0 = hz1;
            u = (r - idz2 * up) * ib;
          } else {
            const C2 tp = top[t];
            const double r = -(part == 0 ? tp.x : tp.y) * dz;
            u = (r + up) * ib;
          }
          if (j < n) st_park(P, (size_t)(j - 1) * NK + t, part, u);
          else st1(P, (size_t)(j - 1) * NK + t, part, u);  // level n: final (the back sweep starts below it)
          up = u;
        }
      }
    }
    // back substitution, level j's gamma and parked forward value in slot (n-1-j) % 4
    double bg[D], bp[D];
    auto loadb = [&](int j, double& g, double& pv) {
      if (j >= 1) {
        g = gam[(size_t)j * NK + t];
        pv = ld_park(P, (size_t)(j - 1) * NK + t, part);
      }
    };
#pragma unroll
    for (int q = 0; q < D; ++q) loadb(n - 1 - q, bg[q], bp[q]);
    for (int jb = n - 1; jb >= 1; jb -= D) {
#pragma unroll
      for (int q = 0; q < D; ++q) {
        const int j = jb - q;
        if (j >= 1) {
          const double gm = bg[q], pv = bp[q];
          loadb(j - D, bg[q], bp[q]);
          const double u = pv - gm * up;
          st1(P, (size_t)(j - 1) * NK + t, part, u);
          up = u;
        }
      }
    }
    return;
  } else {
    const double k_x = kx[t], k_y = ky[t];
    const double idz2 = 1.0 / (dz * dz);
    st1(P, t, part, up);
    double hz0 = ld1<HC>(Hz, t, part);
    // level j's inputs in ring slot (j - 2) % 4, loaded four levels ahead
    double bx[D], by[D], bz[D], bi[D];
    auto load = [&](int j, double& x, double& y, double& z, double& ib) {
      if (j <= n) ib = ibet[(size_t)(j - 1) * NK + t];
      if (j <= nz) {
        x = ld1<HC>(Hx, (size_t)(j - 2) * NK + t, ch);
        y = ld1<HC>(Hy, (size_t)(j - 2) * NK + t, ch);
      }
      z = (j <= nz - 1) ? ld1<HC>(Hz, (size_t)(j - 1) * NK + t, part) : 0.0;
    };
#pragma unroll
    for (int q = 0; q < D; ++q) load(2 + q, bx[q], by[q], bz[q], bi[q]);
    for (int jb = 2; jb <= n; jb += D) {
#pragma unroll
      for (int q = 0; q < D; ++q) {
        const int j = jb + q;
        if (j <= n) {
          const double hx = bx[q], hy = by[q], hz1 = bz[q], ib = bi[q];
          load(j + D, bx[q], by[q], bz[q], bi[q]);
          double a, r;
          if (j <= nz) {
            a = idz2;
            const double s = k_x * hx + k_y * hy;
            const double dh = (hz1 - hz0) / dz;  // divides as the reference does
            r = part == 0 ? -s + dh : s + dh;
            hz0 = hz1;
          } else {
            a = -1.0;
            const C2 tp = top[t];
            r = -(part == 0 ? tp.x : tp.y) * dz;
          }
          const double u = (r - a * up) * ib;
          st1(P, (size_t)(j - 1) * NK + t, part, u);
          up = u;
        }
      }
    }
    // back substitution, level j's gamma and forward value in slot (n-1-j) % 4
    double bg[D], bp[D];
    auto loadb = [&](int j, double& g, double& pv) {
      if (j >= 1) {
        g = gam[(size_t)j * NK + t];
        pv = ld1<PC>(P, (size_t)(j - 1) * NK + t, part);
      }
    };
#pragma unroll
    for (int q = 0; q < D; ++q) loadb(n - 1 - q, bg[q], bp[q]);
    for (int jb = n - 1; jb >= 1; jb -= D) {
#pragma unroll
      for (int q = 0; q < D; ++q) {
        const int j = jb - q;
        if (j >= 1) {
          const double gm = bg[q], pv = bp[q];
          loadb(j - D, bg[q], bp[q]);
          const double u = pv - gm * up;
          st1(P, (size_t)(j - 1) * NK + t, part, u);
          up = u;
        }
      }
    }
  }
}

// Mixed form: press_stag_array.f90:192-264 + tridag_array.f90:41-101 as a
// chunked Thomas solve, the batched hybrid for many short-latency systems:
// the z-recurrences of 16 modes (32 systems: real and imaginary parts; a, b,
// c are real) run per CTA, each of the eight warps on one chunk of about n/8
// rows, lane = system.
//   forward   d_j = al_j d_{j-1} + ib_j r_j  (al_j = -a_j ib_j): each warp
//             runs its chunk from d = 0 and keeps the chunk product
//             A_j = al_s .. al_j; the true d_j = d~_j + A_j D_(chunk-1), with
//             the chunk-end values D passed up the 8 chunks by one warp
//             (the reduced system of the chunk boundaries);
//   backward  x_j = d_j - g_(j+1) x_(j+1): the same from the top chunk down.
// Rows stay in shared memory (66 KB of d / x and 33 KB of chunk products per
// CTA); global memory sees each right-hand-side input, table entry and
// p-hat value once, in 256-byte warp accesses, each warp keeping the loads
// of its next four rows in flight.  The recurrences of the general modes
// run in float-float with the FP64 Thomas tables rounded to float-float.
// Modes with kx^2 + ky^2 <= 4 (near-singular, nearly Neumann systems) run
// the same chunked solve in FP64 in the grid's first CTA, which also
// integrates the kx = ky = 0 mode directly (press_stag_array.f90:238-247,
// a prefix sum over the levels, by one warp); the Nyquist modes are zeroed
// (press_stag_array.f90:263-264).
constexpr int TRI_M = 16, TRI_W = 8, TRI_D = 4;
constexpr int TRI_K2LOW = 4;  // modes with kx^2 + ky^2 <= 4 (integer indices) stay FP64
__device__ __forceinline__ dfloat ldff(const float2* p, size_t i) {
  const float2 v = p[i];
  return dfloat(v.x, v.y);
}
struct TriArgs {
  const float *Hx, *Hy, *Hz;         // float-float complex spectra (4 floats per mode)
  const C2 *bot, *top;               // wall and lid planes (FP64)
  float* P;                          // p-hat, float-float complex
  const float2 *ibd, *gad, *kxd, *kyd;  // float-float tables
  const double *ib, *gm, *kx, *ky;   // FP64 tables
  const int* low;                    // the FP64 modes
  int nlow, nk, lh, ny, nz;
  float2 idz2, a2, dz2;
  double dz;
};
template <typename R> __device__ __forceinline__ R tri_h(const float* H, size_t e, int cmp) {
  const float2 v = *reinterpret_cast<const float2*>(H + 4 * e + 2 * cmp);
  if constexpr (std::is_same<R, dfloat>::value) return dfloat(v.x, v.y);
  else return cvt<double>(dfloat(v.x, v.y));
}
template <typename R> __device__ __forceinline__ R tri_tab(const float2* f, const double* d, size_t i) {
  if constexpr (std::is_same<R, dfloat>::value) return ldff(f, i);
  else return d[i];
}
template <typename R> __device__ __forceinline__ R tri_cst(float2 f, double d) {
  if constexpr (std::is_same<R, dfloat>::value) return dfloat(f.x, f.y);
  else return d;
}
template <typename R> __device__ __forceinline__ R tri_of(double x) {
  if constexpr (std::is_same<R, dfloat>::value) return cvt<dfloat>(x);
  else return x;
}
__device__ __forceinline__ float2 tri_ff(dfloat v) { return make_float2(v.hi, v.lo); }
__device__ __forceinline__ float2 tri_ff(double v) {
  const dfloat d = cvt<dfloat>(v);
  return make_float2(d.hi, d.lo);
}
// One CTA's 32 systems: lane = 2 * (mode slot) + component; mode t, `act`
// false for lanes without a system; `wr` lanes store their p-hat rows
// (zero where not act).  Called by every thread of the CTA.
template <typename R>
__device__ __forceinline__ void tri_chunk(const TriArgs& A, int t, bool act, bool wr, unsigned char* smraw) {
  const int nz = A.nz, n = nz + 1;
  R* D = reinterpret_cast<R*>(smraw);            // (n + 1) x 32: d~, d, then x~, x
  R* Pr = D + (size_t)(n + 1) * 32;              // (n + 1) x 16: chunk products
  R* ce = Pr + (size_t)(n + 1) * TRI_M;          // TRI_W x 32: chunk-end d~ / chunk-start x~
  R* cp = ce + TRI_W * 32;                       // TRI_W x 32: their chunk products
  R* cc = cp + TRI_W * 32;                       // TRI_W x 32: carries into each chunk
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m = lane >> 1, comp = lane & 1;
  const size_t NK = (size_t)A.nk;
  const int L = (n + TRI_W - 1) / TRI_W;
  const int s0 = 1 + warp * L, e0 = min(n, (warp + 1) * L);  // rows of this warp's chunk (may be empty)
  const R zero = tri_cst<R>(make_float2(0.f, 0.f), 0.0), one = tri_cst<R>(make_float2(1.f, 0.f), 1.0);
  const R idz = tri_cst<R>(A.idz2, 1.0 / A.dz), a = tri_cst<R>(A.a2, 1.0 / (A.dz * A.dz));
  const R dz = tri_cst<R>(A.dz2, A.dz);
  const int ch = comp == 0 ? 1 : 0;  // component of Hx, Hy feeding this system
  const bool run = act && s0 <= e0;
  // ---- forward, local to the chunk; row j's inputs in ring slot (j - s0) % TRI_D
  R d = zero, Ap = one;
  if (run) {
    const R k_x = tri_tab<R>(A.kxd, A.kx, t), k_y = tri_tab<R>(A.kyd, A.ky, t);
    R hz0 = zero;
    if (s0 >= 2 && s0 <= nz) hz0 = tri_h<R>(A.Hz, (size_t)(s0 - 2) * NK + t, comp);  // Hz of row s0 - 1
    R bx[TRI_D], by[TRI_D], bz[TRI_D], bi[TRI_D];
    auto load = [&](int j, R& x, R& y, R& z, R& ib) {
      if (j > e0) return;
      ib = tri_tab<R>(A.ibd, A.ib, (size_t)(j - 1) * NK + t);
      if (j >= 2 && j <= nz) {
        x = tri_h<R>(A.Hx, (size_t)(j - 2) * NK + t, ch);
        y = tri_h<R>(A.Hy, (size_t)(j - 2) * NK + t, ch);
        z = (j <= nz - 1) ? tri_h<R>(A.Hz, (size_t)(j - 1) * NK + t, comp) : zero;
      }
    };
#pragma unroll
    for (int q = 0; q < TRI_D; ++q) {
      bx[q] = zero; by[q] = zero; bz[q] = zero; bi[q] = zero;
      load(s0 + q, bx[q], by[q], bz[q], bi[q]);
    }
    for (int jb = s0; jb <= e0; jb += TRI_D) {
#pragma unroll
      for (int q = 0; q < TRI_D; ++q) {
        const int j = jb + q;
        if (j <= e0) {
          const R hx = bx[q], hy = by[q], hz1 = bz[q], ib = bi[q];
          load(j + TRI_D, bx[q], by[q], bz[q], bi[q]);
          R r, al;
          if (j == 1) {
            const C2 b1 = A.bot[t];
            r = -(dz * tri_of<R>(comp == 0 ? b1.x : b1.y));
            al = zero;
            hz0 = tri_h<R>(A.Hz, t, comp);
          } else if (j <= nz) {
            const R sxy = k_x * hx + k_y * hy;
            const R dh = (hz1 - hz0) * idz;
            r = comp == 0 ? dh - sxy : sxy + dh;
            hz0 = hz1;
            al = -(a * ib);
          } else {  // row n: a = -1, r = -dz top
            const C2 tp = A.top[t];
            r = -(dz * tri_of<R>(comp == 0 ? tp.x : tp.y));
            al = ib;
          }
          d = al * d + ib * r;
          Ap = al * Ap;
          D[(size_t)j * 32 + lane] = d;
          if (comp == 0) Pr[(size_t)j * TRI_M + m] = Ap;
        }
      }
    }
  }
  ce[warp * 32 + lane] = d;
  cp[warp * 32 + lane] = Ap;
  __syncthreads();
  if (warp == 0) {  // chunk boundaries: D_w = d~_end(w) + A_end(w) D_(w-1)
    R Dw = ce[lane];
    cc[lane] = zero;
    for (int w = 1; w < TRI_W; ++w) {
      cc[w * 32 + lane] = Dw;
      Dw = ce[w * 32 + lane] + cp[w * 32 + lane] * Dw;
    }
  }
  __syncthreads();
  // ---- fix-up of d, then backward, local to the chunk
  R x = zero, Bp = one;
  if (run && warp > 0) {
    const R Din = cc[warp * 32 + lane];
    for (int j = s0; j <= e0; ++j) {
      const size_t q = (size_t)j * 32 + lane;
      D[q] = D[q] + Pr[(size_t)j * TRI_M + m] * Din;
    }
  }
  __syncwarp();  // (every lane) the fix-up has read Pr before the backward products replace it
  if (run) {
    R bg[TRI_D];
    auto loadg = [&](int j, R& g) {
      if (j >= s0 && j < n) g = tri_tab<R>(A.gad, A.gm, (size_t)j * NK + t);  // g_(j+1)
    };
#pragma unroll
    for (int q = 0; q < TRI_D; ++q) {
      bg[q] = zero;
      loadg(e0 - q, bg[q]);
    }
    for (int jb = e0; jb >= s0; jb -= TRI_D) {
#pragma unroll
      for (int q = 0; q < TRI_D; ++q) {
        const int j = jb - q;
        if (j >= s0) {
          const R gm = (j < n) ? bg[q] : zero;
          loadg(j - TRI_D, bg[q]);
          const size_t qq = (size_t)j * 32 + lane;
          x = D[qq] - gm * x;
          Bp = (j < n) ? -(gm * Bp) : zero;  // B_j; the top row has no carry from above
          D[qq] = x;
          if (comp == 0) Pr[(size_t)j * TRI_M + m] = Bp;
        }
      }
    }
  }
  ce[warp * 32 + lane] = x;
  cp[warp * 32 + lane] = Bp;
  __syncthreads();
  if (warp == 0) {  // from the top chunk down: X_w = x~_start(w) + B_start(w) X_(w+1)
    R Xw = zero;
    for (int w = TRI_W - 1; w >= 0; --w) {
      cc[w * 32 + lane] = Xw;
      Xw = ce[w * 32 + lane] + cp[w * 32 + lane] * Xw;
    }
  }
  __syncthreads();
  if (!wr || s0 > e0) return;
  const R Xin = cc[warp * 32 + lane];
  for (int j = s0; j <= e0; ++j) {
    R v = zero;
    if (act) v = D[(size_t)j * 32 + lane] + Pr[(size_t)j * TRI_M + m] * Xin;
    *reinterpret_cast<float2*>(A.P + 4 * ((size_t)(j - 1) * NK + t) + 2 * comp) = tri_ff(v);
  }
}
// grid 1 + ceil(nk / 16): CTA 0 the FP64 modes, CTA b > 0 the modes
// 16 (b - 1) .. 16 b - 1 in float-float (skipping the FP64 ones)
__global__ void __launch_bounds__(TRI_W * 32) k_tridiag_chunk(TriArgs A, int k2low) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31;
  if (blockIdx.x == 0) {
    const int s = lane >> 1;
    const int t = s < A.nlow ? A.low[s] : 0;
    const bool act = s < A.nlow && t != 0;
    tri_chunk<double>(A, t, act, act, smraw);
    if (threadIdx.x >= 32) return;
    // kx = ky = 0: p(0) = 0, p(1) = -dz bottom, p(jz) = p(jz-1) + dz Hz(jz) for
    // jz = 2..nz (Hz = 0 at jz = nz); each lane sums a run of levels, then a
    // warp scan of the run sums
    const int nz = A.nz, cnt = nz - 1;
    const int per = (cnt + 31) / 32;
    const int j0 = 2 + lane * per, j1 = min(nz, j0 + per - 1);
    const C2 b = A.bot[0];
    const double p1x = -A.dz * b.x, p1y = -A.dz * b.y;
    double sx = 0.0, sy = 0.0;
    for (int jz = j0; jz <= j1; ++jz) {
      if (jz <= nz - 1) {
        sx += tri_h<double>(A.Hz, (size_t)(jz - 1) * A.nk, 0) * A.dz;
        sy += tri_h<double>(A.Hz, (size_t)(jz - 1) * A.nk, 1) * A.dz;
      }
    }
    double ix = sx, iy = sy;  // inclusive scan over lanes
    for (int o = 1; o < 32; o <<= 1) {
      const double ux = __shfl_up_sync(0xffffffffu, ix, o), uy = __shfl_up_sync(0xffffffffu, iy, o);
      if (lane >= o) { ix += ux; iy += uy; }
    }
    double px = p1x + (ix - sx), py = p1y + (iy - sy);
    float2* P2 = reinterpret_cast<float2*>(A.P);
    if (lane == 0) {
      P2[0] = make_float2(0.f, 0.f); P2[1] = make_float2(0.f, 0.f);
      P2[2 * (size_t)A.nk] = tri_ff(p1x); P2[2 * (size_t)A.nk + 1] = tri_ff(p1y);
    }
    for (int jz = j0; jz <= j1; ++jz) {
      if (jz <= nz - 1) {
        px += tri_h<double>(A.Hz, (size_t)(jz - 1) * A.nk, 0) * A.dz;
        py += tri_h<double>(A.Hz, (size_t)(jz - 1) * A.nk, 1) * A.dz;
      }
      P2[2 * (size_t)jz * A.nk] = tri_ff(px);
      P2[2 * (size_t)jz * A.nk + 1] = tri_ff(py);
    }
    return;
  }
  const int t = (blockIdx.x - 1) * TRI_M + (lane >> 1);
  const int jx = t % A.lh, jy = t / A.lh;
  const bool inb = t < A.nk;
  const bool nyq = inb && (jy == A.ny / 2 || jx == A.lh - 1);
  const int my = jy <= A.ny / 2 ? jy : jy - A.ny;  // wrapped ky index
  const bool low = inb && !nyq && jx * jx + my * my <= k2low;  // includes (0,0): CTA 0 solves them
  tri_chunk<dfloat>(A, inb ? t : 0, inb && !nyq && !low, inb && !low, smraw);
}

// Thomas coefficients of press_stag_array.f90:144-210 for every (kx,ky):
// they depend on k^2 and dz only, so they are formed once per context
// (tridag_array.f90:41-69 recurrences, reciprocal of bet stored).
int thomas_tables(les_ctx* c) {
  const Grid& g = c->g;
  const int nz = g.nz, n = nz + 1, lh = g.lh, ny = g.ny;
  const size_t NK = (size_t)lh * ny;
  std::vector<double> kx(NK), ky(NK), ib(NK * n, 0.0), gm(NK * n, 0.0);
  cudaMemcpy(kx.data(), c->kx, NK * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(ky.data(), c->ky, NK * sizeof(double), cudaMemcpyDeviceToHost);
  const double dz = g.dz, idz2 = 1.0 / (dz * dz);
  for (size_t t = 0; t < NK; ++t) {
    const int jx = (int)(t % lh), jy = (int)(t / lh);
    double bet = -1.0;
    ib[t] = 1.0 / bet;
    // modes tridag_array skips: kx = ky = 0 and the Nyquist row / column
    if (t == 0 || jy == ny / 2 || jx == lh - 1) continue;
    const double bmid = -(kx[t] * kx[t] + ky[t] * ky[t] + 2.0 / (dz * dz));
    double cprev = 1.0;
    for (int j = 2; j <= n; ++j) {
      const double a = (j <= nz) ? idz2 : -1.0;
      const double b = (j <= nz) ? bmid : 1.0;
      const double gg = cprev / bet;
      gm[(size_t)(j - 1) * NK + t] = gg;
      bet = b - a * gg;
      if (bet == 0.0) {  // tridag_array.f90:62-67 stops here
        les_set_error("tridag_array failed at mode %zu, row %d: zero pivot", t, j);
        return LES_ERR_PIVOT;
      }
      ib[(size_t)(j - 1) * NK + t] = 1.0 / bet;
      cprev = (j <= nz) ? idz2 : 0.0;
    }
  }
  LES_CUDA_CHECK(cudaMemcpy(c->ibet, ib.data(), ib.size() * sizeof(double), cudaMemcpyHostToDevice));
  LES_CUDA_CHECK(cudaMemcpy(c->gamt, gm.data(), gm.size() * sizeof(double), cudaMemcpyHostToDevice));
  if (c->ibet_ff) {  // the mixed form's chunked solve: the same tables as float-float pairs, and the
                     // list of the modes it leaves to the FP64 solve
    std::vector<float2> f2(ib.size());
    auto ff = [](double v) { const float h = (float)v; return make_float2(h, (float)(v - (double)h)); };
    for (size_t i = 0; i < ib.size(); ++i) f2[i] = ff(ib[i]);
    LES_CUDA_CHECK(cudaMemcpy(c->ibet_ff, f2.data(), f2.size() * sizeof(float2), cudaMemcpyHostToDevice));
    for (size_t i = 0; i < gm.size(); ++i) f2[i] = ff(gm[i]);
    LES_CUDA_CHECK(cudaMemcpy(c->gamt_ff, f2.data(), f2.size() * sizeof(float2), cudaMemcpyHostToDevice));
    std::vector<int> low;
    for (size_t t = 0; t < NK; ++t) {
      const int jx = (int)(t % lh), jy = (int)(t / lh);
      if (jy == ny / 2 || jx == lh - 1) continue;
      const int my = jy <= ny / 2 ? jy : jy - ny;
      if (jx * jx + my * my <= TRI_K2LOW) low.push_back((int)t);
    }
    if ((int)low.size() > c->nlow_cap) { les_set_error("low-mode list overflow"); return LES_ERR_STATE; }
    LES_CUDA_CHECK(cudaMemcpy(c->lowmodes, low.data(), low.size() * sizeof(int), cudaMemcpyHostToDevice));
    c->nlow = (int)low.size();
  }
  return 0;
}

// T: transform precision of the three field transforms and the spectra H,
// p-hat (double: FP64 form and the per-routine entry; dfloat: mixed form).
// The wall planes' spectra and the tridiagonal solve are FP64 in both.
template <typename T>
static int pressT(les_ctx* c, double* p, double* dpdx, double* dpdy, const float2* const* ustar = nullptr) {
  typedef typename CT<T>::type CX;
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  const int nz = g.nz;
  const double cst = 1.0 / (double)(g.nx * g.ny);
  // spectra of u*, v*, w* (levels 1..nz-1), (const/tadv1)*(u/dt); u* is the
  // state itself, or (mixed form) the separate float-float predictor fields
  const double sc3[3] = {cst / 1.5, cst / 1.5, cst / 1.5};
  const double dv3[3] = {k.dt, k.dt, k.dt};
  if (ustar) {
    if constexpr (std::is_same<T, dfloat>::value) {
      const dfloat* in[3] = {reinterpret_cast<const dfloat*>(ustar[0]), reinterpret_cast<const dfloat*>(ustar[1]),
                             reinterpret_cast<const dfloat*>(ustar[2])};
      r2cT<T, dfloat>(c, 3, nz - 1, in, (long)g.nplane, sc3, dv3, c->wsA, false, g.lh);
    } else {
      les_set_error("float-float predictor fields need float-float transforms");
      return LES_ERR_STATE;
    }
  } else {
    const double* in[3] = {c->f[LES_U], c->f[LES_V], c->f[LES_W]};
    r2cT<T, double>(c, 3, nz - 1, in, (long)g.nplane, sc3, dv3, c->wsA, false, g.lh);
  }
  CX* H = (CX*)c->wsP;                                       // 3*(nz-1)*C
  C2* BT = reinterpret_cast<C2*>(H + (size_t)3 * (nz - 1) * g.C);  // bottom, top
  // p-hat in the transform precision (float-float in the mixed form)
  typedef CX PCX;
  PCX* P = reinterpret_cast<PCX*>(BT + 2 * g.C);            // (nz+1)*C
  ColJob J = coljob(c, MAP_SAME, DIR_FWD, nz - 1);
  J.nin = 1; J.nout = 1; J.nf = 3;
  J.in[0] = c->wsA; J.fs_in = (long)(nz - 1) * g.C;
  J.out[0] = H; J.fs_out = (long)(nz - 1) * g.C;
  J.coef[0][0] = CC_KILL;
  colsT<T, CX>(c, J);
  // bottomw, topw from divtz(1), divtz(nz) scaled by 1/(nx*ny)
  {
    const double* bi[2] = {c->f[LES_DIVTZ], c->f[LES_DIVTZ] + (size_t)(nz - 1) * g.nplane};
    const double sc2[2] = {cst, cst};
    r2c(c, 2, 1, bi, (long)g.nplane, sc2, nullptr, (C2*)c->wsA, false, g.lh);
    ColJob K = coljob(c, MAP_SAME, DIR_FWD, 1);
    K.nin = 1; K.nout = 1; K.nf = 2;
    K.in[0] = c->wsA; K.fs_in = (long)g.C;
    K.out[0] = BT; K.fs_out = (long)g.C;
    K.coef[0][0] = CC_KILL;
    cols(c, K);
  }
  const CX* Hx = H;
  const CX* Hy = H + (size_t)(nz - 1) * g.C;
  const CX* Hz = H + (size_t)2 * (nz - 1) * g.C;
  if constexpr (std::is_same<T, dfloat>::value) {
    // chunked float-float Thomas for |k|^2 > TRI_K2LOW, chunked FP64 Thomas for the rest
    const size_t sm = ((size_t)(nz + 2) * (32 + TRI_M) + 3 * TRI_W * 32) * sizeof(dfloat);
    if (sm > 227 * 1024) {
      les_set_error("pressure solve: %d levels exceed the shared-memory row buffer", nz);
      return LES_ERR_UNSUPPORTED;
    }
    static size_t sm_set = 48 * 1024;
    if (sm > sm_set) {
      LES_CUDA_CHECK(cudaFuncSetAttribute(k_tridiag_chunk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      sm_set = sm;
    }
    if (c->nlow > TRI_M) { les_set_error("too many FP64 pressure modes (%d)", c->nlow); return LES_ERR_STATE; }
    const dfloat idz(1.0 / g.dz), a2(1.0 / (g.dz * g.dz)), dz2(g.dz);
    TriArgs A;
    A.Hx = reinterpret_cast<const float*>(Hx);
    A.Hy = reinterpret_cast<const float*>(Hy);
    A.Hz = reinterpret_cast<const float*>(Hz);
    A.bot = BT; A.top = BT + g.C;
    A.P = reinterpret_cast<float*>(P);
    A.ibd = c->ibet_ff; A.gad = c->gamt_ff; A.kxd = c->kxd; A.kyd = c->kyd;
    A.ib = c->ibet; A.gm = c->gamt; A.kx = c->kx; A.ky = c->ky;
    A.low = c->lowmodes; A.nlow = c->nlow;
    A.nk = g.lh * g.ny; A.lh = g.lh; A.ny = g.ny; A.nz = nz;
    A.idz2 = make_float2(idz.hi, idz.lo); A.a2 = make_float2(a2.hi, a2.lo); A.dz2 = make_float2(dz2.hi, dz2.lo);
    A.dz = g.dz;
    k_tridiag_chunk<<<1 + (g.lh * g.ny + TRI_M - 1) / TRI_M, TRI_W * 32, sm, c->stream>>>(A, TRI_K2LOW);
    LES_COUNT_LAUNCH();
  } else {
    k_tridiag2<CX, PCX><<<(2 * g.lh * g.ny + 127) / 128, 128, 0, c->stream>>>(
        Hx, Hy, Hz, BT, BT + g.C, P, c->ibet, c->gamt, c->kx, c->ky, c->kxd, c->kyd, g.lh, g.ny, nz, g.dz,
        nullptr, 0); LES_COUNT_LAUNCH();
  }
  // p level 0 ; levels 1..nz-1 : p, dpdx, dpdy.  p-hat's y round trip for
  // levels 0..nz-1 and i ky's for 1..nz-1; dp/dx by the x wavenumber alone
  // on the inverse y transform (p-hat's Nyquist modes are zero,
  // press_stag_array.f90:263-264, so the y round trip that ddx makes adds
  // nothing)
  {
    ColJob K = coljob(c, MAP_SAME, DIR_INV, nz);
    K.nin = 1; K.nout = 1; K.in[0] = P; K.out[0] = c->wsB; K.coef[0][0] = CC_ONE;
    colsT<T, PCX>(c, K);
    const size_t L1 = (size_t)(nz - 1) * g.C;
    CX* Y = (CX*)c->wsB;
    CX* Yx = Y + (size_t)nz * g.C;
    CX* Yy = Yx + L1;
    ColJob L = coljob(c, MAP_SAME, DIR_INV, nz - 1);
    L.nin = 1; L.nout = 1; L.in[0] = P + g.C; L.out[0] = Yy; L.coef[0][0] = CC_IKY;
    colsT<T, PCX>(c, L);
    k_ikx_rows<CX><<<grid1(L1), 256, 0, c->stream>>>(Y + g.C, Yx, c->kxd, c->kx, g.lh, L1, 0); LES_COUNT_LAUNCH();
    double* o0 = p;
    c2rT<T, double>(c, 1, nz, Y, &o0, (long)g.nplane, false, g.lh);
    double* o1[2] = {dpdx, dpdy};
    c2rT<T, double>(c, 2, nz - 1, Yx, o1, (long)g.nplane, false, g.lh);
  }
  fill(c, dpdx + (size_t)(nz - 1) * g.nplane, g.nplane, LES_BOGUS);
  fill(c, dpdy + (size_t)(nz - 1) * g.nplane, g.nplane, LES_BOGUS);
  fill(c, p + (size_t)nz * g.nplane, g.nplane, LES_BOGUS);
  return 0;
}
int op_press(les_ctx* c, double* p, double* dpdx, double* dpdy) { return pressT<double>(c, p, dpdx, dpdy); }

// tridag_array.f90:1-109 with caller-supplied coefficients (per-routine entry)
__global__ void k_tridag_generic(const double* a, const double* b, const double* cc, const C2* r, C2* u,
                                 double* gam, int lh, int ny, int n, int* flag) {
  const int nk = lh * ny;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nk) return;
  const int jx = t % lh, jy = t / lh;
  const size_t NK = (size_t)nk;
  double bet = b[t];
  C2 up; up.x = r[t].x / bet; up.y = r[t].y / bet;
  u[t] = up;
  if (jy == ny / 2 || jx == lh - 1 || t == 0) return;
  for (int j = 2; j <= n; ++j) {
    const size_t o = (size_t)(j - 1) * NK + t;
    const double gm = cc[o - NK] / bet;
    gam[o] = gm;
    bet = b[o] - a[o] * gm;
    if (bet == 0.0) atomicOr(flag, 1);
    C2 x; x.x = (r[o].x - a[o] * up.x) / bet; x.y = (r[o].y - a[o] * up.y) / bet;
    u[o] = x;
    up = x;
  }
  for (int j = n - 1; j >= 1; --j) {
    const size_t o = (size_t)(j - 1) * NK + t;
    const double gm = gam[o + NK];
    C2 x = u[o];
    x.x = x.x - gm * up.x; x.y = x.y - gm * up.y;
    u[o] = x;
    up = x;
  }
}
int op_tridag(les_ctx* c, const double* a, const double* b, const double* cc, const double* r, double* u) {
  const Grid& g = c->g;
  int* flag = reinterpret_cast<int*>(c->dscal + 8);
  double* gam = (double*)c->wsA;
  k_tridag_generic<<<(g.lh * g.ny + 127) / 128, 128, 0, c->stream>>>(a, b, cc, (const C2*)r, (C2*)u, gam, g.lh, g.ny,
                                                                    g.nz + 1, flag); LES_COUNT_LAUNCH();
  return 0;
}
// The same kernel with caller-supplied scratch (gam: lh*ny*n doubles, flag: one int).
void launch_tridag_generic(const double* a, const double* b, const double* cc, const double* r, double* u,
                           double* gam, int lh, int ny, int n, int* flag, cudaStream_t s) {
  k_tridag_generic<<<(lh * ny + 127) / 128, 128, 0, s>>>(a, b, cc, (const C2*)r, (C2*)u, gam, lh, ny, n, flag);
  LES_COUNT_LAUNCH();
}

// ---------------------------------------------------------------------------
// scalars_module.f90:254-283 surface flux and dsdz(1)
__global__ void k_sflux(const double* __restrict__ theta, const double* __restrict__ wt_s,
                        const double* __restrict__ phi_h, const double* __restrict__ ustar, double* dTdz,
                        double* sgs_t3, int nx, int ny, int ld, double tsus, double vonk, double dz) {
  GSTRIDE(s, (size_t)nx * ny) {
    const int jy = (int)(s / nx), jx = (int)(s - (size_t)jy * nx);
    const double sf = (theta[0] < 2.0) ? wt_s[s] / tsus : 0.0;
    dTdz[(size_t)jy * ld + jx] = -phi_h[s] * sf / (ustar[s] * vonk * dz / 2.0);
    sgs_t3[s] = sf;
  }
}
// scalars_module.f90:321-346 advection product on the 3/2 grid
// uvm: per-level plane-mean wind (U, V) added back to um, vm (the mixed form
// pads the fluctuations u', v'), or null
template <typename S>
__global__ void k_scalar_prod(const S* __restrict__ um, const S* __restrict__ vm,
                              const S* __restrict__ wm, const S* __restrict__ sx,
                              const S* __restrict__ sy, const S* __restrict__ sz, S* R, int ldb,
                              int nx2, int ny2, int nz, const float2* __restrict__ uvm) {
  const size_t np = (size_t)ldb * ny2;
  GSTRIDE(i, np * nz) {
    const int jz = (int)(i / np) + 1;
    const int jx = (int)((i - (size_t)(jz - 1) * np) % ldb);
    if (jx >= nx2) continue;
    S uu = um[i], vv = vm[i];
    if (uvm) {
      const float2 m = uvm[jz];
      uu += (S)m.x;
      vv += (S)m.y;
    }
    if (jz == 1) R[i] = uu * sx[i] + vv * sy[i] + ((S)0.5 * wm[i + np]) * sz[i + np];
    else if (jz == nz) R[i] = uu * sx[i] + vv * sy[i];
    else R[i] = uu * sx[i] + vv * sy[i] + (wm[i] * sz[i] + wm[i + np] * sz[i + np]) / (S)2;
  }
}
// scalars_module.f90:77-82 Pr_: the constant Pr, or the field Pr_t of
// model 7 when prt is not null
__device__ __forceinline__ double pr_at(const double* __restrict__ prt, double pr, size_t i) {
  return prt ? prt[i] : pr;
}
// scalars_module.f90:364-407 horizontal SGS fluxes
template <typename NT>
__global__ void k_scalar_temp_xy(const NT* __restrict__ nut, const double* __restrict__ dsx,
                                 const double* __restrict__ dsy, double* tx, double* ty, int ld, int nx, int ny,
                                 int nz, double pr, const double* __restrict__ prt) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * nz) {
    const int jz = (int)(i / np) + 1;
    const int jx = (int)((i - (size_t)(jz - 1) * np) % ld);
    if (jx >= nx) continue;
    if (jz == nz) { tx[i] = 0.0; ty[i] = 0.0; continue; }
    const double nu = cvt<double, NT>(nut[i]);
    if (jz == 1) {
      const double p1 = pr_at(prt, pr, i);
      tx[i] = (1.0 / p1) * nu * dsx[i];
      ty[i] = (1.0 / p1) * nu * dsy[i];
    } else {
      const double f = (1.0 / (0.5 * (pr_at(prt, pr, i) + pr_at(prt, pr, i + np)))) * 0.5 *
                       (nu + cvt<double, NT>(nut[i + np]));
      tx[i] = f * dsx[i];
      ty[i] = f * dsy[i];
    }
  }
}
// scalars_module.f90:385-452 RHS assembly with the SGS divergence
template <typename NT>
__global__ void k_scalar_rhs(double* R, const double* __restrict__ dxy, const NT* __restrict__ nut,
                             const double* __restrict__ dsz, const double* __restrict__ sgs_t3, int ld, int nx,
                             int ny, int nz, double pr, const double* __restrict__ prt, double cdz) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * (nz - 1)) {
    const int jz = (int)(i / np) + 1;
    const size_t r = i - (size_t)(jz - 1) * np;
    const int jx = (int)(r % ld);
    if (jx >= nx) continue;
    const int jy = (int)(r / ld);
    // temp(k) = Nu_t dsdz / Pr on w-nodes, temp(1) = -surf_flux
    const double t0 = (jz == 1) ? -1.0 * sgs_t3[(size_t)jy * nx + jx]
                                : (1.0 / pr_at(prt, pr, i)) * cvt<double, NT>(nut[i]) * dsz[i];
    const double t1 = (1.0 / pr_at(prt, pr, i + np)) * cvt<double, NT>(nut[i + np]) * dsz[i + np];
    R[i] = (-1.0 * R[i] + dxy[i]) + cdz * (t1 - t0);
  }
}
// scalars_module.f90:175-228 calcbeta from per-level plane sums
// per level: sb = plane mean of theta, 1/sb (the divisions once per level)
// Mixed form: the same from FP32 inputs (the horizontal divergences h from
// FP32 transforms, the FP32-held tau) in FP32 arithmetic, the FP64 outputs
// widened exactly.  grid (ceil(np/256), nz).
__global__ void __launch_bounds__(256) k_divstress_fin32(double* __restrict__ divx, double* __restrict__ divy,
                                                         double* __restrict__ divz, const float* __restrict__ hx,
                                                         const float* __restrict__ hy,
                                                         const float* __restrict__ hz,
                                                         const float* __restrict__ txz,
                                                         const float* __restrict__ tyz,
                                                         const float* __restrict__ tzz, int ld, int nx, int ny,
                                                         int nz, float cdz) {
  const unsigned np = (unsigned)ld * ny;
  const unsigned r = blockIdx.x * 256u + threadIdx.x;
  if (r >= np) return;
  const int jz = blockIdx.y + 1;
  const size_t i = (size_t)(jz - 1) * np + r;
  const bool inx = (int)(r % (unsigned)ld) < nx;
  if (jz == nz) {
    divx[i] = LES_BOGUS;
    divy[i] = LES_BOGUS;
    divz[i] = inx ? cvt_f2d(hz[i]) : 0.0;
    return;
  }
  if (!inx) { divx[i] = 0.0; divy[i] = 0.0; divz[i] = 0.0; return; }
  divx[i] = cvt_f2d(hx[i] + cdz * (txz[i + np] - txz[i]));
  divy[i] = cvt_f2d(hy[i] + cdz * (tyz[i + np] - tyz[i]));
  divz[i] = cvt_f2d((jz == 1) ? hz[i] : hz[i] + cdz * (tzz[i] - tzz[i - np]));
}

// Mixed-form scalar flux kernels, grid (ceil(np/256), levels): FP32 inputs
// (Nu_t, the theta gradients, the advection term and the flux divergence
// come from FP32 arithmetic and transforms), FP32 arithmetic; dsz (theta
// differences, FP64) and the surface flux are read in FP64 and narrowed.
__global__ void __launch_bounds__(256) k_scalar_temp_xy32(const float* __restrict__ nut,
                                                          const float* __restrict__ dsx,
                                                          const float* __restrict__ dsy, float* tx, float* ty,
                                                          int ld, int nx, int ny, int nz, float ipr) {
  const unsigned np = (unsigned)ld * ny;
  const unsigned r = blockIdx.x * 256u + threadIdx.x;
  if (r >= np || (int)(r % (unsigned)ld) >= nx) return;
  const int jz = blockIdx.y + 1;
  const size_t i = (size_t)(jz - 1) * np + r;
  if (jz == nz) { tx[i] = 0.0f; ty[i] = 0.0f; return; }
  const float f = (jz == 1) ? ipr * nut[i] : ipr * 0.5f * (nut[i] + nut[i + np]);
  tx[i] = f * dsx[i];
  ty[i] = f * dsy[i];
}
__global__ void __launch_bounds__(256) k_scalar_rhs32(double* R, const float* __restrict__ adv,
                                                      const float* __restrict__ dxy, const float* __restrict__ nut,
                                                      const double* __restrict__ dsz,
                                                      const double* __restrict__ sgs_t3, int ld, int nx, int ny,
                                                      float ipr, float cdz) {
  const unsigned np = (unsigned)ld * ny;
  const unsigned r = blockIdx.x * 256u + threadIdx.x;
  if (r >= np) return;
  const int jy = (int)(r / (unsigned)ld), jx = (int)(r - (unsigned)jy * ld);
  if (jx >= nx) return;
  const int jz = blockIdx.y + 1;
  const size_t i = (size_t)(jz - 1) * np + r;
  const float t0 = (jz == 1) ? -cvt_d2f(sgs_t3[(size_t)jy * nx + jx]) : ipr * nut[i] * cvt_d2f(dsz[i]);
  const float t1 = ipr * nut[i + np] * cvt_d2f(dsz[i + np]);
  R[i] = cvt_f2d((-adv[i] + dxy[i]) + cdz * (t1 - t0));
}

__global__ void k_calcbeta_levels(const double* __restrict__ sums, double* sbr, int nz, double nxny, double gh) {
  for (int j = threadIdx.x; j < nz; j += blockDim.x) {
    const double sb = sums[j] / nxny;
    sbr[2 * j] = sb;
    sbr[2 * j + 1] = gh / sb;
  }
}
// grid (ceil(np/256), ceil(nz/KZ)): a thread takes KZ consecutive levels of
// one plane point, so each level's g_hat/2 (theta - sb)/sb is formed once and
// is both the 'above' term of its level and the 'below' term of the next; the
// kernel is bound by the FP64 pipe, and this takes three FP64 operations per
// point instead of six.  sbr holds sb and g_hat / (2 sb) per level.
template <int KZ>
__global__ void k_calcbeta(const double* __restrict__ theta, const double* __restrict__ sbr, double* __restrict__ bs,
                           int ld, int nx, int ny, int nz) {
  const int np = ld * ny;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= np) return;
  const int z0 = blockIdx.y * KZ;  // plane index (level - 1) of the thread's first level
  const bool inx = r % ld < nx;
  double qb = 0.0;  // g_hat/2 (theta - sb) / sb of the plane below
  if (inx && z0 > 0) qb = (theta[(size_t)(z0 - 1) * np + r] - sbr[2 * (z0 - 1)]) * sbr[2 * (z0 - 1) + 1];
#pragma unroll
  for (int k = 0; k < KZ; ++k) {
    const int p = z0 + k;
    if (p < nz) {
      const size_t i = (size_t)p * np + r;
      double qa = 0.0;
      if (inx) qa = (theta[i] - sbr[2 * p]) * sbr[2 * p + 1];
      bs[i] = (inx && p > 0 && p < nz - 1) ? qa + qb : 0.0;
      qb = qa;
    }
  }
}
// virtual potential temperature theta (1 + 0.61 * 0.001 qmix q_scale)
// (scalars_module.f90:203,221-222), padding columns zero
__global__ void k_thetav(const double* __restrict__ theta, const double* __restrict__ q, double* __restrict__ tv,
                         size_t n, int ld, int nx, double q_scale) {
  GSTRIDE(i, n) {
    tv[i] = ((int)(i % ld) < nx) ? theta[i] * (1.0 + 0.61 * 0.001 * q[i] * q_scale) : 0.0;
  }
}
// with humidity, calcbeta reads the virtual temperature of the start-of-step
// theta and qmix (q_all_in_one runs after theta_all_in_one, main.f90:273-274),
// formed in c->tmp (free at this point of the scalar step)
static void calcbeta(les_ctx* c) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  double* sbr = c->dred + 20 * (size_t)(g.nz + 8);  // 2 * nz values
  const double* th = c->f[LES_THETA];
  if (k.q_flag) {
    k_thetav<<<grid1(g.nfield), 256, 0, c->stream>>>(c->f[LES_THETA], c->f[LES_Q], c->tmp, g.nfield, g.ld, g.nx,
                                                     k.q_scale); LES_COUNT_LAUNCH();
    th = c->tmp;
  }
  plane_sums(c, th, (long)g.nplane, g.nz, 4, 1.0, c->dred);
  const double g_hat = k.g * (k.z_i / (k.u_star * k.u_star));
  k_calcbeta_levels<<<1, 256, 0, c->stream>>>(c->dred, sbr, g.nz, (double)(g.nx * g.ny), 0.5 * g_hat); LES_COUNT_LAUNCH();
  k_calcbeta<8><<<dim3((unsigned)((g.nplane + 255) / 256), (g.nz + 7) / 8), 256, 0, c->stream>>>(
      th, sbr, c->f[LES_BETA_SCAL], g.ld, g.nx, g.ny, g.nz);
  LES_COUNT_LAUNCH();
}
// One active scalar of the step: theta (scalars_module.f90:57-504) or the
// humidity qmix (scalars_module_q.f90:31-397), which share the algorithm and
// differ in their arrays, surface flux scale, lid gradient and in theta
// alone feeding the buoyancy.
struct ScalarDesc {
  int s, rhs, rhsf, dsdx, dsdy, dsdz, flux, sgs3;
  double flux_scale;  // surf_flux = flux / flux_scale  (T_scale u_star or q_scale u_star)
  double top_grad;    // dsdz(nz) (dTdz_top / T_scale z_i or dqdz_top / q_scale z_i)
  int mean_slot;      // dred slot of the mixed form's plane means
  bool buoyancy;
};
static ScalarDesc theta_desc(const les_ctx* c) {
  const les_config& k = c->cfg;
  return ScalarDesc{LES_THETA, LES_RHS_T, LES_RHS_TF, LES_DTDX, LES_DTDY, LES_DTDZ, LES_WT_S, LES_SGS_T3_SFC,
                    k.t_scale * k.u_star, k.dtdz_top / k.t_scale * k.z_i, 14, true};
}
static ScalarDesc q_desc(const les_ctx* c) {
  const les_config& k = c->cfg;
  return ScalarDesc{LES_Q, LES_RHS_Q, LES_RHS_QF, LES_DQDX, LES_DQDY, LES_DQDZ, LES_WQ_S, LES_SGS_Q3_SFC,
                    k.q_scale * k.u_star, k.dqdz_top / k.q_scale * k.z_i, 15, false};
}
// scalars_module.f90:457-504 step_scalar
// grid (ceil(np/256), nz-1): one element per thread (a column walk per
// thread serialises the levels behind the stores); the thread of level
// nz-1 also sets the top level from the value it has just written
__global__ void k_step_scalar(double* __restrict__ theta, const double* __restrict__ R,
                              const double* __restrict__ Rf, int ld, int nx, int ny, int nz, double dt,
                              int top_grad, double inc) {
  const int np = ld * ny;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= np) return;
  const int jz = blockIdx.y + 1;
  const size_t i = r + (size_t)(jz - 1) * np;
  double t = theta[i];
  if (r % ld < nx) {
    t = t + dt * (1.5 * R[i] - 0.5 * Rf[i]);
    theta[i] = t;
  }
  if (jz == nz - 1) theta[i + np] = top_grad ? t + inc : t;
}
// scalars_module.f90:57-171 theta_all_in_one / scalars_module_q.f90:31-141
// q_all_in_one (S_FLAG, lbc = 1, model 5 Pr)
static int op_scalar(les_ctx* c, const ScalarDesc& d) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  const int nz = g.nz;
  op_filt_da(c, c->f[d.s], c->f[d.dsdx], c->f[d.dsdy], nz);
  op_ddz(c, c->f[d.dsdz], c->f[d.s], 1);
  fill(c, c->f[d.dsdz] + (size_t)(nz - 1) * g.nplane, g.nplane, d.top_grad);
  // RHS_Tf = RHS_T (RHS_T is fully rewritten below)
  cudaMemcpyAsync(c->f[d.rhsf], c->f[d.rhs], g.nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  k_sflux<<<grid1((size_t)g.nx * g.ny), 256, 0, c->stream>>>(c->f[d.s], c->f[d.flux], c->f[LES_PHI_H],
                                                            c->f[LES_USTAR_AVG], c->f[d.dsdz],
                                                            c->f[d.sgs3], g.nx, g.ny, g.ld,
                                                            d.flux_scale, k.vonk, g.dz); LES_COUNT_LAUNCH();
  double* bigf[7];
  for (int q = 0; q < 7; ++q) bigf[q] = c->big + (size_t)q * g.nfield_big;
  const double* in[6] = {c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[d.dsdx], c->f[d.dsdy], c->f[d.dsdz]};
  op_dealias1(c, in, bigf, 6, nz);
  k_scalar_prod<double><<<grid1(g.nfield_big), 256, 0, c->stream>>>(bigf[0], bigf[1], bigf[2], bigf[3], bigf[4], bigf[5],
                                                           bigf[6], g.ld_big, g.nx2, g.ny2, nz, nullptr); LES_COUNT_LAUNCH();
  double* rt = c->f[d.rhs];
  const double* b6 = bigf[6];
  op_dealias2(c, &rt, &b6, 1, nz, 1.0 / (double)(g.nx2 * g.ny2));
  // horizontal SGS flux divergence (ddx + ddy summed in spectral space)
  double* tx = c->tmp;
  double* ty = c->tmp + g.nfield;
  double* dxy = c->tmp + 2 * g.nfield;
  k_scalar_temp_xy<double><<<grid1(g.nfield), 256, 0, c->stream>>>(c->f[LES_NU_T], c->f[d.dsdx], c->f[d.dsdy], tx, ty,
                                                          g.ld, g.nx, g.ny, nz, k.pr, c->f[LES_PR_T]);
  LES_COUNT_LAUNCH();
  {
    const double sc = 1.0 / (double)(g.nx * g.ny);
    const double* ii[2] = {tx, ty};
    const double s2[2] = {sc, sc};
    r2c(c, 2, nz, ii, (long)g.nplane, s2, nullptr, c->wsA, false, g.lh);
    ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nz);
    J.nin = 2; J.nout = 1; J.in[0] = c->wsA; J.in[1] = (C2*)c->wsA + (size_t)nz * g.C; J.out[0] = c->wsB;
    J.coef[0][0] = CC_IKX; J.coef[0][1] = CC_IKY;
    cols(c, J);
    c2r(c, 1, nz, c->wsB, &dxy, (long)g.nplane, false, g.lh);
  }
  k_scalar_rhs<double><<<grid1(g.nplane * (nz - 1)), 256, 0, c->stream>>>(rt, dxy, c->f[LES_NU_T], c->f[d.dsdz],
                                                                 c->f[d.sgs3], g.ld, g.nx, g.ny, nz, k.pr,
                                                                 c->f[LES_PR_T], 1.0 / g.dz); LES_COUNT_LAUNCH();
  // calcbeta on theta before the update
  if (d.buoyancy) calcbeta(c);
  if (c->jt == 1 && !k.initsc)
    cudaMemcpyAsync(c->f[d.rhsf], c->f[d.rhs], g.nfield * sizeof(double), cudaMemcpyDeviceToDevice,
                    c->stream);
  const int topg = k.lz_over_zi > 1.0 ? 1 : 0;
  k_step_scalar<<<dim3((unsigned)((g.nplane + 255) / 256), nz - 1), 256, 0, c->stream>>>(
      c->f[d.s], c->f[d.rhs], c->f[d.rhsf], g.ld, g.nx, g.ny, nz, k.dt, topg,
      d.top_grad * g.dz); LES_COUNT_LAUNCH();
  return 0;
}

int op_theta(les_ctx* c) { return op_scalar(c, theta_desc(c)); }
int op_q(les_ctx* c) { return op_scalar(c, q_desc(c)); }

// atm_thermodynamics.f90:37-52 for levels 1..nz-1, columns 1..nx
__global__ void k_thermo(const double* __restrict__ theta, const double* __restrict__ q, double* aT, double* aTv,
                         double* svp, double* pa, double* vp, double* sq, double* rh, double* rhq, double* zl,
                         int ld, int nx, int ny, int nz, double dz, double z_i, double T_scale, double q_scale,
                         double g, double cp, double Rd, double pr_surf) {
  const size_t np = (size_t)ld * ny;
  GSTRIDE(i, np * (nz - 1)) {
    if ((int)(i % ld) >= nx) continue;
    const int jz = (int)(i / np) + 1;  // k_global = jz (one domain)
    const double zg = jz * dz * z_i;
    const double T = theta[i] - (g / cp) * zg / T_scale;
    const double Tv = T * (1 + 0.61 * 0.001 * q[i] * q_scale);
    const double Tc = T * T_scale - 273.2;
    const double es = 611.2 * exp(17.62 * Tc / (243.12 + Tc));
    const double p = pr_surf * exp(-zg / (Rd * Tv * T_scale / g));
    const double qq = 0.001 * q_scale * q[i];
    const double e = (qq / (qq + 0.622)) * p;
    const double qs = 0.622 * es / (p - es);
    const double rq = qq / qs;
    aT[i] = T; aTv[i] = Tv; svp[i] = es; pa[i] = p; vp[i] = e; sq[i] = qs;
    rh[i] = e / es;
    rhq[i] = rq;
    zl[i] = zg + (cp / g) * (T * T_scale - 55 - 1.0 / (1 / (T * T_scale - 55) - log(rq) / 2840));
  }
}
int op_thermo(les_ctx* c, double* const* o) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  // param.f90:90-96
  const double cp = 1005.0, Rd = 287.04, pr_surf = 100000.0;
  k_thermo<<<grid1(g.nplane * (g.nz - 1)), 256, 0, c->stream>>>(
      c->f[LES_THETA], c->f[LES_Q], o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7], o[8], g.ld, g.nx, g.ny, g.nz,
      g.dz, k.z_i, k.t_scale, k.q_scale, k.g, cp, Rd, pr_surf); LES_COUNT_LAUNCH();
  return 0;
}

// ---------------------------------------------------------------------------
// rmsdiv.f90:93-100 (deterministic two-level sum) and timestep_conditions
__global__ void __launch_bounds__(512) k_rmsdiv_part(const double* __restrict__ du, const double* __restrict__ dv,
                                                     const double* __restrict__ dw, double* part, int ld, int nx,
                                                     int ny) {
  __shared__ double sh[512];
  const size_t o = (size_t)blockIdx.x * ld * ny;
  double s = 0.0;
  for (int e = threadIdx.x; e < nx * ny; e += blockDim.x) {
    const int jy = e / nx, jx = e - jy * nx;
    const size_t i = o + (size_t)jy * ld + jx;
    s += fabs(du[i] + (dv ? dv[i] : 0.0) + dw[i]);  // dv null: du holds dudx + dvdy
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 256; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_rmsdiv_fin(const double* part, int n, double denom, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += part[i];
    out[0] = s / denom;
  }
}
int op_rmsdiv(les_ctx* c, double* out_dev) {
  const Grid& g = c->g;
  double* part = c->dred;
  k_rmsdiv_part<<<g.nz - 1, 512, 0, c->stream>>>(c->f[LES_DUDX], c->f[LES_DVDY], c->f[LES_DWDZ], part, g.ld, g.nx,
                                                g.ny); LES_COUNT_LAUNCH();
  k_rmsdiv_fin<<<1, 32, 0, c->stream>>>(part, g.nz - 1, (double)(g.nx * g.ny * (g.nz - 1)), out_dev); LES_COUNT_LAUNCH();
  return 0;
}
// timestep_conditions maxima: one block per level reduces max |u|^2 and
// max Nu_t over its plane, then one warp reduces the per-level partials
template <typename NT>
__global__ void __launch_bounds__(512) k_tsc_part(const double* __restrict__ u, const double* __restrict__ v,
                                                  const double* __restrict__ w, const NT* __restrict__ nut,
                                                  double* part1, double* part2, int ld, int nx, int ny) {
  __shared__ double s1[16], s2[16];
  double m1 = -1e300, m2 = -1e300;
  const size_t base = (size_t)ld * ny * blockIdx.x;
  const int n = nx * ny;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const size_t i = base + (size_t)(e % nx) + (size_t)ld * (e / nx);
    m1 = fmax(m1, u[i] * u[i] + v[i] * v[i] + w[i] * w[i]);
    m2 = fmax(m2, cvt<double, NT>(nut[i]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    m1 = fmax(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmax(m2, __shfl_xor_sync(0xffffffffu, m2, o));
  }
  if ((threadIdx.x & 31) == 0) { s1[threadIdx.x >> 5] = m1; s2[threadIdx.x >> 5] = m2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { m1 = fmax(m1, s1[k]); m2 = fmax(m2, s2[k]); }
    part1[blockIdx.x] = m1;
    part2[blockIdx.x] = m2;
  }
}
__global__ void k_tsc_fin(const double* part1, const double* part2, int n, double* out) {
  double m1 = -1e300, m2 = -1e300;
  for (int k = threadIdx.x; k < n; k += 32) { m1 = fmax(m1, part1[k]); m2 = fmax(m2, part2[k]); }
  for (int o = 16; o > 0; o >>= 1) {
    m1 = fmax(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmax(m2, __shfl_xor_sync(0xffffffffu, m2, o));
  }
  if (threadIdx.x == 0) { out[0] = m1; out[1] = m2; }
}
int op_tsc(les_ctx* c, double* cflu, double* visc) {
  const Grid& g = c->g;
  double* p1 = c->dred + 12 * (size_t)(g.nz + 8);  // slots 12, 13
  double* p2 = c->dred + 13 * (size_t)(g.nz + 8);
  if (c->cfg.precision == 1)
    k_tsc_part<float><<<g.nz - 1, 512, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W], f32(c, LES_NU_T),
                                                       p1, p2, g.ld, g.nx, g.ny);
  else
    k_tsc_part<double><<<g.nz - 1, 512, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[LES_NU_T],
                                                        p1, p2, g.ld, g.nx, g.ny);
  LES_COUNT_LAUNCH();
  k_tsc_fin<<<1, 32, 0, c->stream>>>(p1, p2, g.nz - 1, c->dscal + 2); LES_COUNT_LAUNCH();
  LES_CUDA_CHECK(cudaMemcpyAsync(c->host_scal + 2, c->dscal + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  const double delta = std::min(g.dx, g.dy);
  *cflu = std::sqrt(c->host_scal[2]) * c->cfg.dt / g.dx;
  *visc = c->cfg.dt * c->host_scal[3] / (delta * delta);
  return 0;
}

// ---------------------------------------------------------------------------
// Fused time step.  The per-routine versions above restate each routine on
// arbitrary module state; inside one step the state is consistent, so the
// fused step reuses the spectra filt_da already computes:
//   * F(u/(nx*ny)) etc. (Nyquist removed) are saved by filt_da's y pass;
//   * the padded velocities of convec (convec.f90:45-65) and of the scalar
//     advection (scalars_module.f90:286-288) are the same fields: built once;
//   * vorticity (convec.f90:67-114), the padded theta gradients
//     (scalars_module.f90:289-291) and the G/G_test_test inputs u_bar, S_ij of
//     lagrange_Sdep are linear in the saved spectra (vertical differences of
//     spectra = spectra of vertical differences), so only the wall planes
//     set by wallstress / the surface flux need transforms of their own.
// Every identity is exact in exact arithmetic; results differ from the
// per-routine path at the rounding level only.

// one (ld,ny) plane of several fields -> full 2-D spectra (forward only)
static void plane_spectra(les_ctx* c, int np, const double* const* planes, const double* scale, C2* out) {
  const Grid& g = c->g;
  r2c(c, np, 1, planes, (long)g.nplane, scale, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_SAME, DIR_FWD, 1);
  J.nin = 1; J.nout = 1; J.nf = np;
  J.in[0] = c->wsA; J.fs_in = (long)g.C;
  J.out[0] = out; J.fs_out = (long)g.C;
  J.coef[0][0] = CC_ONE;
  cols(c, J);
}

// complex value of a FP64-layout spectrum in arithmetic type R (FP32: the
// narrowing on the integer pipe), and a store into the output type
template <typename R> __device__ __forceinline__ typename CT<R>::type ldR(const C2* p, size_t i);
template <> __device__ __forceinline__ double2 ldR<double>(const C2* p, size_t i) { return p[i]; }
template <> __device__ __forceinline__ float2 ldR<float>(const C2* p, size_t i) {
  const double2 v = p[i];
  return make_float2(cvt_d2f(v.x), cvt_d2f(v.y));
}
template <typename CO, typename CI> __device__ __forceinline__ void stC(CO* o, CI v) {
  o->x = cvt<decltype(o->x)>(v.x);
  o->y = cvt<decltype(o->y)>(v.y);
}

// convec.f90:67-114 vorticity spectra (x 1/(nx*ny)) from U,V,W spectra.
// R: arithmetic (FP32 in the mixed form, where the spectra are FP32-accurate
// except the (0,0) mode, which carries the plane means and is done in FP64)
template <typename R>
__device__ __forceinline__ void vort_point(size_t t, int jz, size_t m, const C2* __restrict__ U,
                                           const C2* __restrict__ V, const C2* __restrict__ W,
                                           const C2* __restrict__ D1, const C2* __restrict__ D2, R k_x, R k_y,
                                           int nk, int nz, R idz, typename CT<R>::type* o) {
  typedef typename CT<R>::type CR;
  const CR w = ldR<R>(W, t), u = ldR<R>(U, t), v = ldR<R>(V, t);
  CR a, b;
  if (jz == 1) {
    const CR w2 = ldR<R>(W, t + nk);
    const CR wy = cadd(ik(w, k_y), ik(w2, k_y));
    const CR wx = cadd(ik(w, k_x), ik(w2, k_x));
    a = csub(cscale(wy, (R)0.5), ldR<R>(D2, m));
    b = csub(ldR<R>(D1, m), cscale(wx, (R)0.5));
  } else if (jz == nz) {
    a = ik(w, k_y);
    b = cscale(ik(w, k_x), (R)-1.0);
  } else {
    const CR vz = cscale(csub(v, ldR<R>(V, t - nk)), idz);
    const CR uz = cscale(csub(u, ldR<R>(U, t - nk)), idz);
    a = csub(ik(w, k_y), vz);
    b = csub(uz, ik(w, k_x));
  }
  o[0] = a;
  o[1] = b;
  o[2] = csub(ik(v, k_x), ik(u, k_y));
}
template <typename CO, typename R>
__global__ void k_vort_spec32(const C2* __restrict__ U, const C2* __restrict__ V, const C2* __restrict__ W,
                              const C2* __restrict__ D1, const C2* __restrict__ D2, CO* o1, CO* o2, CO* o3,
                              const R* __restrict__ kx, const R* __restrict__ ky, int nk, int nz, double idz) {
  GSTRIDE(t, (size_t)nk * nz) {
    const int jz = (int)(t / nk) + 1;
    const size_t m = t - (size_t)(jz - 1) * nk;
    if (m == 0) {
      double2 r[3];
      vort_point<double>(t, jz, m, U, V, W, D1, D2, 0.0, 0.0, nk, nz, idz, r);
      stC(o1 + t, r[0]); stC(o2 + t, r[1]); stC(o3 + t, r[2]);
    } else {
      typename CT<R>::type r[3];
      vort_point<R>(t, jz, m, U, V, W, D1, D2, kx[m], ky[m], nk, nz, (R)idz, r);
      stC(o1 + t, r[0]); stC(o2 + t, r[1]); stC(o3 + t, r[2]);
    }
  }
}

// convec.f90:67-114 vorticity spectra (x 1/(nx*ny)) from U,V,W spectra
template <typename CO>
__global__ void k_vort_spec(const C2* __restrict__ U, const C2* __restrict__ V, const C2* __restrict__ W,
                            const C2* __restrict__ D1, const C2* __restrict__ D2, CO* o1, CO* o2, CO* o3,
                            const double* __restrict__ kx, const double* __restrict__ ky, int nk, int nz,
                            double idz) {
  GSTRIDE(t, (size_t)nk * nz) {
    const int jz = (int)(t / nk) + 1;
    const size_t m = t - (size_t)(jz - 1) * nk;
    const double k_x = kx[m], k_y = ky[m];
    const C2 w = W[t], u = U[t], v = V[t];
    C2 a, b;
    if (jz == 1) {
      const C2 w2 = W[t + nk];
      const C2 wy = cadd(ik(w, k_y), ik(w2, k_y));
      const C2 wx = cadd(ik(w, k_x), ik(w2, k_x));
      a = csub(cscale(wy, 0.5), D2[m]);
      b = csub(D1[m], cscale(wx, 0.5));
    } else if (jz == nz) {
      a = ik(w, k_y);
      b = cscale(ik(w, k_x), -1.0);
    } else {
      const C2 vz = cscale(csub(v, V[t - nk]), idz);
      const C2 uz = cscale(csub(u, U[t - nk]), idz);
      a = csub(ik(w, k_y), vz);
      b = csub(uz, ik(w, k_x));
    }
    const C2 c3 = csub(ik(v, k_x), ik(u, k_y));
    o1[t].x = a.x; o1[t].y = a.y;
    o2[t].x = b.x; o2[t].y = b.y;
    o3[t].x = c3.x; o3[t].y = c3.y;
  }
}

// scalars_module.f90:289-291 padded-gradient inputs: F(dTdx/(nx ny)),
// F(dTdy/(nx ny)), F(dTdz/(nx ny)) from the theta spectrum; levels 1 and nz
// of dTdz come from their own plane transforms (Z1, ZN)
template <typename CI, typename CO>
__global__ void k_dtheta_spec(const CI* __restrict__ T, const C2* __restrict__ Z1, const C2* __restrict__ ZN,
                              CO* o1, CO* o2, CO* o3, const double* __restrict__ kx,
                              const double* __restrict__ ky, int nk, int nz, double idz,
                              const double* __restrict__ th0) {
  GSTRIDE(t, (size_t)nk * nz) {
    const int jz = (int)(t / nk) + 1;
    const size_t m = t - (size_t)(jz - 1) * nk;
    const C2 th = to_d2(T[t]);
    const C2 a = ik(th, kx[m]);
    const C2 b = ik(th, ky[m]);
    C2 z;
    if (jz == 1) z = Z1[m];
    else if (jz == nz) z = ZN[m];
    else {
      z = cscale(csub(th, to_d2(T[t - nk])), idz);
      // the spectra are of theta - th0(level): restore the mean gradient
      if (th0 && m == 0) z.x += (th0[jz - 1] - th0[jz - 2]) * idz;
    }
    o1[t].x = a.x; o1[t].y = a.y;
    o2[t].x = b.x; o2[t].y = b.y;
    o3[t].x = z.x; o3[t].y = z.y;
  }
}
// Mixed form: the same in FP32 (theta's spectrum is FP32 there); the (0,0)
// mode, which restores the mean gradient from th0, and the wall planes' FP64
// spectra are narrowed on the integer pipe after FP64 arithmetic
__global__ void k_dtheta_spec32(const float2* __restrict__ T, const C2* __restrict__ Z1, const C2* __restrict__ ZN,
                                float2* o1, float2* o2, float2* o3, const float* __restrict__ kx,
                                const float* __restrict__ ky, int nk, int nz, double idz,
                                const double* __restrict__ th0) {
  GSTRIDE(t, (size_t)nk * nz) {
    const int jz = (int)(t / nk) + 1;
    const size_t m = t - (size_t)(jz - 1) * nk;
    const float2 th = T[t];
    o1[t] = ik(th, kx[m]);
    o2[t] = ik(th, ky[m]);
    if (jz == 1) stC(o3 + t, Z1[m]);
    else if (jz == nz) stC(o3 + t, ZN[m]);
    else if (m == 0) {
      const double2 tp = make_double2(cvt_f2d(th.x), cvt_f2d(th.y));
      const double2 tm = make_double2(cvt_f2d(T[t - nk].x), cvt_f2d(T[t - nk].y));
      double2 z = cscale(csub(tp, tm), idz);
      z.x += (th0[jz - 1] - th0[jz - 2]) * idz;
      stC(o3 + t, z);
    } else {
      o3[t] = cscale(csub(th, T[t - nk]), (float)idz);
    }
  }
}

// lagrange_Sdep.f90:131-141, sgs_stag.f90:371-498 : spectra of u_bar, v_bar,
// w_bar and S_ij (x 1/(nx*ny)) for the levels jz0..jz0+nl-1.
// out layout: q = 0..8 (u_bar, v_bar, w_bar, S11, S12, S13, S22, S23, S33)
template <typename CO>
__global__ void k_lag_spec(const C2* __restrict__ U, const C2* __restrict__ V, const C2* __restrict__ W,
                           const C2* __restrict__ D1, const C2* __restrict__ D2, CO* out,
                           const double* __restrict__ kx, const double* __restrict__ ky, int nk, int nz,
                           int jz0, int nl, double idz, int shift) {
  const size_t st = (size_t)nk * nl;
  GSTRIDE(t, st) {
    const int lc = (int)(t / nk);
    const size_t m = t - (size_t)lc * nk;
    const int jz = jz0 + lc;
    const size_t i = (size_t)(jz - 1) * nk + m;
    const double k_x = kx[m], k_y = ky[m];
    C2 ub, vb, wb, ux, uy, uz, vx, vy, vz, wx, wy, wz;
    // vertical differences as ddz_uv / ddz_w define them (top level 0)
    auto ddz_uv = [&](const C2* F, int j) -> C2 {  // level j >= 2
      if (j >= nz) return make_double2(0.0, 0.0);
      return cscale(csub(F[(size_t)(j - 1) * nk + m], F[(size_t)(j - 2) * nk + m]), idz);
    };
    auto ddz_w = [&](int j) -> C2 {  // dwdz at level j
      if (j >= nz) return make_double2(0.0, 0.0);
      return cscale(csub(W[(size_t)j * nk + m], W[(size_t)(j - 1) * nk + m]), idz);
    };
    if (jz == 1) {
      const C2 u1 = U[i], v1 = V[i], w1 = W[i], w2 = W[i + nk];
      ub = u1; vb = v1; wb = cscale(w2, 0.25);
      ux = ik(u1, k_x); uy = ik(u1, k_y); uz = D1[m];
      vx = ik(v1, k_x); vy = ik(v1, k_y); vz = D2[m];
      wx = cscale(cadd(ik(w1, k_x), ik(w2, k_x)), 0.5);
      wy = cscale(cadd(ik(w1, k_y), ik(w2, k_y)), 0.5);
      wz = ddz_w(1);
    } else {
      const C2 u0 = U[i], um = U[i - nk], v0 = V[i], vm = V[i - nk], w0 = W[i];
      ub = cscale(cadd(u0, um), 0.5); vb = cscale(cadd(v0, vm), 0.5); wb = w0;
      ux = cscale(cadd(ik(u0, k_x), ik(um, k_x)), 0.5);
      uy = cscale(cadd(ik(u0, k_y), ik(um, k_y)), 0.5);
      uz = ddz_uv(U, jz);
      vx = cscale(cadd(ik(v0, k_x), ik(vm, k_x)), 0.5);
      vy = cscale(cadd(ik(v0, k_y), ik(vm, k_y)), 0.5);
      vz = ddz_uv(V, jz);
      wx = ik(w0, k_x);
      wy = ik(w0, k_y);
      wz = cscale(cadd(ddz_w(jz), ddz_w(jz - 1)), 0.5);
    }
    if (shift && m == 0) {  // filtered fluctuations about the plane mean
      ub = make_double2(0.0, 0.0);
      vb = make_double2(0.0, 0.0);
    }
    const C2 r[9] = {ub, vb, wb, ux, cscale(cadd(uy, vx), 0.5), cscale(cadd(uz, wx), 0.5),
                     vy, cscale(cadd(vz, wy), 0.5), wz};
#pragma unroll
    for (int q = 0; q < 9; ++q) { out[t + q * st].x = r[q].x; out[t + q * st].y = r[q].y; }
  }
}

// The same in arithmetic type R (mixed form: FP32, the (0,0) mode in FP64)
template <typename R>
__device__ __forceinline__ void lag_spec_point(int jz, size_t m, size_t i, const C2* __restrict__ U,
                                               const C2* __restrict__ V, const C2* __restrict__ W,
                                               const C2* __restrict__ D1, const C2* __restrict__ D2, R k_x, R k_y,
                                               int nk, int nz, R idz, int shift, typename CT<R>::type* r) {
  typedef typename CT<R>::type CR;
  const CR z = mk<R>((R)0, (R)0);
  auto ddz_uv = [&](const C2* F, int j) -> CR {  // level j >= 2
    if (j >= nz) return z;
    return cscale(csub(ldR<R>(F, (size_t)(j - 1) * nk + m), ldR<R>(F, (size_t)(j - 2) * nk + m)), idz);
  };
  auto ddz_w = [&](int j) -> CR {  // dwdz at level j
    if (j >= nz) return z;
    return cscale(csub(ldR<R>(W, (size_t)j * nk + m), ldR<R>(W, (size_t)(j - 1) * nk + m)), idz);
  };
  CR ub, vb, wb, ux, uy, uz, vx, vy, vz, wx, wy, wz;
  const R h = (R)0.5;
  if (jz == 1) {
    const CR u1 = ldR<R>(U, i), v1 = ldR<R>(V, i), w1 = ldR<R>(W, i), w2 = ldR<R>(W, i + nk);
    ub = u1; vb = v1; wb = cscale(w2, (R)0.25);
    ux = ik(u1, k_x); uy = ik(u1, k_y); uz = ldR<R>(D1, m);
    vx = ik(v1, k_x); vy = ik(v1, k_y); vz = ldR<R>(D2, m);
    wx = cscale(cadd(ik(w1, k_x), ik(w2, k_x)), h);
    wy = cscale(cadd(ik(w1, k_y), ik(w2, k_y)), h);
    wz = ddz_w(1);
  } else {
    const CR u0 = ldR<R>(U, i), um = ldR<R>(U, i - nk), v0 = ldR<R>(V, i), vm = ldR<R>(V, i - nk), w0 = ldR<R>(W, i);
    ub = cscale(cadd(u0, um), h); vb = cscale(cadd(v0, vm), h); wb = w0;
    ux = cscale(cadd(ik(u0, k_x), ik(um, k_x)), h);
    uy = cscale(cadd(ik(u0, k_y), ik(um, k_y)), h);
    uz = ddz_uv(U, jz);
    vx = cscale(cadd(ik(v0, k_x), ik(vm, k_x)), h);
    vy = cscale(cadd(ik(v0, k_y), ik(vm, k_y)), h);
    vz = ddz_uv(V, jz);
    wx = ik(w0, k_x);
    wy = ik(w0, k_y);
    wz = cscale(cadd(ddz_w(jz), ddz_w(jz - 1)), h);
  }
  if (shift && m == 0) { ub = z; vb = z; }
  r[0] = ub; r[1] = vb; r[2] = wb; r[3] = ux; r[4] = cscale(cadd(uy, vx), h); r[5] = cscale(cadd(uz, wx), h);
  r[6] = vy; r[7] = cscale(cadd(vz, wy), h); r[8] = wz;
}
template <typename CO, typename R>
__global__ void k_lag_spec32(const C2* __restrict__ U, const C2* __restrict__ V, const C2* __restrict__ W,
                             const C2* __restrict__ D1, const C2* __restrict__ D2, CO* out,
                             const R* __restrict__ kx, const R* __restrict__ ky, int nk, int nz, int jz0, int nl,
                             double idz, int shift) {
  const size_t st = (size_t)nk * nl;
  GSTRIDE(t, st) {
    const int lc = (int)(t / nk);
    const size_t m = t - (size_t)lc * nk;
    const int jz = jz0 + lc;
    const size_t i = (size_t)(jz - 1) * nk + m;
    if (m == 0) {
      double2 r[9];
      lag_spec_point<double>(jz, m, i, U, V, W, D1, D2, 0.0, 0.0, nk, nz, idz, shift, r);
#pragma unroll
      for (int q = 0; q < 9; ++q) stC(out + t + q * st, r[q]);
    } else {
      typename CT<R>::type r[9];
      lag_spec_point<R>(jz, m, i, U, V, W, D1, D2, kx[m], ky[m], nk, nz, (R)idz, shift, r);
#pragma unroll
      for (int q = 0; q < 9; ++q) stC(out + t + q * st, r[q]);
    }
  }
}

// Mixed form lagrange_Sdep.f90:142-266 products: the shift about the plane
// mean in FP64, the products and |S| S_ij in FP32
__global__ void k_lag_prod32(const double* __restrict__ u, const double* __restrict__ v,
                             const double* __restrict__ w, Ptr6f Sp, float* out, int ld, int jz0, int nlev,
                             size_t np, const C2* __restrict__ U, const C2* __restrict__ V, size_t nk) {
  const size_t tot = np * nlev;
  GSTRIDE(t, tot) {
    const int lc = (int)(t / np);
    const size_t r = t - (size_t)lc * np;
    const int jz = jz0 + lc;
    const size_t i = (size_t)(jz - 1) * np + r;
    double ubd, vbd;
    float wb;
    if (jz == 1) { ubd = u[i]; vbd = v[i]; wb = 0.25f * cvt_d2f(w[i + np]); }
    else { ubd = 0.5 * (u[i] + u[i - np]); vbd = 0.5 * (v[i] + v[i - np]); wb = cvt_d2f(w[i]); }
    const double u0 = (jz == 1) ? U[0].x : 0.5 * (U[(size_t)(jz - 1) * nk].x + U[(size_t)(jz - 2) * nk].x);
    const double v0 = (jz == 1) ? V[0].x : 0.5 * (V[(size_t)(jz - 1) * nk].x + V[(size_t)(jz - 2) * nk].x);
    const float ub = cvt_d2f(ubd - u0), vb = cvt_d2f(vbd - v0);
    const size_t stride = np * nlev;
    float* o = out + t;
    o[0] = ub * ub; o[stride] = ub * vb; o[2 * stride] = ub * wb;
    o[3 * stride] = vb * vb; o[4 * stride] = vb * wb; o[5 * stride] = wb * wb;
    const float s11 = Sp.p[0][i], s12 = Sp.p[1][i], s13 = Sp.p[2][i];
    const float s22 = Sp.p[3][i], s23 = Sp.p[4][i], s33 = Sp.p[5][i];
    const float Sm = sqrtf(2.0f * (s11 * s11 + s22 * s22 + s33 * s33 + 2.0f * (s12 * s12 + s13 * s13 + s23 * s23)));
    o[6 * stride] = Sm * s11; o[7 * stride] = Sm * s12; o[8 * stride] = Sm * s13;
    o[9 * stride] = Sm * s22; o[10 * stride] = Sm * s23; o[11 * stride] = Sm * s33;
  }
}

// lagrange_Sdep.f90:142-266 physical products (12 planes per level)
template <typename S>
__global__ void k_lag_prod(const double* __restrict__ u, const double* __restrict__ v,
                           const double* __restrict__ w, Ptr6 Sp, S* out, int ld, int jz0, int nlev,
                           size_t np, const C2* __restrict__ U, const C2* __restrict__ V, size_t nk) {
  const size_t tot = np * nlev;
  GSTRIDE(t, tot) {
    const int lc = (int)(t / np);
    const size_t r = t - (size_t)lc * np;
    const int jz = jz0 + lc;
    const size_t i = (size_t)(jz - 1) * np + r;
    double ub, vb, wb;
    if (jz == 1) { ub = u[i]; vb = v[i]; wb = 0.25 * w[i + np]; }
    else { ub = 0.5 * (u[i] + u[i - np]); vb = 0.5 * (v[i] + v[i - np]); wb = w[i]; }
    if (U) {  // L_ij is invariant to a constant shift: form it about the plane mean
      const double u0 = (jz == 1) ? U[0].x : 0.5 * (U[(size_t)(jz - 1) * nk].x + U[(size_t)(jz - 2) * nk].x);
      const double v0 = (jz == 1) ? V[0].x : 0.5 * (V[(size_t)(jz - 1) * nk].x + V[(size_t)(jz - 2) * nk].x);
      ub -= u0;
      vb -= v0;
    }
    const size_t stride = np * nlev;
    S* o = out + t;
    o[0] = (S)(ub * ub); o[stride] = (S)(ub * vb); o[2 * stride] = (S)(ub * wb);
    o[3 * stride] = (S)(vb * vb); o[4 * stride] = (S)(vb * wb); o[5 * stride] = (S)(wb * wb);
    const double s11 = Sp.p[0][i], s12 = Sp.p[1][i], s13 = Sp.p[2][i], s22 = Sp.p[3][i], s23 = Sp.p[4][i], s33 = Sp.p[5][i];
    const double Sm = smag(s11, s22, s33, s12, s13, s23);
    o[6 * stride] = (S)(Sm * s11); o[7 * stride] = (S)(Sm * s12); o[8 * stride] = (S)(Sm * s13);
    o[9 * stride] = (S)(Sm * s22); o[10 * stride] = (S)(Sm * s23); o[11 * stride] = (S)(Sm * s33);
  }
}

// Precision of the fused-step transforms: MX = false -> FP64 everywhere;
// MX = true -> FP32 transforms and FP32 3/2-grid / filter temporaries for the
// scalar, convective, stress-divergence and SGS terms (the projection path,
// the Nyquist filtering of u, v, w, rmsdiv and the plane/wall quantities
// stay FP64).
template <int M> struct PX {
  typedef typename std::conditional<M == 1, float,
                                    typename std::conditional<M == 2, dfloat, double>::type>::type T;  // transforms
  typedef typename CT<T>::type CX;                                              // their complex type
  typedef typename std::conditional<M == 1, float, double>::type S;             // temporary storage
};

template <int M>
static int lagrangeT(les_ctx* c) {
  constexpr bool MX = M == 1;  // the FP32-mixed form
  typedef typename PX<M>::T T;
  typedef typename PX<M>::CX CX;
  typedef typename PX<M>::S S;
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  if (MX) op_interpolag32(c);
  else op_interpolag(c);
  const double delta = g.delta;
  const double cst = 2.0 * (delta * delta);
  const double opftdelta = 1.5 * delta;
  const double lagran_dt = k.dt * (double)k.cs_count;
  const double bexp = std::log(2.0) / (std::log(4.0) - std::log(2.0));
  const int bone = (bexp == 1.0) ? 1 : 0;
  Ptr6 Sp;
  const int sid[6] = {LES_S11, LES_S12, LES_S13, LES_S22, LES_S23, LES_S33};
  for (int q = 0; q < 6; ++q) Sp.p[q] = c->f[sid[q]];
  Ptr6f Sf;  // the mixed form's FP32-held strain
  for (int q = 0; q < 6; ++q) Sf.p[q] = f32(c, sid[q]);
  const C2* U = c->spec;
  const C2* V = c->spec + (size_t)g.nz * g.C;
  const C2* W = c->spec + (size_t)2 * g.nz * g.C;
  const int nch = c->lag_chunk;
  S* tmpS = reinterpret_cast<S*>(c->tmp);
  for (int jz0 = 1; jz0 <= g.nz; jz0 += nch) {
    const int nl = std::min(nch, g.nz - jz0 + 1);
    const long FS = (long)nl * g.C;
    S* prod = tmpS;                                   // 12 * nl planes
    S* flt = tmpS + (size_t)21 * nch * g.nplane;      // 42 * nl planes
    CX* xs = (CX*)c->wsA;
    CX* sp = xs + (size_t)12 * FS;
    if (MX)
      k_lag_spec32<CX, float><<<grid1((size_t)g.C * nl), 256, 0, c->stream>>>(
          U, V, W, c->wspec, c->wspec + g.C, sp, c->kxf, c->kyf, (int)g.C, g.nz, jz0, nl, 1.0 / g.dz, 1);
    else
      k_lag_spec<CX><<<grid1((size_t)g.C * nl), 256, 0, c->stream>>>(U, V, W, c->wspec, c->wspec + g.C, sp, c->kx,
                                                                  c->ky, (int)g.C, g.nz, jz0, nl, 1.0 / g.dz,
                                                                  M != 0 ? 1 : 0); LES_COUNT_LAUNCH();
    if constexpr (MX)
      k_lag_prod32<<<grid1(g.nplane * nl), 256, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W], Sf, prod,
                                                                g.ld, jz0, nl, g.nplane, U, V, g.C);
    else
      k_lag_prod<S><<<grid1(g.nplane * nl), 256, 0, c->stream>>>(c->f[LES_U], c->f[LES_V], c->f[LES_W], Sp, prod, g.ld,
                                                              jz0, nl, g.nplane, M != 0 ? U : nullptr,
                                                              M != 0 ? V : nullptr, g.C); LES_COUNT_LAUNCH();
    const S* in[12];
    for (int q = 0; q < 12; ++q) in[q] = prod + (size_t)q * nl * g.nplane;
    // G_test and G_test_test are cutoffs: only the first ncG (ncGG) kx columns of
    // the filtered spectra are nonzero, so the x pass stores, the y pass
    // transforms and the inverse x pass reads only those
    const int nG = c->ncG, nGG = c->ncGG;
    r2cT<T, S>(c, 12, nl, in, (long)g.nplane, nullptr, nullptr, xs, false, nG);
    CX* ob = (CX*)c->wsB;
    struct Blk { CX* base; int dir; int code_g, code_gg; int count; int q0; };
    const Blk blks[4] = {{sp, DIR_INV, CC_MASK, CC_MASK4, 3, 0},
                         {sp + 3 * FS, DIR_INV, CC_MASK, CC_MASK4, 6, 9},
                         {xs, DIR_BOTH, CC_G, CC_GG, 6, 3},
                         {xs + 6 * FS, DIR_BOTH, CC_G, CC_GG, 6, 15}};
    for (const Blk& b : blks) {
      ColJob J = coljob(c, MAP_SAME, b.dir, nl);
      J.inv_mask = 3u;
      J.nin = 1; J.nout = 2; J.nf = b.count;
      J.in[0] = b.base; J.fs_in = FS;
      J.out[0] = ob + (size_t)b.q0 * FS;
      J.out[1] = ob + (size_t)(21 + b.q0) * FS;
      J.fs_out = FS;
      J.coef[0][0] = b.code_g; J.coef[1][0] = b.code_gg;
      J.ncols = nG;
      colsT<T, CX>(c, J);
    }
    S* out[42];
    for (int q = 0; q < 42; ++q) out[q] = flt + (size_t)q * nl * g.nplane;
    c2rT<T, S>(c, 21, nl, c->wsB, out, (long)g.nplane, false, nG);              // G_test outputs
    c2rT<T, S>(c, 21, nl, ob + (size_t)21 * FS, out + 21, (long)g.nplane, false, nGG);  // G_test_test
    k_lag_final<S, S><<<grid1(g.nplane * nl), 256, 0, c->stream>>>(
        flt, c->f[LES_F_LM], c->f[LES_F_MM], c->f[LES_F_QN], c->f[LES_F_NN], c->f[LES_BETA],
        c->f[LES_CS_OPT2], MX ? nullptr : c->f[LES_TN_LMMM], MX ? nullptr : c->f[LES_TN_QNNN], g.ld, g.nx, g.ny,
        g.nz, jz0, nl, g.nplane, (S)cst, (S)opftdelta, (S)lagran_dt, bone, (S)bexp); LES_COUNT_LAUNCH();
  }
  return 0;
}

template <int M>
static int sgs_stagT(les_ctx* c) {
  constexpr bool MX = M == 1;  // the FP32-mixed form
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  const bool lag = (k.model == 4 || k.model == 5 || k.model == 7);
  const dim3 gpl((unsigned)((g.nplane + 255) / 256), (unsigned)g.nz);
  if (MX)
    k_calc_sij32<<<gpl, 256, 0, c->stream>>>(
        f32(c, LES_DUDX), f32(c, LES_DUDY), c->f[LES_DUDZ], f32(c, LES_DVDX), f32(c, LES_DVDY), c->f[LES_DVDZ],
        f32(c, LES_DWDX), f32(c, LES_DWDY), c->f[LES_DWDZ], f32(c, LES_S11), f32(c, LES_S12), f32(c, LES_S13),
        f32(c, LES_S22), f32(c, LES_S23), f32(c, LES_S33), c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[LES_U_LAG],
        c->f[LES_V_LAG], c->f[LES_W_LAG], g.ld, g.nx, g.ny, lag ? 1 : 0);
  else
    k_calc_sij<<<grid1(g.nfield), 256, 0, c->stream>>>(
        c->f[LES_DUDX], c->f[LES_DUDY], c->f[LES_DUDZ], c->f[LES_DVDX], c->f[LES_DVDY], c->f[LES_DVDZ],
        c->f[LES_DWDX], c->f[LES_DWDY], c->f[LES_DWDZ], c->f[LES_S11], c->f[LES_S12], c->f[LES_S13],
        c->f[LES_S22], c->f[LES_S23], c->f[LES_S33], c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[LES_U_LAG],
        c->f[LES_V_LAG], c->f[LES_W_LAG], c->f[LES_U_LAG_S], c->f[LES_V_LAG_S], c->f[LES_W_LAG_S], g.ld, g.nx,
        g.ny, g.nz, lag ? 1 : 0);
  LES_COUNT_LAUNCH();
  const double* S[6] = {c->f[LES_S11], c->f[LES_S12], c->f[LES_S13], c->f[LES_S22], c->f[LES_S23], c->f[LES_S33]};
  if ((c->jt >= 1 || k.initu) && (c->jt % k.cs_count == 0)) {
    if (k.model == 2 || k.model == 3) {
      double* csz = c->dred;
      if (k.model == 2) op_stddyn(c, csz, S);
      else op_scaledep(c, csz, S);
      k_bcast_levels<<<grid1(g.nfield), 256, 0, c->stream>>>(c->f[LES_CS_OPT2], csz, g.nplane, g.nfield); LES_COUNT_LAUNCH();
    } else if (k.model == 4) {
      op_lagrange_ssim(c, S);
    } else if (k.model == 5) {
      lagrangeT<M>(c);
    } else if (k.model == 7) {  // sgs_stag.f90:150-152 (FP64 form only)
      lagrangeT<M>(c);
      op_lagrange_scalar(c, S, nullptr);
    }
  }
  int ov = 0;
  double csov = 0.0;
  if ((k.model == 5 || k.model == 6 || k.model == 7) && c->jt_total < 500) {
    ov = 1;
    const float c016 = 0.16f;
    csov = (double)(c016 * c016);
    if (k.model == 7) fill(c, c->f[LES_PR_T], g.nfield, k.pr);  // Pr_t = Pr (:171)
  }
  if (MX) {
    Ptr6f Sp;
    const int sid[6] = {LES_S11, LES_S12, LES_S13, LES_S22, LES_S23, LES_S33};
    for (int q = 0; q < 6; ++q) Sp.p[q] = f32(c, sid[q]);
    k_nut_tau32<<<gpl, 256, 0, c->stream>>>(Sp, c->f[LES_CS_OPT2], f32(c, LES_NU_T), f32(c, LES_TXX),
                                            f32(c, LES_TXY), f32(c, LES_TYY), f32(c, LES_TXZ), f32(c, LES_TYZ),
                                            f32(c, LES_TZZ), g.ld, g.nx, g.ny, g.nz, (float)(g.delta * g.delta), ov,
                                            csov); LES_COUNT_LAUNCH();
    return 0;
  }
  k_nut<<<grid1(g.nfield), 256, 0, c->stream>>>(S[0], S[1], S[2], S[3], S[4], S[5], c->f[LES_CS_OPT2],
                                               c->f[LES_NU_T], g.ld, g.nx, g.ny, g.nz, g.delta * g.delta, ov, csov);
  LES_COUNT_LAUNCH();
  k_tau<<<grid1(g.nfield), 256, 0, c->stream>>>(S[0], S[1], S[2], S[3], S[4], S[5], c->f[LES_NU_T],
                                               c->f[LES_TXX], c->f[LES_TXY], c->f[LES_TYY], c->f[LES_TXZ],
                                               c->f[LES_TYZ], c->f[LES_TZZ], g.ld, g.nx, g.ny, g.nz); LES_COUNT_LAUNCH();
  return 0;
}

// inverse-only 3/2 padding of full spectra (field stride nz*C) -> big physical
template <int M, typename CIn>
static void padT(les_ctx* c, const CIn* spec, int nf, typename PX<M>::S* const* out) {
  typedef typename PX<M>::T T;
  const Grid& g = c->g;
  ColJob J = coljob(c, MAP_PAD, DIR_INV, g.nz);
  J.nin = 1; J.nout = 1; J.nf = nf;
  J.in[0] = spec; J.fs_in = (long)g.nz * g.C;
  J.out[0] = c->wsB; J.fs_out = (long)g.nz * g.CB;
  J.coef[0][0] = CC_ONE;
  colsT<T, CIn>(c, J);
  c2rT<T, typename PX<M>::S>(c, nf, g.nz, c->wsB, out, (long)g.nplane_big, true, g.nx / 2);
}
// dealias2 of nf big fields (already scaled) into FP64 small fields
template <int M, typename TO = double>
static void unpadT(les_ctx* c, typename PX<M>::S* const* in, TO* const* out, int nf, int nlev, double scale) {
  typedef typename PX<M>::T T;
  typedef typename PX<M>::CX CX;
  typedef typename PX<M>::S S;
  const Grid& g = c->g;
  double sc[JOB_MAXF];
  for (int i = 0; i < nf; ++i) sc[i] = scale;
  const S* ii[JOB_MAXF];
  for (int i = 0; i < nf; ++i) ii[i] = in[i];
  r2cT<T, S>(c, nf, nlev, ii, (long)g.nplane_big, sc, nullptr, c->wsA, true, g.nx / 2);
  ColJob J = coljob(c, MAP_UNPAD, DIR_BOTH, nlev);
  J.nin = 1; J.nout = 1; J.nf = nf;
  J.in[0] = c->wsA; J.fs_in = (long)nlev * g.CB;
  J.out[0] = c->wsB; J.fs_out = (long)nlev * g.C;
  J.coef[0][0] = CC_ONE;
  colsT<T, CX>(c, J);
  c2rT<T, TO>(c, nf, nlev, c->wsB, out, (long)g.nplane, false, g.nx / 2);
}

// ddx + ddy of two fields summed in spectral space (one inverse); TS: their
// storage (FP64, or FP32 in the mixed form's scalar flux)
template <int M, typename TS = double>
static void div_xyT(les_ctx* c, const TS* tx, const TS* ty, TS* out, int nlev) {
  typedef typename PX<M>::T T;
  typedef typename PX<M>::CX CX;
  const Grid& g = c->g;
  const double sc = 1.0 / (double)(g.nx * g.ny);
  const TS* ii[2] = {tx, ty};
  const double s2[2] = {sc, sc};
  r2cT<T, TS>(c, 2, nlev, ii, (long)g.nplane, s2, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nlev);
  J.nin = 2; J.nout = 1; J.in[0] = c->wsA; J.in[1] = (CX*)c->wsA + (size_t)nlev * g.C; J.out[0] = c->wsB;
  J.coef[0][0] = CC_IKX; J.coef[0][1] = CC_IKY;
  colsT<T, CX>(c, J);
  c2rT<T, TS>(c, 1, nlev, c->wsB, &out, (long)g.nplane, false, g.lh);
}

// rmsdiv.f90:93-100 for the mixed form: its SGS-only dudx, dvdy are FP32
// accurate, so dudx + dvdy is formed here in FP64 (one spectral sum, one
// inverse) into dh (one field) from the filtered u, v.
static void rmsdiv_mixed(les_ctx* c, double* dh, const double* dwdz, double* out_dev) {
  const Grid& g = c->g;
  div_xyT<0>(c, c->f[LES_U], c->f[LES_V], dh, g.nz);
  double* part = c->dred;
  k_rmsdiv_part<<<g.nz - 1, 512, 0, c->stream>>>(dh, nullptr, dwdz, part, g.ld, g.nx, g.ny); LES_COUNT_LAUNCH();
  k_rmsdiv_fin<<<1, 32, 0, c->stream>>>(part, g.nz - 1, (double)(g.nx * g.ny * (g.nz - 1)), out_dev); LES_COUNT_LAUNCH();
}
// les_rmsdiv between steps in the mixed form: the FP64 divergence of the
// current state as the next step's filt_da sees it (w Nyquist-filtered; the
// horizontal derivatives ignore the Nyquist modes by construction).
int op_rmsdiv_state(les_ctx* c, double* out_dev) {
  const Grid& g = c->g;
  double* dh = c->tmp;
  double* wf = c->tmp + g.nfield;
  double* dwz = c->tmp + 2 * g.nfield;
  cudaMemcpyAsync(wf, c->f[LES_W], g.nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  double* f1[1] = {wf};
  nyq_kill(c, f1, 1, g.nz, c->dred + 16 * (size_t)(g.nz + 8), g.nz + 8, c->wsB);
  op_ddz(c, dwz, wf, 0);
  rmsdiv_mixed(c, dh, dwz, out_dev);
  return 0;
}

template <int M>
static int divstressT(les_ctx* c, double* divtx, double* divty, double* divtz) {
  constexpr bool MX = M == 1;  // the FP32-mixed form
  typedef typename PX<M>::T T;
  typedef typename PX<M>::CX CX;
  typedef typename std::conditional<MX, float, double>::type TS;  // tau and h storage
  const Grid& g = c->g;
  const double sc = 1.0 / (double)(g.nx * g.ny);
  const TS* in[5];
  const int tid[5] = {LES_TXX, LES_TXY, LES_TYY, LES_TXZ, LES_TYZ};
  for (int q = 0; q < 5; ++q) in[q] = reinterpret_cast<const TS*>(c->f[tid[q]]);
  double scs[5] = {sc, sc, sc, sc, sc};
  // FP32 and float-float transforms: txz, tyz carry the plane-mean shear
  // stress (large near the wall); the transforms see tau - plane mean, which
  // the horizontal derivatives do not see, so the derivatives keep the
  // fluctuation's precision
  const double* offs[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  if (M != 0) {
    const size_t ms = (size_t)g.nz + 8;
    double* m13 = c->dred + 34 * ms;
    double* m23 = c->dred + 35 * ms;
    plane_sums(c, in[3], (long)g.nplane, g.nz, 4, (double)(g.nx * g.ny), m13);
    plane_sums(c, in[4], (long)g.nplane, g.nz, 4, (double)(g.nx * g.ny), m23);
    offs[3] = m13;
    offs[4] = m23;
  }
  r2cT<T, TS>(c, 5, g.nz, in, (long)g.nplane, scs, nullptr, c->wsA, false, g.lh, offs);
  const long FS = (long)g.nz * g.C;
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, g.nz);
  J.nin = 3; J.nout = 2;
  J.in[0] = c->wsA; J.in[1] = (CX*)c->wsA + FS; J.in[2] = (CX*)c->wsA + 2 * FS;
  J.out[0] = c->wsB; J.out[1] = (CX*)c->wsB + FS;
  J.coef[0][0] = CC_IKX; J.coef[0][1] = CC_IKY;
  J.coef[1][1] = CC_IKX; J.coef[1][2] = CC_IKY;
  colsT<T, CX>(c, J);
  ColJob K = coljob(c, MAP_SAME, DIR_BOTH, g.nz);
  K.nin = 2; K.nout = 1;
  K.in[0] = (CX*)c->wsA + 3 * FS; K.in[1] = (CX*)c->wsA + 4 * FS;
  K.out[0] = (CX*)c->wsB + 2 * FS;
  K.coef[0][0] = CC_IKX; K.coef[0][1] = CC_IKY;
  colsT<T, CX>(c, K);
  TS* tmpS = reinterpret_cast<TS*>(c->tmp);
  TS* h[3] = {tmpS, tmpS + g.nfield, tmpS + 2 * g.nfield};
  c2rT<T, TS>(c, 3, g.nz, c->wsB, h, (long)g.nplane, false, g.lh);
  if constexpr (MX)
    k_divstress_fin32<<<dim3((unsigned)((g.nplane + 255) / 256), (unsigned)g.nz), 256, 0, c->stream>>>(
        divtx, divty, divtz, h[0], h[1], h[2], f32(c, LES_TXZ), f32(c, LES_TYZ), f32(c, LES_TZZ), g.ld, g.nx, g.ny,
        g.nz, (float)(1.0 / g.dz));
  else
    k_divstress_fin<<<grid1(g.nfield), 256, 0, c->stream>>>(divtx, divty, divtz, h[0], h[1], h[2], c->f[LES_TXZ],
                                                           c->f[LES_TYZ], c->f[LES_TZZ], g.ld, g.nx, g.ny, g.nz,
                                                           1.0 / g.dz, 7);
  LES_COUNT_LAUNCH();
  return 0;
}

template <int M>
static int scalarT(les_ctx* c, typename PX<M>::S* const* bigf, const ScalarDesc& d) {
  constexpr bool MX = M == 1;  // the FP32-mixed form
  typedef typename PX<M>::T T;
  typedef typename PX<M>::CX CX;
  typedef typename PX<M>::S S;
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  const int nz = g.nz;
  const size_t FS = (size_t)nz * g.C;
  // the scalar's spectrum (precision of the transform) in the fourth saved
  // spectrum slot: theta's, then (qmix after theta) the humidity's
  CX* specT = reinterpret_cast<CX*>(c->spec + 3 * FS);
  // FP32 and float-float transforms see theta - th0(level) (th0 = plane
  // mean): the filter and the horizontal derivatives are unchanged by a
  // per-level constant, and the perturbation keeps its precision; th0 is added
  // back in FP64
  double* th0 = M != 0 ? c->dred + d.mean_slot * (size_t)(nz + 8) : nullptr;
  if (M != 0) {
    plane_sums(c, c->f[d.s], (long)g.nplane, nz, 4, (double)(g.nx * g.ny), th0);
  }
  {  // filt_da(theta) with the spectrum saved
    const double* in[1] = {c->f[d.s]};
    const double sc[1] = {1.0 / (double)(g.nx * g.ny)};
    const double* offs[1] = {th0};
    r2cT<T, double>(c, 1, nz, in, (long)g.nplane, sc, nullptr, c->wsA, false, g.lh, offs);
    ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nz);
    J.nin = 1; J.nout = 4; J.inv_mask = 7u;
    J.in[0] = c->wsA;
    J.out[0] = c->wsB; J.out[1] = (CX*)c->wsB + FS; J.out[2] = (CX*)c->wsB + 2 * FS; J.out[3] = specT;
    J.coef[0][0] = CC_KILL; J.coef[1][0] = CC_IKX; J.coef[2][0] = CC_IKY; J.coef[3][0] = CC_KILL;
    colsT<T, CX>(c, J);
    if constexpr (MX) {  // theta in FP64 (plane mean added back), the gradients FP32-held
      double* o1[1] = {c->f[d.s]};
      const double* offo[1] = {th0};
      c2rT<T, double>(c, 1, nz, c->wsB, o1, (long)g.nplane, false, g.lh, offo);
      float* o2[2] = {f32(c, d.dsdx), f32(c, d.dsdy)};
      c2rT<T, float>(c, 2, nz, (CX*)c->wsB + FS, o2, (long)g.nplane, false, g.lh);
    } else {
      double* out[3] = {c->f[d.s], c->f[d.dsdx], c->f[d.dsdy]};
      const double* offo[3] = {th0, nullptr, nullptr};
      c2rT<T, double>(c, 3, nz, c->wsB, out, (long)g.nplane, false, g.lh, offo);
    }
  }
  op_ddz(c, c->f[d.dsdz], c->f[d.s], 1);
  fill(c, c->f[d.dsdz] + (size_t)(nz - 1) * g.nplane, g.nplane, d.top_grad);
  // RHS_Tf = RHS_T: exchanged with the momentum RHS at the start of the step
  k_sflux<<<grid1((size_t)g.nx * g.ny), 256, 0, c->stream>>>(c->f[d.s], c->f[d.flux], c->f[LES_PHI_H],
                                                            c->f[LES_USTAR_AVG], c->f[d.dsdz],
                                                            c->f[d.sgs3], g.nx, g.ny, g.ld,
                                                            d.flux_scale, k.vonk, g.dz); LES_COUNT_LAUNCH();
  {
    const double cs = 1.0 / (double)(g.nx * g.ny);
    const double* pl[2] = {c->f[d.dsdz], c->f[d.dsdz] + (size_t)(nz - 1) * g.nplane};
    const double sc[2] = {cs, cs};
    plane_spectra(c, 2, pl, sc, c->wspec + 2 * g.C);
  }
  CX* ds = (CX*)c->wsA;
  if constexpr (MX)
    k_dtheta_spec32<<<grid1(FS), 256, 0, c->stream>>>(specT, c->wspec + 2 * g.C, c->wspec + 3 * g.C, ds, ds + FS,
                                                      ds + 2 * FS, c->kxf, c->kyf, (int)g.C, nz, 1.0 / g.dz, th0);
  else
    k_dtheta_spec<CX, CX><<<grid1(FS), 256, 0, c->stream>>>(specT, c->wspec + 2 * g.C, c->wspec + 3 * g.C, ds, ds + FS,
                                                         ds + 2 * FS, c->kx, c->ky, (int)g.C, nz, 1.0 / g.dz,
                                                         th0); LES_COUNT_LAUNCH();
  {
    S* o3[3] = {bigf[3], bigf[4], bigf[5]};
    padT<M, CX>(c, ds, 3, o3);
  }
  k_scalar_prod<S><<<grid1(g.nfield_big), 256, 0, c->stream>>>(bigf[0], bigf[1], bigf[2], bigf[3], bigf[4], bigf[5],
                                                              bigf[6], g.ld_big, g.nx2, g.ny2, nz,
                                                              MX ? mean_tab(c).UVf : nullptr); LES_COUNT_LAUNCH();
  if constexpr (MX) {
    // FP32 scalar flux: the advection term, tx, ty and their divergence in
    // FP32 scratch (tmp), the theta RHS itself FP64
    float* tf = reinterpret_cast<float*>(c->tmp);
    float* tx = tf;
    float* ty = tf + g.nfield;
    float* dxy = tf + 2 * g.nfield;
    float* rtf = tf + 3 * g.nfield;
    {
      S* b6[1] = {bigf[6]};
      float* o[1] = {rtf};
      unpadT<M, float>(c, b6, o, 1, nz, 1.0 / (double)(g.nx2 * g.ny2));
    }
    const dim3 gpl((unsigned)((g.nplane + 255) / 256), (unsigned)nz);
    k_scalar_temp_xy32<<<gpl, 256, 0, c->stream>>>(f32(c, LES_NU_T), f32(c, d.dsdx), f32(c, d.dsdy), tx, ty,
                                                   g.ld, g.nx, g.ny, nz, (float)(1.0 / k.pr)); LES_COUNT_LAUNCH();
    div_xyT<M, float>(c, tx, ty, dxy, nz);
    k_scalar_rhs32<<<dim3(gpl.x, (unsigned)(nz - 1)), 256, 0, c->stream>>>(
        c->f[d.rhs], rtf, dxy, f32(c, LES_NU_T), c->f[d.dsdz], c->f[d.sgs3], g.ld, g.nx, g.ny,
        (float)(1.0 / k.pr), (float)(1.0 / g.dz)); LES_COUNT_LAUNCH();
  } else {
    double* rt = c->f[d.rhs];
    {
      S* b6[1] = {bigf[6]};
      double* o[1] = {rt};
      unpadT<M>(c, b6, o, 1, nz, 1.0 / (double)(g.nx2 * g.ny2));
    }
    double* tx = c->tmp;
    double* ty = c->tmp + g.nfield;
    double* dxy = c->tmp + 2 * g.nfield;
    k_scalar_temp_xy<double><<<grid1(g.nfield), 256, 0, c->stream>>>(c->f[LES_NU_T], c->f[d.dsdx],
                                                                    c->f[d.dsdy], tx, ty, g.ld, g.nx, g.ny, nz,
                                                                    k.pr, c->f[LES_PR_T]); LES_COUNT_LAUNCH();
    div_xyT<M>(c, tx, ty, dxy, nz);
    k_scalar_rhs<double><<<grid1(g.nplane * (nz - 1)), 256, 0, c->stream>>>(rt, dxy, c->f[LES_NU_T],
                                                                           c->f[d.dsdz], c->f[d.sgs3],
                                                                           g.ld, g.nx, g.ny, nz, k.pr, c->f[LES_PR_T],
                                                                           1.0 / g.dz);
    LES_COUNT_LAUNCH();
  }
  if (d.buoyancy) calcbeta(c);
  if (c->jt == 1 && !k.initsc)
    cudaMemcpyAsync(c->f[d.rhsf], c->f[d.rhs], g.nfield * sizeof(double), cudaMemcpyDeviceToDevice,
                    c->stream);
  const int topg = k.lz_over_zi > 1.0 ? 1 : 0;
  k_step_scalar<<<dim3((unsigned)((g.nplane + 255) / 256), nz - 1), 256, 0, c->stream>>>(
      c->f[d.s], c->f[d.rhs], c->f[d.rhsf], g.ld, g.nx, g.ny, nz, k.dt, topg,
      d.top_grad * g.dz); LES_COUNT_LAUNCH();
  return 0;
}

template <int M>
static int convecT(les_ctx* c, typename PX<M>::S* const* bigf, double* cx, double* cy, double* cz) {
  constexpr bool MX = M == 1;  // the FP32-mixed form
  typedef typename PX<M>::CX CX;
  typedef typename PX<M>::S S;
  const Grid& g = c->g;
  const size_t FS = (size_t)g.nz * g.C;
  CX* vs = (CX*)c->wsA;
  if (MX)
    k_vort_spec32<CX, float><<<grid1(FS), 256, 0, c->stream>>>(c->spec, c->spec + FS, c->spec + 2 * FS, c->wspec,
                                                              c->wspec + g.C, vs, vs + FS, vs + 2 * FS, c->kxf,
                                                              c->kyf, (int)g.C, g.nz, 1.0 / g.dz);
  else
    k_vort_spec<CX><<<grid1(FS), 256, 0, c->stream>>>(c->spec, c->spec + FS, c->spec + 2 * FS, c->wspec, c->wspec + g.C,
                                                   vs, vs + FS, vs + 2 * FS, c->kx, c->ky, (int)g.C, g.nz,
                                                   1.0 / g.dz); LES_COUNT_LAUNCH();
  {
    S* o3[3] = {bigf[3], bigf[4], bigf[5]};
    padT<M, CX>(c, vs, 3, o3);
  }
  const S cst2 = (S)(1.0 / (double)(g.nx2 * g.ny2));
  k_convec_prod<S><<<grid1(g.nplane_big * (g.nz - 1)), 256, 0, c->stream>>>(
      bigf[0], bigf[1], bigf[2], bigf[3], bigf[4], bigf[5], bigf[6], bigf[7], bigf[8], g.ld_big, g.nx2, g.ny2,
      g.nz, cst2); LES_COUNT_LAUNCH();
  {
    S* bins[3] = {bigf[6], bigf[7], bigf[8]};
    double* outs[3] = {cx, cy, cz};
    unpadT<M>(c, bins, outs, 3, g.nz - 1, 1.0);
  }
  const size_t top = (size_t)(g.nz - 1) * g.nplane;
  fill(c, cx + top, g.nplane, LES_BOGUS);
  fill(c, cy + top, g.nplane, LES_BOGUS);
  fill(c, cz + top, g.nplane, LES_BOGUS);
  return 0;
}

// Mixed form, the linear part of the convective term split about the plane
// mean wind (see k_rhs_ab2_mx): the per-level factors, then w_z = dv/dx -
// du/dy and dw/dx of the Nyquist-filtered u', v', w from float-float
// transforms of the fluctuations, into the free half of the 3/2-grid pool
// (the mixed form keeps its nine 3/2-grid fields in FP32 in the first half).
static dfloat* mlin_fields(les_ctx* c) {
  const size_t half = ((size_t)9 * c->g.nfield_big + 1) / 2;
  const size_t off = (half + 63) / 64 * 64;  // 512-byte aligned
  return reinterpret_cast<dfloat*>(c->big + off);
}
// the mixed form's predictor fields u*, v*, w* (after the two fields above)
// the float-float predictor u*, v*, w* (three fields after the linear terms)
static float2* ustar_fields(les_ctx* c) {
  return reinterpret_cast<float2*>(mlin_fields(c) + 2 * c->g.nfield);
}
static void meanflow_lin(les_ctx* c) {
  const Grid& g = c->g;
  const int nz = g.nz;
  const int ms = nz + 8;
  const double* mean = c->dred + 16 * (size_t)ms;  // u, v, w plane means (filt_da_uvw_mixed)
  k_mean_tab<<<(nz + 127) / 128, 128, 0, c->stream>>>(mean, ms, nz, g.dz, mean_tab(c)); LES_COUNT_LAUNCH();
  // the transforms are unnormalised: u's x and y round trips gain nx ny,
  // v's and w's x round trip alone gains nx
  const double sc = 1.0 / (double)(g.nx * g.ny), scx = 1.0 / (double)g.nx;
  const double* in[3] = {c->f[LES_U], c->f[LES_V], c->f[LES_W]};
  const double scs[3] = {sc, scx, scx};
  const double* offs[3] = {mean, mean + ms, mean + 2 * ms};
  r2cT<dfloat, double>(c, 3, nz, in, (long)g.nplane, scs, nullptr, c->wsA, false, g.lh, offs);
  const long FS = (long)nz * g.C;
  // w_z = i kx v - i ky u: -du/dy needs the y round trip, dv/dx and dw/dx do
  // not (x wavenumber alone, k_ikx_rows)
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nz);
  J.nin = 1; J.nout = 1; J.nf = 1;
  J.in[0] = c->wsA;
  J.out[0] = c->wsB;
  J.coef[0][0] = CC_MIKY;
  colsT<dfloat, dcomplex>(c, J);
  const dcomplex* sa = (const dcomplex*)c->wsA;
  dcomplex* sb = (dcomplex*)c->wsB;
  k_ikx_rows<dcomplex><<<grid1((size_t)FS), 256, 0, c->stream>>>(sa + FS, sb, c->kxd, c->kx, g.lh, (size_t)FS, 1);
  LES_COUNT_LAUNCH();
  k_ikx_rows<dcomplex><<<grid1((size_t)FS), 256, 0, c->stream>>>(sa + 2 * FS, sb + FS, c->kxd, c->kx, g.lh,
                                                                 (size_t)FS, 0);
  LES_COUNT_LAUNCH();
  dfloat* ml = mlin_fields(c);
  dfloat* out[2] = {ml, ml + g.nfield};
  c2rT<dfloat, dfloat>(c, 2, nz, c->wsB, out, (long)g.nplane, false, g.lh);
}
// the (0,0) modes of the saved u, v spectra (the plane means) set to zero:
// the 3/2-grid u', v' and the vorticity fluctuations are padded from them
__global__ void k_zero_mean_modes(C2* spec, size_t fs, size_t nk, int nz) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nz) return;
  const int f = t / nz, lev = t - f * nz;
  spec[(size_t)f * fs + (size_t)lev * nk] = make_double2(0.0, 0.0);
}

// float-float spectra of f - plane mean widened to FP64 in place (hi + lo,
// exact), the plane mean put back into each level's (0,0) mode
__global__ void k_widen_dc(C2* p, size_t n, size_t nk, int nz, const double* __restrict__ mean, int ms) {
  GSTRIDE(i, n) {
    const dcomplex v = reinterpret_cast<const dcomplex*>(p)[i];
    double2 w = to_d2(v);
    const size_t pl = i / nk;
    if (i - pl * nk == 0) {
      const int f = (int)(pl / (size_t)nz), lev = (int)(pl - (size_t)f * nz);
      w.x += mean[(size_t)f * ms + lev];
    }
    p[i] = w;
  }
}
// filt_da of u, v, w in float-float transforms (FP64 state in and out), the
// Nyquist-filtered spectra F(f/(nx ny)) saved in FP64 like filt_da_multi_spec.
// The transforms see f - plane mean: a float-float rounding is relative to
// the values transformed, and u's mean is a hundred times v's and w's
// fluctuations; the mean is added back in FP64.
static int filt_da_uvw_ff(les_ctx* c) {
  const Grid& g = c->g;
  const int nz = g.nz;
  const int ms = nz + 8;
  const long FS = (long)nz * g.C;
  double* f3[3] = {c->f[LES_U], c->f[LES_V], c->f[LES_W]};
  double* mean = c->dred + 16 * (size_t)ms;  // slots 16..18
  for (int q = 0; q < 3; ++q) plane_sums(c, f3[q], (long)g.nplane, nz, 4, (double)(g.nx * g.ny), mean + q * ms);
  const double sc = 1.0 / (double)(g.nx * g.ny);
  const double* in[3] = {f3[0], f3[1], f3[2]};
  const double scs[3] = {sc, sc, sc};
  const double* offs[3] = {mean, mean + ms, mean + 2 * ms};
  r2cT<dfloat, double>(c, 3, nz, in, (long)g.nplane, scs, nullptr, c->wsA, false, g.lh, offs);
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nz);
  J.nin = 1; J.nout = 4; J.nf = 3; J.inv_mask = 7u;  // output 3 (the spectrum) stays spectral
  J.in[0] = c->wsA; J.fs_in = FS;
  J.out[0] = c->wsB;
  J.out[1] = (dcomplex*)c->wsB + 3 * FS;
  J.out[2] = (dcomplex*)c->wsB + 6 * FS;
  J.out[3] = reinterpret_cast<dcomplex*>(c->spec);
  J.fs_out = FS;
  J.coef[0][0] = CC_KILL; J.coef[1][0] = CC_IKX; J.coef[2][0] = CC_IKY; J.coef[3][0] = CC_KILL;
  colsT<dfloat, dcomplex>(c, J);
  k_widen_dc<<<grid1(3 * (size_t)FS), 256, 0, c->stream>>>(c->spec, 3 * (size_t)FS, g.C, nz, mean, ms);
  LES_COUNT_LAUNCH();
  double* o9[9] = {f3[0], f3[1], f3[2], c->f[LES_DUDX], c->f[LES_DVDX], c->f[LES_DWDX],
                   c->f[LES_DUDY], c->f[LES_DVDY], c->f[LES_DWDY]};
  const double* offo[9] = {mean, mean + ms, mean + 2 * ms, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  c2rT<dfloat, double>(c, 9, nz, c->wsB, o9, (long)g.nplane, false, g.lh, offo);
  return 0;
}

// main.f90:202-478, one iteration on the device-resident state
void rhs_swap(les_ctx* c) {
  std::swap(c->f[LES_RHSX], c->f[LES_RHSX_F]);
  std::swap(c->f[LES_RHSY], c->f[LES_RHSY_F]);
  std::swap(c->f[LES_RHSZ], c->f[LES_RHSZ_F]);
  std::swap(c->f[LES_RHS_T], c->f[LES_RHS_TF]);
  std::swap(c->f[LES_RHS_Q], c->f[LES_RHS_QF]);  // null without humidity
  c->rhs_par ^= 1;
}

template <int M>
static int stepT(les_ctx* c) {
  constexpr bool MX = M == 1;  // the FP32-mixed form
  typedef typename PX<M>::S S;
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  c->jt += 1;
  c->jt_total += 1;
  // RHS*_f = RHS* (main.f90:212-214, and RHS_Tf = RHS_T of the scalar): the
  // buffers are exchanged; RHS* is rewritten below before it is read
  rhs_swap(c);
  // filtered surface u, v for obukhov and wallstress (u, v do not change in
  // between): the last two temp planes, which nothing before wallstress uses
  const double* uv1 = c->tmp + (size_t)(c->ntmp - 2) * g.nplane;
  surface_uv_filtered(c, const_cast<double*>(uv1));
  op_obukhov(c, uv1);
  if (M == 2) {
    filt_da_uvw_ff(c);
  } else if (!MX) {
    double* f3[3] = {c->f[LES_U], c->f[LES_V], c->f[LES_W]};
    double* x3[3] = {c->f[LES_DUDX], c->f[LES_DVDX], c->f[LES_DWDX]};
    double* y3[3] = {c->f[LES_DUDY], c->f[LES_DVDY], c->f[LES_DWDY]};
    filt_da_multi_spec(c, f3, x3, y3, 3, g.nz, c->spec);
  } else {
    filt_da_uvw_mixed(c);
    meanflow_lin(c);
  }
  op_ddz(c, c->f[LES_DUDZ], c->f[LES_U], 1);
  op_ddz(c, c->f[LES_DVDZ], c->f[LES_V], 1);
  op_ddz(c, c->f[LES_DWDZ], c->f[LES_W], 0);
  const bool rms_step = k.rmsdiv_every > 0 && c->jt % k.rmsdiv_every == 0;
  if (MX && rms_step) rmsdiv_mixed(c, c->tmp, c->f[LES_DWDZ], c->dscal + 1);
  op_wallstress(c, uv1);
  {  // spectra of the wall planes dudz(1), dvdz(1) set by wallstress
    const double cs = 1.0 / (double)(g.nx * g.ny);
    const double* pl[2] = {c->f[LES_DUDZ], c->f[LES_DVDZ]};
    const double sc[2] = {cs, cs};
    plane_spectra(c, 2, pl, sc, c->wspec);
  }
  sgs_stagT<M>(c);
  S* bigf[9];
  for (int q = 0; q < 9; ++q) bigf[q] = reinterpret_cast<S*>(c->big) + (size_t)q * g.nfield_big;
  if (MX) {  // the mixed form pads u', v' (its linear terms use the plane means)
    k_zero_mean_modes<<<(2 * g.nz + 127) / 128, 128, 0, c->stream>>>(c->spec, (size_t)g.nz * g.C, g.C, g.nz);
    LES_COUNT_LAUNCH();
  }
  padT<M, C2>(c, c->spec, 3, bigf);  // padded u, v, w (convec.f90:45-65)
  if (k.s_flag) {
    scalarT<M>(c, bigf, theta_desc(c));
    if (k.q_flag) scalarT<M>(c, bigf, q_desc(c));  // main.f90:273-274
  } else {
    fill(c, c->f[LES_BETA_SCAL], g.nfield, 0.0);
  }
  divstressT<M>(c, c->f[LES_DIVTX], c->f[LES_DIVTY], c->f[LES_DIVTZ]);
  convecT<M>(c, bigf, c->f[LES_RHSX], c->f[LES_RHSY], c->f[LES_RHSZ]);
  const size_t nv = g.nplane * (g.nz - 1);
  const int euler = (c->jt == 1 && !k.initu) ? 1 : 0;
  if (MX) {
    const dfloat* ml = mlin_fields(c);
    const dfloat idz(1.0 / g.dz), dtd(k.dt);
    k_rhs_ab2_mx<<<dim3((unsigned)((g.nplane + 255) / 256), (unsigned)g.nz), 256, 0, c->stream>>>(
        c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[LES_RHSX], c->f[LES_RHSY], c->f[LES_RHSZ], ff2(c, LES_RHSX_F),
        ff2(c, LES_RHSY_F), ff2(c, LES_RHSZ_F), c->f[LES_DIVTX], c->f[LES_DIVTY], c->f[LES_DIVTZ],
        c->f[LES_BETA_SCAL], ml, ml + g.nfield, f32(c, LES_DWDY), mean_tab(c), ustar_fields(c),
        ustar_fields(c) + g.nfield, ustar_fields(c) + 2 * g.nfield, g.ld, g.ny, g.nz, make_float2(idz.hi, idz.lo),
        make_float2(dtd.hi, dtd.lo), k.s_flag, euler);
  } else
    k_rhs_ab2<<<grid1(nv + g.nplane), 256, 0, c->stream>>>(
        c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[LES_RHSX], c->f[LES_RHSY], c->f[LES_RHSZ], c->f[LES_RHSX_F],
        c->f[LES_RHSY_F], c->f[LES_RHSZ_F], c->f[LES_DIVTX], c->f[LES_DIVTY], c->f[LES_DIVTZ], c->f[LES_BETA_SCAL],
        nv, g.nplane, k.dt, k.s_flag, euler);
  LES_COUNT_LAUNCH();
  if (MX) {
    const float2* ust = ustar_fields(c);
    const float2* u3[3] = {ust, ust + g.nfield, ust + 2 * g.nfield};
    pressT<dfloat>(c, c->f[LES_P], c->f[LES_DPDX], c->f[LES_DPDY], u3);
    k_dpdz_project32<<<dim3((unsigned)((g.nplane + 255) / 256), (unsigned)(g.nz - 1)), 256, 0, c->stream>>>(
        c->f[LES_U], c->f[LES_V], c->f[LES_W], u3[0], u3[1], u3[2], ff2(c, LES_RHSX), ff2(c, LES_RHSY),
        ff2(c, LES_RHSZ), c->f[LES_P], c->f[LES_DPDX], c->f[LES_DPDY], c->f[LES_DPDZ], g.ld, g.nx, g.ny, g.nz,
        1.0 / g.dz, k.dt);
  } else {
    // FP64 projection in the FP64 form and in the float-float transform form:
    // float-float transforms of the predictor would leave its rounding times
    // the wavenumber in the divergence (rmsdiv 4e-12 instead of 1e-13 at 128^3)
    pressT<double>(c, c->f[LES_P], c->f[LES_DPDX], c->f[LES_DPDY]);
  }
  if (!MX)
    k_dpdz_project<<<grid1(g.nplane * (g.nz - 1)), 256, 0, c->stream>>>(
        c->f[LES_U], c->f[LES_V], c->f[LES_W], c->f[LES_RHSX], c->f[LES_RHSY], c->f[LES_RHSZ], c->f[LES_P],
        c->f[LES_DPDX], c->f[LES_DPDY], c->f[LES_DPDZ], g.ld, g.nx, g.ny, g.nz, g.dz, k.dt);
  LES_COUNT_LAUNCH();
  LES_CUDA_CHECK(cudaGetLastError());
  if (rms_step) {
    if (!MX) op_rmsdiv(c, c->dscal + 1);
    LES_CUDA_CHECK(cudaMemcpyAsync(c->host_scal + 1, c->dscal + 1, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    double cflu, visc;
    int st = op_tsc(c, &cflu, &visc);
    if (st) return st;
    c->rmsdiv_last = c->host_scal[1];
    if (cflu > 0.1 || cflu < 0.0) return LES_ERR_CFL;
  }
  return 0;
}

// One representative transform batch (filt_da of three fields) on scratch
// planes in the given precision; used by the autotuner.
template <typename T>
static void tune_probe(les_ctx* c) {
  typedef typename CT<T>::type CX;
  const Grid& g = c->g;
  const int nz = g.nz;
  const double sc = 1.0 / (double)(g.nx * g.ny);
  const double* in[3] = {c->f[LES_U], c->f[LES_V], c->f[LES_W]};
  const double scs[3] = {sc, sc, sc};
  r2cT<T, double>(c, 3, nz, in, (long)g.nplane, scs, nullptr, c->wsA, false, g.lh);
  ColJob J = coljob(c, MAP_SAME, DIR_BOTH, nz);
  J.nin = 1; J.nout = 3; J.nf = 3;
  J.in[0] = c->wsA; J.fs_in = (long)nz * g.C;
  J.out[0] = c->wsB; J.out[1] = (CX*)c->wsB + 3 * (size_t)nz * g.C; J.out[2] = (CX*)c->wsB + 6 * (size_t)nz * g.C;
  J.fs_out = (long)nz * g.C;
  J.coef[0][0] = CC_KILL; J.coef[1][0] = CC_IKX; J.coef[2][0] = CC_IKY;
  colsT<T, CX>(c, J);
  double* out[9];
  for (int q = 0; q < 9; ++q) out[q] = c->big + (size_t)q * g.nfield;  // scratch (the 3/2-grid pool)
  c2rT<T, double>(c, 9, nz, c->wsB, out, (long)g.nplane, false, g.lh);
  // the padded size too
  const double* bi[3] = {c->big, c->big + g.nfield_big, c->big + 2 * g.nfield_big};
  r2cT<T, double>(c, 3, nz, bi, (long)g.nplane_big, nullptr, nullptr, c->wsA, true, g.nx / 2);
  double* bo[3] = {c->big + 3 * g.nfield_big, c->big + 4 * g.nfield_big, c->big + 5 * g.nfield_big};
  c2rT<T, double>(c, 3, nz, c->wsA, bo, (long)g.nplane_big, true, g.nx / 2);
}
// fp32: the FP32 transforms' knobs; else the 8-byte-real knobs, probed with
// the kernels the form runs them with (FP64 in the FP64 form, float-float in
// the mixed and float-float transform forms)
void autotune_probe(les_ctx* c, int fp32) {
  if (fp32) tune_probe<float>(c);
  else if (c->cfg.precision != 0) tune_probe<dfloat>(c);
  else tune_probe<double>(c);
}

int step_fp64(les_ctx* c) { return stepT<0>(c); }
int step_mixed(les_ctx* c) { return stepT<1>(c); }
int step_ff(les_ctx* c) { return stepT<2>(c); }

}  // namespace les
