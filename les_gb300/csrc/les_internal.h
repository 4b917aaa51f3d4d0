// Internal context of the GB300 LES core (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include <string>
#include "../../include/les_gb300.h"
#include "fft.cuh"

namespace les {

template <typename T, typename TIn>
int launch_rows_r2c(const RowJob& J, const RealPlanDev& P, cudaStream_t s);
template <typename T, typename TOut>
int launch_rows_c2r(const RowJob& J, const RealPlanDev& P, cudaStream_t s);
template <typename T, typename CIn>
int launch_cols(const ColJob& J, const FftPlanDev& Pin, const FftPlanDev& Pout, cudaStream_t s);

// Host-side FFT plan: owns the device twiddle table.
struct HostPlan {
  FftPlanDev c{};
  double2* dev = nullptr;
  float2* devf = nullptr;
  void* devd = nullptr;  // float-float twiddles (float4)
  void* devuf = nullptr;  // unit-circle tables (float2, float4)
  void* devud = nullptr;
};
struct HostRealPlan {
  RealPlanDev r{};
  double2* dev = nullptr;
  float2* devf = nullptr;
  void* devd = nullptr;
};

// Grid constants computed once on the host in the reference's expression
// order (param.f90:56-65, fft.f90:54-81, test_filtermodule.f90:32-63).
struct Grid {
  int nx, ny, nz, ld, lh, nx2, ny2, ld_big, lh_big;
  double dx, dy, dz, delta;
  size_t nplane, nfield, nplane_big, nfield_big;
  size_t C, CB;  // complex entries of a small x-spectrum plane (ny*lh) and a
                 // big truncated one (ny2*(nx/2))
};

}  // namespace les

struct les_ctx {
  les_config cfg;
  les::Grid g;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int device = 0;
  int ptr_mode = 0;  // 0 host pointers, 1 device pointers
  int jt = 0, jt_total = 0;
  bool surface_set = false;

  // module arrays (device), indexed by les_field
  double* f[LES_NUM_FIELDS] = {};
  size_t fsize[LES_NUM_FIELDS] = {};
  double* reg[LES_NUM_FIELDS] = {};  // registered host arrays

  // derived surface plane
  double* z_os = nullptr;
  // spectral tables (lh,ny)
  double *kx = nullptr, *ky = nullptr, *G = nullptr, *GG = nullptr;
  float *kxf = nullptr, *kyf = nullptr, *Gf = nullptr, *GGf = nullptr;
  int ncG = 0, ncGG = 0;  // kx columns holding a nonzero G_test / G_test_test (the rest are zero)
  float2 *kxd = nullptr, *kyd = nullptr;  // kx, ky as float-float pairs
  // FFT plans
  les::HostRealPlan rx, rxb;   // real x-transforms of length nx, nx2
  les::HostPlan cy, cyb;       // complex y-transforms of length ny, ny2
  // scratch
  void* wsA = nullptr;  size_t wsA_bytes = 0;
  void* wsB = nullptr;  size_t wsB_bytes = 0;
  void* wsP = nullptr;  size_t wsP_bytes = 0;  // pressure spectra + gam
  double* big = nullptr;  int nbig = 0;        // big physical fields
  double* tmp = nullptr;  int ntmp = 0;        // small physical temp planes
  double* spare = nullptr;                     // 4 fields (interpolated F_*)
  double2* spec = nullptr;                     // U, V, W, Theta spectra F(u/(nx*ny)), (nz,ny,lh) each
  double2* wspec = nullptr;                    // wall-plane spectra: dudz(1), dvdz(1), dTdz(1), dTdz(nz)
  double* ibet = nullptr;                      // Thomas 1/bet per (row, mode), FP64
  double* gamt = nullptr;                      // Thomas gam per (row, mode), FP64
  float2* ibet_ff = nullptr;                   // the same two tables as float-float pairs (mixed form)
  float2* gamt_ff = nullptr;
  int* lowmodes = nullptr;                     // modes the mixed form solves in FP64 (kx^2 + ky^2 <= 4)
  int nlow = 0, nlow_cap = 0;
  int lag_chunk = 32;
  double* dscal = nullptr;                     // device scalars / reductions
  // per-level reduction results, 36 slots of nz+8 doubles: 0 plane sums /
  // rmsdiv partials / model-3 Cs(z); 2..11 scaledep sums; 12..13
  // timestep_conditions partial maxima; 14 theta, 15 qmix plane means
  // (mixed); 16..18 u, v, w plane means (mixed filt_da); 20..21 the (virtual)
  // theta level mean and its reciprocal (calcbeta); 24..27 partial plane sums;
  // 28..33 the mixed form's per-level mean-wind factors (float-float);
  // 34..35 the mixed form's txz, tyz plane means
  double* dred = nullptr;
  // running statistics (MM_XYZ_Out): 133 accumulators of nx ny (nz-1)
  double* stats = nullptr;
  int stats_c = 0, stats_p = 0, stats_auto = 0;
  double* host_scal = nullptr;                 // pinned host mirror
  size_t bytes = 0;
  std::vector<void*> allocs;
  double rmsdiv_last = 0.0;
  int status_flags = 0;
  // launch shapes chosen by the autotuner (0: built-in defaults)
  int tx64 = 0, tx32 = 0;       // kx columns per CTA of the y-pass kernels
  int rpc_scale = 0;            // rows per CTA of the x-pass kernels: default * 2^rpc_scale
  int rpc64 = 0, rpc32 = 0, rpcb64 = 0, rpcb32 = 0;   // resolved rows per CTA (small/big planes)
  // CUDA graphs of one step, by variant (dynamic-model step, Cs override)
  cudaGraphExec_t gexec[2][2][2] = {};  // [Lagrangian step][Cs^2 override][rhs_par]
  // The fused step takes RHS*_f = RHS* (main.f90:212-214) by exchanging the
  // two arrays' buffers instead of copying; rhs_par is the exchange parity
  // (a captured step graph holds the buffer addresses of one parity).
  int rhs_par = 0;
};

namespace les {
// An FP32-mixed context (precision 1) holds these SGS intermediates in FP32:
// the horizontal velocity and theta gradients (FP32 transforms), S_ij, Nu_t
// and tau_ij.  Each keeps its FP64 allocation and (ld, ny, nz) layout; the FP32
// values sit in the first half.  les_get_field / les_set_field convert.
inline bool mixed_f32_field(int f) {
  switch (f) {
    case LES_DUDX: case LES_DUDY: case LES_DVDX: case LES_DVDY: case LES_DWDX: case LES_DWDY:
    case LES_S11: case LES_S12: case LES_S13: case LES_S22: case LES_S23: case LES_S33:
    case LES_NU_T:
    case LES_TXX: case LES_TXY: case LES_TYY: case LES_TXZ: case LES_TYZ: case LES_TZZ:
    case LES_DTDX: case LES_DTDY: case LES_DQDX: case LES_DQDY:
      return true;
    default:
      return false;
  }
}
// humidity arrays: stored only when q_flag = 1
inline bool is_q_field(int f) {
  return (f >= LES_Q && f <= LES_DQDZ) || f == LES_WQ_S || f == LES_SGS_Q3_SFC;
}
// model 7 arrays: stored only when model = 7
inline bool is_m7_field(int f) { return f >= LES_G_LM && f <= LES_TN_QNNN; }
// An FP32-mixed context keeps the momentum right-hand sides (this step's
// and the previous step's) as float-float pairs: hi and lo floats in each
// 8-byte slot of the FP64 layout.  les_get_field / les_set_field convert.
inline bool mixed_ff_field(int f) {
  return f == LES_RHSX || f == LES_RHSY || f == LES_RHSZ || f == LES_RHSX_F || f == LES_RHSY_F || f == LES_RHSZ_F;
}
inline float2* ff2(les_ctx* c, int f) { return reinterpret_cast<float2*>(c->f[f]); }
inline float* f32(les_ctx* c, int f) { return reinterpret_cast<float*>(c->f[f]); }
void rhs_swap(les_ctx* c);  // exchange RHSx/RHSx_f, RHSy/.., RHSz/.., RHS_T/RHS_Tf (RHS_q/RHS_qf) buffers
int step_fp64(les_ctx* c);
int step_mixed(les_ctx* c);
int step_ff(les_ctx* c);  // precision 2: FP64 state and arithmetic, float-float transforms
int op_filt_da(les_ctx* c, double* f, double* dfdx, double* dfdy, int nlev);
int op_ddxy(les_ctx* c, double* dfdx, double* dfdy, const double* f, int nlev);
int op_test_filter(les_ctx* c, double* out, const double* in, int nplanes, int which, long pstride);
int op_dealias1(les_ctx* c, const double* const* in, double* const* out, int nf, int nlev);
int op_dealias2(les_ctx* c, double* const* out, const double* const* in, int nf, int nlev, double scale);
int op_fft(les_ctx* c, double* planes, int nplanes, int big, int inverse);
int op_rmsdiv_state(les_ctx* c, double* out_dev);
int op_cvt_selftest(size_t n, unsigned long long seed, unsigned long long* bad_dev, cudaStream_t s);
int op_tridag(les_ctx* c, const double* a, const double* b, const double* cc, const double* r, double* u);
void launch_tridag_generic(const double* a, const double* b, const double* cc, const double* r, double* u,
                           double* gam, int lh, int ny, int n, int* flag, cudaStream_t s);
int op_obukhov(les_ctx* c, const double* uv1 = nullptr);     // uv1: filtered surface u, v (null: filtered here)
int op_wallstress(les_ctx* c, const double* uv1 = nullptr);
int op_sgs_stag(les_ctx* c);
int op_lagrange(les_ctx* c, const double* const* S);
int op_interpolag(les_ctx* c);
int op_interpolag_n(les_ctx* c, int nf);  // nf 4: interpolag_Sdep, 2: interpolag_Ssim
int op_lagrange_ssim(les_ctx* c, const double* const* S);
int op_scaledep(les_ctx* c, double* cs_z_dev, const double* const* S);
int op_stddyn(les_ctx* c, double* cs_z_dev, const double* const* S);
int op_theta(les_ctx* c);
int op_q(les_ctx* c);
int op_thermo(les_ctx* c, double* const* out);  // 9 (ld,ny,nz) arrays, atm_thermodynamics.f90 order
int op_stats(les_ctx* c);                        // one MM_XYZ_Out accumulation (io.f90:403-866)
int op_lagrange_scalar(les_ctx* c, const double* const* S, double* cs2_pr);  // model 7 (cs2_pr may be null)
int op_interpolag_scalar(les_ctx* c);
int op_divstress(les_ctx* c, double* divtx, double* divty, double* divtz);
int op_divstress_one(les_ctx* c, double* divt, const double* tx, const double* ty, const double* tz, int w_variant);
int op_convec(les_ctx* c, double* cx, double* cy, double* cz);
int op_press(les_ctx* c, double* p, double* dpdx, double* dpdy);
int op_project(les_ctx* c);
int op_rmsdiv(les_ctx* c, double* out);
int op_tsc(les_ctx* c, double* cflu, double* visc);  // Nu_t read in the context's storage precision
int op_ddz(les_ctx* c, double* dfdz, const double* f, int uv);
int thomas_tables(les_ctx* c);
void autotune_probe(les_ctx* c, int fp32);
}  // namespace les
