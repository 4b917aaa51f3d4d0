// Batched plane FFT kernels (rows_r2c, cols, rows_c2r); see fft.cuh.
#include "fft_kernels.cuh"
#include "les_internal.h"

namespace les {

// ---------------------------------------------------------------------------
// host launchers

template <typename T, typename TIn>
int launch_rows_r2c(const RowJob& J, const RealPlanDev& P, cudaStream_t s) {
  typedef typename CT<T>::type C;
  const int rpc = J.rpc > 0 ? J.rpc : rows_pc<T>(P.nx);
  const size_t sm = (size_t)2 * rpc * (P.nx / 2) * sizeof(C);
  RowJob JJ = J;
  JJ.dnc = FastDiv((unsigned)J.ncols);
  dim3 grid((J.ny + rpc - 1) / rpc, J.nlev, J.nfield);
  const bool pr = g_prof && prof_mark(sizeof(T) == 8 ? PROF_ROWS64 : PROF_ROWS32, s);
  if (!launch_rows_r2c_fixed<T, TIn>(JJ, P, rpc, sm, s)) {
    static size_t sm_set = 48 * 1024;  // opt-in raised once per instantiation (not during capture)
    if (sm > sm_set) {
      cudaFuncSetAttribute(k_rows_r2c<T, TIn, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      sm_set = sm;
    }
    k_rows_r2c<T, TIn, 0><<<grid, 256, sm, s>>>(JJ, P, rpc);
  }
  LES_COUNT_LAUNCH();
  if (pr)
    prof_done(s, (double)J.nfield * J.nlev * J.ny * ((double)P.nx * sizeof(TIn) + (double)J.ncols * sizeof(C)));
  return 0;
}

template <typename T, typename TOut>
int launch_rows_c2r(const RowJob& J, const RealPlanDev& P, cudaStream_t s) {
  typedef typename CT<T>::type C;
  const int rpc = J.rpc > 0 ? J.rpc : rows_pc<T>(P.nx);
  const int m = P.nx / 2;
  const size_t sm = (size_t)rpc * ((m + 1) + 2 * m) * sizeof(C);
  dim3 grid((J.ny + rpc - 1) / rpc, J.nlev, J.nfield);
  const bool pr = g_prof && prof_mark(sizeof(T) == 8 ? PROF_ROWS64 : PROF_ROWS32, s);
  if (!launch_rows_c2r_fixed<T, TOut>(J, P, rpc, sm, s)) {
    static size_t sm_set = 48 * 1024;  // opt-in raised once per instantiation (not during capture)
    if (sm > sm_set) {
      cudaFuncSetAttribute(k_rows_c2r<T, TOut, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      sm_set = sm;
    }
    k_rows_c2r<T, TOut, 0><<<grid, 256, sm, s>>>(J, P, rpc);
  }
  LES_COUNT_LAUNCH();
  if (pr)
    prof_done(s, (double)J.nfield * J.nlev * J.ny * ((double)J.ncols * sizeof(C) + (double)J.ld * sizeof(TOut)));
  return 0;
}

template <typename T, int TX, typename CIn>
static int launch_cols_tx(const ColJob& J, const FftPlanDev& Pin, const FftPlanDev& Pout, cudaStream_t s) {
  typedef typename CT<T>::type C;
  const int nymax = J.ny_in > J.ny_out ? J.ny_in : J.ny_out;
  const size_t sm = (size_t)(J.nin * J.ny_in + 2 * nymax) * TX * sizeof(C);
  dim3 grid((J.ncols + TX - 1) / TX, J.nlev, J.nf > 0 ? J.nf : 1);
  const bool pr = g_prof && prof_mark(sizeof(T) == 8 ? PROF_COLS64 : PROF_COLS32, s);
  if (!launch_cols_fixed<T, TX, CIn>(J, Pin, Pout, sm, grid, s)) {
    static size_t sm_set = 48 * 1024;  // opt-in raised once per instantiation (not during capture)
    if (sm > sm_set) {
      cudaFuncSetAttribute(k_cols<T, TX, CIn>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      sm_set = sm;
    }
    k_cols<T, TX, CIn><<<grid, 256, sm, s>>>(J, Pin, Pout);
  }
  LES_COUNT_LAUNCH();
  if (pr) {
    const double nf = J.nf > 0 ? J.nf : 1;
    prof_done(s, nf * J.nlev * J.ncols *
                     ((double)J.nin * J.ny_in * sizeof(CIn) + (double)J.nout * J.ny_out * sizeof(C)));
  }
  return 0;
}

// kx tile width: 8-byte reals (FP64, float-float) {2, 4, 8} (default 4),
// FP32 {4, 8, 16} (default 8); the autotuner picks one per grid size
template <typename T, typename CIn>
int launch_cols(const ColJob& J, const FftPlanDev& Pin, const FftPlanDev& Pout, cudaStream_t s) {
  if (sizeof(T) == 8) {
    switch (J.tx) {
      case 2: return launch_cols_tx<T, 2, CIn>(J, Pin, Pout, s);
      case 8: return launch_cols_tx<T, 8, CIn>(J, Pin, Pout, s);
      default: return launch_cols_tx<T, 4, CIn>(J, Pin, Pout, s);
    }
  } else {
    switch (J.tx) {
      case 4: return launch_cols_tx<T, 4, CIn>(J, Pin, Pout, s);
      case 16: return launch_cols_tx<T, 16, CIn>(J, Pin, Pout, s);
      default: return launch_cols_tx<T, 8, CIn>(J, Pin, Pout, s);
    }
  }
}

template int launch_rows_r2c<double, double>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_rows_c2r<double, double>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_cols<double, double2>(const ColJob&, const FftPlanDev&, const FftPlanDev&, cudaStream_t);
template int launch_rows_r2c<float, float>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_rows_r2c<float, double>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_rows_c2r<float, float>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_rows_c2r<float, double>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_cols<float, float2>(const ColJob&, const FftPlanDev&, const FftPlanDev&, cudaStream_t);
template int launch_cols<float, double2>(const ColJob&, const FftPlanDev&, const FftPlanDev&, cudaStream_t);
template int launch_rows_r2c<dfloat, double>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_rows_r2c<dfloat, dfloat>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_rows_c2r<dfloat, double>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_rows_c2r<dfloat, dfloat>(const RowJob&, const RealPlanDev&, cudaStream_t);
template int launch_cols<dfloat, dcomplex>(const ColJob&, const FftPlanDev&, const FftPlanDev&, cudaStream_t);
template int launch_cols<dfloat, double2>(const ColJob&, const FftPlanDev&, const FftPlanDev&, cudaStream_t);

}  // namespace les
