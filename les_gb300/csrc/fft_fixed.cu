// Fixed-length FP32 and float-float instantiations of the transform
// kernels.  The launchers return false for lengths (or precisions) without an
// instantiation; the caller then launches the runtime-length kernel.
#include "fft_kernels.cuh"
#include "les_internal.h"

namespace les {
namespace {

template <typename K>
void raise_smem(K kernel, size_t sm, size_t& set) {
  if (sm > set) {  // opt-in raised once per instantiation (not during capture)
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    set = sm;
  }
}

template <typename T, typename TIn, int NF>
void r2c_fixed(const RowJob& J, const RealPlanDev& P, int rpc, cudaStream_t s) {
  typedef typename CT<T>::type C;
  const size_t smf = ((size_t)2 * rpc * skn(NF) + 2 * NF + 1) * sizeof(C);
  static size_t set = 48 * 1024;
  raise_smem(k_rows_r2c<T, TIn, NF>, smf, set);
  const dim3 grid((J.ny + rpc - 1) / rpc, J.nlev, J.nfield);
  k_rows_r2c<T, TIn, NF><<<grid, 256, smf, s>>>(J, P, rpc);
}
template <typename T, typename TOut, int NF>
void c2r_fixed(const RowJob& J, const RealPlanDev& P, int rpc, cudaStream_t s) {
  typedef typename CT<T>::type C;
  const size_t smf = ((size_t)rpc * (NF + 1) + (size_t)2 * rpc * skn(NF) + 2 * NF + 1) * sizeof(C);
  static size_t set = 48 * 1024;
  raise_smem(k_rows_c2r<T, TOut, NF>, smf, set);
  const dim3 grid((J.ny + rpc - 1) / rpc, J.nlev, J.nfield);
  k_rows_c2r<T, TOut, NF><<<grid, 256, smf, s>>>(J, P, rpc);
}
template <typename T, int TX, typename CIn, int NIN, int NOUT>
void cols_fixed(const ColJob& J, const FftPlanDev& Pin, const FftPlanDev& Pout, dim3 grid, cudaStream_t s) {
  typedef typename CT<T>::type C;
  constexpr int PMAX = skn(NIN > NOUT ? NIN : NOUT);
  const size_t smf = ((size_t)(J.nin * skn(NIN) + 2 * PMAX) * TX + NIN + NOUT) * sizeof(C);
  static size_t set = 48 * 1024;
  raise_smem(k_colsf<T, TX, CIn, NIN, NOUT>, smf, set);
  k_colsf<T, TX, CIn, NIN, NOUT><<<grid, 256, smf, s>>>(J, Pin, Pout);
}

}  // namespace

// x pass: half lengths m = nx/2 of the small and 3/2 grids of nx in
// {32, 48, 64, 96, 128, 192, 256, 384}
#define LES_ROW_SIZES(X) X(16) X(24) X(32) X(48) X(64) X(72) X(96) X(128) X(144) X(192)

template <typename T, typename TIn>
bool launch_rows_r2c_fixed(const RowJob& J, const RealPlanDev& P, int rpc, size_t sm, cudaStream_t s) {
  if constexpr (std::is_same<T, double>::value) {
    return false;
  } else {
    switch (P.nx / 2) {
#define LES_CASE(n) \
  case n: r2c_fixed<T, TIn, n>(J, P, rpc, s); return true;
      LES_ROW_SIZES(LES_CASE)
#undef LES_CASE
      default: return false;
    }
  }
}
template <typename T, typename TOut>
bool launch_rows_c2r_fixed(const RowJob& J, const RealPlanDev& P, int rpc, size_t sm, cudaStream_t s) {
  if constexpr (std::is_same<T, double>::value) {
    return false;
  } else {
    switch (P.nx / 2) {
#define LES_CASE(n) \
  case n: c2r_fixed<T, TOut, n>(J, P, rpc, s); return true;
      LES_ROW_SIZES(LES_CASE)
#undef LES_CASE
      default: return false;
    }
  }
}

// y pass: (ny_in, ny_out) = (ny, ny), (ny, 3ny/2) padding, (3ny/2, ny)
// unpadding, for ny in {32, 64, 96, 128, 192, 256}; kx tile 8, FP32 input
#define LES_COL_PAIRS(X)                                                              \
  X(32, 32) X(32, 48) X(48, 32) X(64, 64) X(64, 96) X(96, 64) X(96, 96) X(96, 144)   \
  X(144, 96) X(128, 128) X(128, 192) X(192, 128) X(192, 192) X(192, 288) X(288, 192) \
  X(256, 256) X(256, 384) X(384, 256)

// padding from the saved spectra: (ny, 3ny/2)
#define LES_COL_PAD(X) X(32, 48) X(64, 96) X(96, 144) X(128, 192) X(192, 288) X(256, 384)

// float-float y pass (the projection path): same-length pairs, kx tile 4
#define LES_COL_SAME(X) X(32, 32) X(64, 64) X(96, 96) X(128, 128) X(192, 192) X(256, 256)

template <typename T, int TX, typename CIn>
bool launch_cols_fixed(const ColJob& J, const FftPlanDev& Pin, const FftPlanDev& Pout, size_t sm, dim3 grid,
                       cudaStream_t s) {
  const int key = J.ny_in * 10000 + J.ny_out;
  if constexpr (std::is_same<T, float>::value && TX == 8 && std::is_same<CIn, float2>::value) {
    switch (key) {
#define LES_CASE(a, b) \
  case a * 10000 + b: cols_fixed<T, TX, CIn, a, b>(J, Pin, Pout, grid, s); return true;
      LES_COL_PAIRS(LES_CASE)
#undef LES_CASE
      default: return false;
    }
  } else if constexpr (std::is_same<T, float>::value && TX == 8 && std::is_same<CIn, double2>::value) {
    switch (key) {  // FP32 transforms of the saved FP64-layout spectra (padding to the 3/2 grid)
#define LES_CASE(a, b) \
  case a * 10000 + b: cols_fixed<T, TX, CIn, a, b>(J, Pin, Pout, grid, s); return true;
      LES_COL_PAD(LES_CASE)
#undef LES_CASE
      default: return false;
    }
  } else if constexpr (std::is_same<T, dfloat>::value && TX == 4 && std::is_same<CIn, dcomplex>::value) {
    switch (key) {
#define LES_CASE(a, b) \
  case a * 10000 + b: cols_fixed<T, TX, CIn, a, b>(J, Pin, Pout, grid, s); return true;
      LES_COL_SAME(LES_CASE)
#undef LES_CASE
      default: return false;
    }
  } else {
    return false;
  }
}

template bool launch_rows_r2c_fixed<double, double>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_r2c_fixed<float, float>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_r2c_fixed<float, double>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_c2r_fixed<double, double>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_c2r_fixed<float, float>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_c2r_fixed<float, double>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_r2c_fixed<dfloat, double>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_c2r_fixed<dfloat, double>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
#define LES_INST_COLS(T, TX, CIn)                                                                   \
  template bool launch_cols_fixed<T, TX, CIn>(const ColJob&, const FftPlanDev&, const FftPlanDev&, \
                                              size_t, dim3, cudaStream_t);
LES_INST_COLS(double, 2, double2)
LES_INST_COLS(double, 4, double2)
LES_INST_COLS(double, 8, double2)
LES_INST_COLS(float, 4, float2)
LES_INST_COLS(float, 8, float2)
LES_INST_COLS(float, 16, float2)
LES_INST_COLS(float, 4, double2)
LES_INST_COLS(float, 8, double2)
LES_INST_COLS(float, 16, double2)
LES_INST_COLS(dfloat, 2, dcomplex)
LES_INST_COLS(dfloat, 4, dcomplex)
LES_INST_COLS(dfloat, 8, dcomplex)

}  // namespace les
