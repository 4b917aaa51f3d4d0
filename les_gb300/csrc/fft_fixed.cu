// Fixed-length FP32 and float-float instantiations of the transform
// kernels.  The launchers return false for lengths (or precisions) without an
// instantiation; the caller then launches the runtime-length kernel.
#include <algorithm>
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

// register-resident x pass (FP32): factors (N1, N2) of the half length M,
// 0 when the length has none
template <int M> struct RowSplit { static constexpr int n1 = 0, n2 = 0; };
template <> struct RowSplit<32> { static constexpr int n1 = 8, n2 = 4; };
template <> struct RowSplit<48> { static constexpr int n1 = 16, n2 = 3; };
template <> struct RowSplit<192> { static constexpr int n1 = 16, n2 = 12; };
template <typename T, int N1, int N2>
struct RegRows {
  static constexpr int TT = N1 > N2 ? N1 : N2;
  static constexpr int RPB = 256 / TT, NT = RPB * TT, M = N1 * N2;
  static size_t smem() { return (size_t)(RPB * N2 * (N1 + 1) + 2 * M + 1) * sizeof(typename CT<T>::type); }
};

// FP32 x pass, half length 128 = 16 x 8 with eight threads per row (every
// lane busy in both steps).  The float-float x pass keeps the shared-memory
// kernels: this form in float-float takes 128 registers (two CTAs per SM)
// and made the 256^3 steps slower (FP32-mixed 13.10 -> 13.23 ms, float-float
// transform form 36.9 -> 37.5 ms).
template <typename T, int NF> struct RowSplit2 { static constexpr int n1 = 0, n2 = 0, tt = 0; };
template <> struct RowSplit2<float, 128> { static constexpr int n1 = 16, n2 = 8, tt = 8; };
template <typename T, int N1, int N2, int TT>
struct RegRows2 {
  static constexpr int NT = 256, RPB = NT / TT, M = N1 * N2;
  static size_t smem() { return (size_t)(RPB * N2 * (N1 + 1) + 2 * M + 1) * sizeof(typename CT<T>::type); }
};

template <typename T, typename TIn, int NF>
void r2c_fixed(const RowJob& J, const RealPlanDev& P, int rpc, cudaStream_t s) {
  typedef typename CT<T>::type C;
  constexpr int A1 = RowSplit2<T, NF>::n1, A2 = RowSplit2<T, NF>::n2, AT = RowSplit2<T, NF>::tt;
  if constexpr (A1 > 0) {
    typedef RegRows2<T, A1, A2, AT> G;
    static size_t set2 = 48 * 1024;
    raise_smem(k_r2c_reg2<T, TIn, A1, A2, AT, G::NT>, G::smem(), set2);
    const dim3 grid((J.ny + G::RPB - 1) / G::RPB, J.nlev, J.nfield);
    k_r2c_reg2<T, TIn, A1, A2, AT, G::NT><<<grid, G::NT, G::smem(), s>>>(J, P);
    return;
  }
  constexpr int N1 = RowSplit<NF>::n1, N2 = RowSplit<NF>::n2;
  if constexpr (N1 > 0 && std::is_same<T, float>::value) {
    typedef RegRows<T, N1, N2> G;
    static size_t set = 48 * 1024;
    raise_smem(k_r2c_reg<T, TIn, N1, N2, G::NT>, G::smem(), set);
    const dim3 grid((J.ny + G::RPB - 1) / G::RPB, J.nlev, J.nfield);
    k_r2c_reg<T, TIn, N1, N2, G::NT><<<grid, G::NT, G::smem(), s>>>(J, P);
    return;
  }
  const size_t smf = ((size_t)2 * rpc * skn(NF) + 2 * NF + 1) * sizeof(C);
  static size_t set = 48 * 1024;
  raise_smem(k_rows_r2c<T, TIn, NF>, smf, set);
  const dim3 grid((J.ny + rpc - 1) / rpc, J.nlev, J.nfield);
  k_rows_r2c<T, TIn, NF><<<grid, 256, smf, s>>>(J, P, rpc);
}
template <typename T, typename TOut, int NF>
void c2r_fixed(const RowJob& J, const RealPlanDev& P, int rpc, cudaStream_t s) {
  typedef typename CT<T>::type C;
  constexpr int A1 = RowSplit2<T, NF>::n1, A2 = RowSplit2<T, NF>::n2, AT = RowSplit2<T, NF>::tt;
  if constexpr (A1 > 0) {
    typedef RegRows2<T, A1, A2, AT> G;
    static size_t set2 = 48 * 1024;
    raise_smem(k_c2r_reg2<T, TOut, A1, A2, AT, G::NT>, G::smem(), set2);
    const dim3 grid((J.ny + G::RPB - 1) / G::RPB, J.nlev, J.nfield);
    k_c2r_reg2<T, TOut, A1, A2, AT, G::NT><<<grid, G::NT, G::smem(), s>>>(J, P);
    return;
  }
  constexpr int N1 = RowSplit<NF>::n1, N2 = RowSplit<NF>::n2;
  if constexpr (N1 > 0 && std::is_same<T, float>::value) {
    typedef RegRows<T, N1, N2> G;
    static size_t set = 48 * 1024;
    raise_smem(k_c2r_reg<T, TOut, N1, N2, G::NT>, G::smem(), set);
    const dim3 grid((J.ny + G::RPB - 1) / G::RPB, J.nlev, J.nfield);
    k_c2r_reg<T, TOut, N1, N2, G::NT><<<grid, G::NT, G::smem(), s>>>(J, P);
    return;
  }
  const size_t smf = ((size_t)rpc * (NF + 1) + (size_t)2 * rpc * skn(NF) + 2 * NF + 1) * sizeof(C);
  static size_t set = 48 * 1024;
  raise_smem(k_rows_c2r<T, TOut, NF>, smf, set);
  const dim3 grid((J.ny + rpc - 1) / rpc, J.nlev, J.nfield);
  k_rows_c2r<T, TOut, NF><<<grid, 256, smf, s>>>(J, P, rpc);
}
// register-resident y pass (FP32, one input, same length N = R * R), 16 kx
// columns per CTA.  The float-float transforms keep the shared-memory
// kernels: their arithmetic is heavy enough that the idle lanes and the
// register pressure of the register-resident form cost more than they save.
template <typename T, typename CIn, int R>
void cols_reg(const ColJob& J, const FftPlanDev& P, cudaStream_t s) {
  typedef typename CT<T>::type C;
  constexpr int TX = 16, N = R * R;
  const size_t smf = (size_t)N * TX * (sizeof(C) + sizeof(CIn)) + (size_t)N * (sizeof(C) + sizeof(T));
  static size_t set = 48 * 1024;
  raise_smem(k_colsr<T, TX, CIn, R>, smf, set);
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 1;
  }
  // lh = nx/2 + 1 columns leave one column in the last tile of each
  // (level, field) set.  Packing those columns of sixteen sets into one item
  // made the FP32 y pass slower in the 256^3 step (2.21 -> 2.33 ms), so the
  // last tile stays one item per set.
  const int ntile = (J.ncols + TX - 1) / TX;
  const int nitems = ntile * J.nlev * (J.nf > 0 ? J.nf : 1);
  const int nblk = std::min(nitems, 3 * nsm);  // three resident CTAs per SM (registers, shared memory)
  k_colsr<T, TX, CIn, R><<<nblk, TX * R, smf, s>>>(J, P, ntile, nitems);
}

// several inputs summed into at most two outputs, same length N = R * R
template <typename T, typename CIn, int R>
void cols_reg_sum(const ColJob& J, const FftPlanDev& P, cudaStream_t s) {
  typedef typename CT<T>::type C;
  constexpr int TX = 16, N = R * R;
  const size_t smf = (size_t)(3 * N * TX + N) * sizeof(C) + (size_t)N * sizeof(T);
  static size_t set = 48 * 1024;
  raise_smem(k_colsr_sum<T, TX, CIn, R, 2>, smf, set);
  const dim3 grid((J.ncols + TX - 1) / TX, J.nlev, J.nf > 0 ? J.nf : 1);
  k_colsr_sum<T, TX, CIn, R, 2><<<grid, TX * R, smf, s>>>(J, P);
}

// register-resident 3/2 padding / truncation (FP32), 16 kx columns per CTA
template <typename T, typename CIn, int NIN, int NOUT>
void cols_pad(const ColJob& J, const FftPlanDev& Pin, const FftPlanDev& Pout, cudaStream_t s) {
  typedef typename CT<T>::type C;
  typedef PadShape<NIN, NOUT> PS;
  constexpr int TX = 16;
  const size_t smf = (size_t)(16 * PS::b * TX + PS::ns + PS::nb) * sizeof(C);
  static size_t set = 48 * 1024;
  raise_smem(k_colsr_pad<T, TX, CIn, NIN, NOUT>, smf, set);
  const dim3 grid((J.ncols + TX - 1) / TX, J.nlev, J.nf > 0 ? J.nf : 1);
  k_colsr_pad<T, TX, CIn, NIN, NOUT><<<grid, TX * PS::tt, smf, s>>>(J, Pin, Pout);
}

template <typename T, int TX, typename CIn, int NIN, int NOUT>
void cols_fixed(const ColJob& J, const FftPlanDev& Pin, const FftPlanDev& Pout, dim3 grid, cudaStream_t s) {
  typedef typename CT<T>::type C;
  if constexpr (NIN == NOUT && (NIN == 256 || NIN == 64) && std::is_same<T, float>::value) {
    if (J.nin == 1 && J.map == MAP_SAME) {
      cols_reg<T, CIn, NIN == 256 ? 16 : 8>(J, Pin, s);
      return;
    }
    if (J.nin > 1 && J.nout <= 2 && J.map == MAP_SAME) {
      cols_reg_sum<T, CIn, NIN == 256 ? 16 : 8>(J, Pin, s);
      return;
    }
  }
  if constexpr (std::is_same<T, float>::value && NIN != NOUT &&
                ((NIN < NOUT ? NIN : NOUT) == 256 || (NIN < NOUT ? NIN : NOUT) == 128)) {
    const bool pad = NOUT > NIN;
    if (J.nin == 1 && J.nout == 1 && J.coef[0][0] == CC_ONE && (J.inv_mask & 1u) &&
        J.map == (pad ? MAP_PAD : MAP_UNPAD) && J.ny_small == (pad ? NIN : NOUT) && (pad || (J.dir & DIR_FWD))) {
      cols_pad<T, CIn, NIN, NOUT>(J, Pin, Pout, s);
      return;
    }
  }
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
// float-float 3/2 padding and truncation (the float-float transform form's
// convective and scalar terms), kx tile 4
#define LES_COL_FF_PAD(X) X(32, 48) X(64, 96) X(96, 144) X(128, 192) X(192, 288) X(256, 384)
#define LES_COL_FF_UNPAD(X) X(48, 32) X(96, 64) X(144, 96) X(192, 128) X(288, 192) X(384, 256)

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
      LES_COL_FF_PAD(LES_CASE)
      LES_COL_FF_UNPAD(LES_CASE)
#undef LES_CASE
      default: return false;
    }
  } else if constexpr (std::is_same<T, dfloat>::value && TX == 4 && std::is_same<CIn, double2>::value) {
    switch (key) {  // float-float transforms of the saved FP64 spectra (same length, and padding)
#define LES_CASE(a, b) \
  case a * 10000 + b: cols_fixed<T, TX, CIn, a, b>(J, Pin, Pout, grid, s); return true;
      LES_COL_SAME(LES_CASE)
      LES_COL_FF_PAD(LES_CASE)
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
template bool launch_rows_r2c_fixed<dfloat, dfloat>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_c2r_fixed<dfloat, double>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
template bool launch_rows_c2r_fixed<dfloat, dfloat>(const RowJob&, const RealPlanDev&, int, size_t, cudaStream_t);
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
LES_INST_COLS(dfloat, 2, double2)
LES_INST_COLS(dfloat, 4, double2)
LES_INST_COLS(dfloat, 8, double2)

}  // namespace les
