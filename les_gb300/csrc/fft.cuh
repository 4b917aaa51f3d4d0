// Batched shared-memory Stockham FFTs for the horizontal planes of the LES
// fields.  They replace FFTW 2's in-place 2-D real transforms
// (rfftwnd_f77_one_real_to_complex / complex_to_real with the plans of
// fft.f90:40-47): unnormalised, forward sign -1, x (the contiguous Fortran
// dimension) is the halved real dimension, complex output (lh,ny) over an
// (ld,ny) plane.  A 2-D transform is split into
//   rows_r2c  : real x-FFT of every row (length nx through an nx/2 complex FFT)
//   cols      : complex y-FFT of tiles of kx columns, with a spectral operator
//               between the forward and inverse passes (derivatives, test
//               filters, 3/2 zero padding / truncation, oddball removal)
//   rows_c2r  : real inverse x-FFT of every row
// so that one launch of each kernel processes every level of several fields.
// Sizes are 2^a 3^b (radix 4, 2, 3 stages).
#pragma once
#include "common.cuh"

namespace les {

constexpr int FFT_MAX_STAGES = 12;

// q = n / d by one multiply-high: with inv = ceil(2^32/d) = (2^32 + e)/d,
// 0 <= e < d, umulhi(n, inv) = floor(n/d + n*e/(d*2^32)), which is exact
// while n*e < 2^32.  Plans are limited to lengths <= 4096 and thread indices
// stay below 2^20, so n*d < 2^32 holds everywhere it is used.
struct FastDiv {
  unsigned inv;  // ceil(2^32 / d)
  unsigned d;
  __host__ __device__ FastDiv() : inv(0), d(1) {}
  __host__ FastDiv(unsigned dd) : inv((unsigned)((((unsigned long long)1 << 32) + dd - 1) / dd)), d(dd) {}
  __device__ __forceinline__ unsigned div(unsigned n) const { return d == 1 ? n : __umulhi(n, inv); }
  __device__ __forceinline__ unsigned mod(unsigned n) const { return n - div(n) * d; }
};

struct FftPlanDev {
  int n;
  int nst;
  int radix[FFT_MAX_STAGES];
  int twoff[FFT_MAX_STAGES];
  FastDiv dm[FFT_MAX_STAGES];   // n / radix of each stage (butterflies per transform)
  FastDiv dns[FFT_MAX_STAGES];  // Ns of each stage (product of the previous radices)
  const double2* tw;  // forward twiddles, per stage (R-1)*Ns entries
  const float2* twf;  // the same rounded to FP32 (FP32 kernels read these: a
                      // double->float conversion runs on GB300's FP64 pipe)
  const float4* twd;  // the same as float-float pairs (re.hi, re.lo, im.hi, im.lo)
  const float2* unitf;  // exp(-2 pi i m / n), m < n, in FP32 (fixed-length kernels)
  const float4* unitd;  // the same as float-float pairs
};

struct RealPlanDev {
  FftPlanDev c;       // complex FFT of length m = nx/2
  int nx;
  FastDiv dm, dm1;    // m and m + 1
  const double2* w;   // exp(-2 pi i k / nx), k = 0..m
  const float2* wf;   // the same in FP32
  const float4* wd;   // the same as float-float pairs
};

// ---- radix butterflies -----------------------------------------------------
template <typename C> __device__ __forceinline__ void dft2(C* v) {
  C a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}
template <typename C> __device__ __forceinline__ void dft4(C* v, int sign) {
  C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  C t2 = cadd(v[1], v[3]), d = csub(v[1], v[3]);
  C t3 = sign < 0 ? cmulmi(d) : cmuli(d);
  v[0] = cadd(t0, t2);
  v[1] = cadd(t1, t3);
  v[2] = csub(t0, t2);
  v[3] = csub(t1, t3);
}
template <typename C, typename T> __device__ __forceinline__ void dft3(C* v, int sign) {
  const T s3 = (T)0.86602540378443864676372317075294;
  C a0 = v[0];
  C sum = cadd(v[1], v[2]), dif = csub(v[1], v[2]);
  C m = csub(a0, cscale(sum, (T)0.5));
  const T ss = sign < 0 ? -s3 : s3;
  C rot; rot.x = -ss * dif.y; rot.y = ss * dif.x;
  v[0] = cadd(a0, sum);
  v[1] = cadd(m, rot);
  v[2] = csub(m, rot);
}

template <typename T> struct TwSel;
template <> struct TwSel<double> {
  static __device__ __forceinline__ double2 get(const FftPlanDev& P, int idx) { return __ldg(&P.tw[idx]); }
};
template <> struct TwSel<float> {
  static __device__ __forceinline__ float2 get(const FftPlanDev& P, int idx) { return __ldg(&P.twf[idx]); }
};
template <> struct TwSel<dfloat> {
  static __device__ __forceinline__ dcomplex get(const FftPlanDev& P, int idx) {
    const float4 v = __ldg(&P.twd[idx]);
    dcomplex r;
    r.x = dfloat(v.x, v.y);
    r.y = dfloat(v.z, v.w);
    return r;
  }
};
template <typename T> __device__ __forceinline__ typename CT<T>::type twid(const FftPlanDev& P, int idx, int sign) {
  typename CT<T>::type w = TwSel<T>::get(P, idx);
  if (sign > 0) w.y = -w.y;
  return w;
}

// One Stockham pass over all batches.  Element (b, i) lives at
//   COLS : x[i * nb + b]          (tiles of columns, b fastest)
//   ROWS : x[b * bstride + i]     (rows, i fastest)
template <typename T, bool COLS>
__device__ __forceinline__ void fft_pass(const typename CT<T>::type* __restrict__ x,
                                         typename CT<T>::type* __restrict__ y, int n, int nb,
                                         int bstride, int R, int Ns, const FftPlanDev& P, int st, int sign) {
  typedef typename CT<T>::type C;
  const int m = n / R;
  const int total = m * nb;
  const int toff = P.twoff[st];
  const FastDiv dm = P.dm[st], dns = P.dns[st];
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int b, j;
    if (COLS) { b = t % nb; j = t / nb; }  // nb is a compile-time tile width at the call sites
    else { b = (int)dm.div((unsigned)t); j = t - b * m; }
    const int jq = (int)dns.div((unsigned)j);
    const int k = j - jq * Ns;
    C v[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (r < R) v[r] = COLS ? x[(j + r * m) * nb + b] : x[b * bstride + j + r * m];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < 4; ++r)
        if (r < R) v[r] = cmul(v[r], twid<T>(P, toff + (r - 1) * Ns + k, sign));
    }
    if (R == 4) dft4(v, sign);
    else if (R == 2) dft2(v);
    else dft3<C, T>(v, sign);
    const int base = jq * Ns * R + k;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (r < R) {
        if (COLS) y[(base + r * Ns) * nb + b] = v[r];
        else y[b * bstride + base + r * Ns] = v[r];
      }
  }
}

// Full transform; returns the buffer holding the result (x or y).
template <typename T, bool COLS>
__device__ typename CT<T>::type* fft_smem(typename CT<T>::type* x, typename CT<T>::type* y, int nb,
                                          int bstride, const FftPlanDev& P, int sign) {
  int Ns = 1;
  for (int s = 0; s < P.nst; ++s) {
    const int R = P.radix[s];
    fft_pass<T, COLS>(x, y, P.n, nb, bstride, R, Ns, P, s, sign);
    __syncthreads();
    typename CT<T>::type* t = x; x = y; y = t;
    Ns *= R;
  }
  return x;
}

// ---- fixed-length transforms -------------------------------------------------
// Stockham passes with the length known at compile time: every index,
// butterfly count and twiddle offset is a constant; the butterflies are
// radix 16 (4 x 4), 8 (4 x 2), 4, 2 and 3, evaluated in registers, so a
// 256-point transform takes two passes through shared memory; twiddles come
// from a unit-circle table exp(-2 pi i m / N), m < N, staged in shared
// memory.  Shared-memory element i of a transform sits at sk(i) = i + i/16,
// which spreads the stride-16 accesses of the radix-16 passes over the
// banks.  Used for the FP32 and float-float kernels at the lengths the
// workloads use; other lengths take the runtime path above.
__host__ __device__ constexpr int sk(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int skn(int n) { return n + (n >> 4); }  // padded length
constexpr int ct2_radix(int n, int s, int maxr) {
  int m = n, st = 0;
  while (m > 1) {
    int r = 0;
    if (maxr >= 16 && m % 16 == 0) r = 16;
    else if (maxr >= 8 && m % 8 == 0) r = 8;
    else if (m % 4 == 0) r = 4;
    else if (m % 2 == 0) r = 2;
    else if (m % 3 == 0) r = 3;
    else return 0;
    if (st == s) return r;
    m /= r;
    ++st;
  }
  return 0;
}
constexpr bool ct_ok(int n) { return ct2_radix(n, 0, 4) != 0 || n == 1; }

template <typename C, typename T> __device__ __forceinline__ C cmulc(C a, T wr, T wi) {
  C r;
  r.x = a.x * wr - a.y * wi;
  r.y = a.x * wi + a.y * wr;
  return r;
}
// natural-order DFT8 (r = 2a + b: two DFT4 over a, twiddles W8^c, DFT2 over b)
template <typename C, typename T> __device__ __forceinline__ void dft8(C* v, int sign) {
  const T c2 = (T)0.70710678118654752440084436210485;
  const T sc2 = sign < 0 ? -c2 : c2;
  C e[4] = {v[0], v[2], v[4], v[6]};
  C o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e, sign);
  dft4(o, sign);
  o[1] = cmulc(o[1], c2, sc2);
  o[2] = sign < 0 ? cmulmi(o[2]) : cmuli(o[2]);
  o[3] = cmulc(o[3], -c2, sc2);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    v[c] = cadd(e[c], o[c]);
    v[c + 4] = csub(e[c], o[c]);
  }
}
// natural-order DFT16 (r = 4a + b: four DFT4 over a, twiddles W16^(bc),
// four DFT4 over b; output q = c + 4d)
template <typename C, typename T> __device__ __forceinline__ void dft16(C* v, int sign) {
  const T c1 = (T)0.92387953251128675612818318939679;  // cos(pi/8)
  const T s1 = (T)0.38268343236508977172845998403040;  // sin(pi/8)
  const T c2 = (T)0.70710678118654752440084436210485;  // cos(pi/4)
  const T gs1 = sign < 0 ? -s1 : s1, gc1 = sign < 0 ? -c1 : c1, gc2 = sign < 0 ? -c2 : c2;
  C t[4][4];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    t[b][0] = v[b]; t[b][1] = v[b + 4]; t[b][2] = v[b + 8]; t[b][3] = v[b + 12];
    dft4(t[b], sign);
  }
  t[1][1] = cmulc(t[1][1], c1, gs1);   // W16^1
  t[1][2] = cmulc(t[1][2], c2, gc2);   // W16^2
  t[1][3] = cmulc(t[1][3], s1, gc1);   // W16^3
  t[2][1] = cmulc(t[2][1], c2, gc2);   // W16^2
  t[2][2] = sign < 0 ? cmulmi(t[2][2]) : cmuli(t[2][2]);  // W16^4
  t[2][3] = cmulc(t[2][3], -c2, gc2);  // W16^6
  t[3][1] = cmulc(t[3][1], s1, gc1);   // W16^3
  t[3][2] = cmulc(t[3][2], -c2, gc2);  // W16^6
  t[3][3] = cmulc(t[3][3], -c1, -gs1);  // W16^9
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    C u[4] = {t[0][c], t[1][c], t[2][c], t[3][c]};
    dft4(u, sign);
    v[c] = u[0]; v[c + 4] = u[1]; v[c + 8] = u[2]; v[c + 12] = u[3];
  }
}

// natural-order DFT12 (n = a + 4b: four DFT3 over b, twiddles W12^(ac),
// three DFT4 over a; output k = c + 3d)
template <typename C, typename T> __device__ __forceinline__ void dft12(C* v, int sign) {
  const T h = (T)0.5;
  const T s3 = (T)0.86602540378443864676372317075294;  // sin(pi/3)
  const T gh = sign < 0 ? -h : h, gs3 = sign < 0 ? -s3 : s3;
  C t[4][3];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    t[a][0] = v[a]; t[a][1] = v[a + 4]; t[a][2] = v[a + 8];
    dft3<C, T>(t[a], sign);
  }
  t[1][1] = cmulc(t[1][1], s3, gh);   // W12^1
  t[1][2] = cmulc(t[1][2], h, gs3);   // W12^2
  t[2][1] = cmulc(t[2][1], h, gs3);   // W12^2
  t[2][2] = cmulc(t[2][2], -h, gs3);  // W12^4
  t[3][1] = sign < 0 ? cmulmi(t[3][1]) : cmuli(t[3][1]);  // W12^3
  t[3][2].x = -t[3][2].x; t[3][2].y = -t[3][2].y;         // W12^6
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    C u[4] = {t[0][c], t[1][c], t[2][c], t[3][c]};
    dft4(u, sign);
    v[c] = u[0]; v[c + 3] = u[1]; v[c + 6] = u[2]; v[c + 9] = u[3];
  }
}
// natural-order DFT24 (n = a + 8b: eight DFT3 over b, twiddles W24^(ac),
// three DFT8 over a; output k = c + 3d)
template <typename C, typename T> __device__ __forceinline__ void dft24(C* v, int sign) {
  // cos / sin of 15 degrees x m, m = 0..14
  constexpr double cs[15] = {1.0, 0.96592582628906828675, 0.86602540378443864676, 0.70710678118654752440, 0.5,
                             0.25881904510252076235, 0.0, -0.25881904510252076235, -0.5, -0.70710678118654752440,
                             -0.86602540378443864676, -0.96592582628906828675, -1.0, -0.96592582628906828675,
                             -0.86602540378443864676};
  constexpr double sn[15] = {0.0, 0.25881904510252076235, 0.5, 0.70710678118654752440, 0.86602540378443864676,
                             0.96592582628906828675, 1.0, 0.96592582628906828675, 0.86602540378443864676,
                             0.70710678118654752440, 0.5, 0.25881904510252076235, 0.0, -0.25881904510252076235,
                             -0.5};
  C t[8][3];
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    t[a][0] = v[a]; t[a][1] = v[a + 8]; t[a][2] = v[a + 16];
    dft3<C, T>(t[a], sign);
  }
#pragma unroll
  for (int a = 1; a < 8; ++a)
#pragma unroll
    for (int c = 1; c < 3; ++c) {
      const int m = a * c;
      t[a][c] = cmulc(t[a][c], (T)cs[m], sign < 0 ? (T)(-sn[m]) : (T)sn[m]);
    }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    C u[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) u[a] = t[a][c];
    dft8<C, T>(u, sign);
#pragma unroll
    for (int d = 0; d < 8; ++d) v[c + 3 * d] = u[d];
  }
}
// natural-order DFT of a compile-time length in registers
template <typename T, int N> __device__ __forceinline__ void dft_n(typename CT<T>::type* v, int sign) {
  typedef typename CT<T>::type C;
  if constexpr (N == 24) dft24<C, T>(v, sign);
  else if constexpr (N == 16) dft16<C, T>(v, sign);
  else if constexpr (N == 12) dft12<C, T>(v, sign);
  else if constexpr (N == 8) dft8<C, T>(v, sign);
  else if constexpr (N == 4) dft4(v, sign);
  else if constexpr (N == 3) dft3<C, T>(v, sign);
  else if constexpr (N == 2) dft2(v);
  else static_assert(N == 1, "register DFT length");
}

// One pass.  COLS: element (b, i) at x[sk(i) * NB + b]; rows: x[b * skn(N)
// + sk(i)] for nbr batches.  SIGN -1 forward, +1 inverse (conjugated
// twiddles); tw: the unit-circle table of length N.
template <typename T, bool COLS, int N, int NB, int R, int NS, int SIGN, int NT>
__device__ __forceinline__ void fft_pass_ct(const typename CT<T>::type* __restrict__ x,
                                            typename CT<T>::type* __restrict__ y,
                                            const typename CT<T>::type* __restrict__ tw, int nbr) {
  typedef typename CT<T>::type C;
  constexpr int M = N / R, PN = skn(N), TS = N / (NS * R);
  const int total = M * (COLS ? NB : nbr);
  for (int t = threadIdx.x; t < total; t += NT) {
    int b, j;
    if (COLS) { b = t % NB; j = t / NB; }
    else { b = t / M; j = t - b * M; }
    const int jq = j / NS, k = j - jq * NS;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = COLS ? x[sk(j + r * M) * NB + b] : x[b * PN + sk(j + r * M)];
    if (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        C w = tw[r * k * TS];
        if (SIGN > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    if constexpr (R == 16) dft16<C, T>(v, SIGN);
    else if constexpr (R == 8) dft8<C, T>(v, SIGN);
    else if constexpr (R == 4) dft4(v, SIGN);
    else if constexpr (R == 2) dft2(v);
    else dft3<C, T>(v, SIGN);
    const int base = jq * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (COLS) y[sk(base + r * NS) * NB + b] = v[r];
      else y[b * PN + sk(base + r * NS)] = v[r];
    }
  }
}
// All passes from stage S on; returns the buffer holding the result.
// MAXR: largest radix.
template <typename T, bool COLS, int N, int NB, int SIGN, int NT, int MAXR, int S = 0, int NS = 1>
__device__ __forceinline__ typename CT<T>::type* fft_ct(typename CT<T>::type* x, typename CT<T>::type* y,
                                                        const typename CT<T>::type* tw, int nbr) {
  if constexpr (NS >= N) {
    return x;
  } else {
    constexpr int R = ct2_radix(N, S, MAXR);
    fft_pass_ct<T, COLS, N, NB, R, NS, SIGN, NT>(x, y, tw, nbr);
    __syncthreads();
    return fft_ct<T, COLS, N, NB, SIGN, NT, MAXR, S + 1, NS * R>(y, x, tw, nbr);
  }
}
// largest radix of the y pass (FP32: 16; float-float: 4, register use);
// the x pass uses radix <= 4 (its many short rows keep more blocks resident)
template <typename T> struct CtMaxR { static constexpr int v = 16; };
template <> struct CtMaxR<dfloat> { static constexpr int v = 4; };
constexpr int CT_MAXR_ROWS = 4;

// unit-circle table entry m of a plan, in the kernel's precision
template <typename T> struct UnitSel;
template <> struct UnitSel<float> {
  static __device__ __forceinline__ float2 get(const FftPlanDev& P, int m) { return __ldg(&P.unitf[m]); }
};
template <> struct UnitSel<dfloat> {
  static __device__ __forceinline__ dcomplex get(const FftPlanDev& P, int m) {
    const float4 v = __ldg(&P.unitd[m]);
    dcomplex r;
    r.x = dfloat(v.x, v.y);
    r.y = dfloat(v.z, v.w);
    return r;
  }
};
template <> struct UnitSel<double> {  // not used by the fixed-length kernels
  static __device__ __forceinline__ double2 get(const FftPlanDev& P, int m) { return make_double2(0.0, 0.0); }
};

// ---- job descriptors --------------------------------------------------------
constexpr int JOB_MAXF = 24;

// rows_r2c / rows_c2r: nfield fields x nlev planes.
struct RowJob {
  int nfield, nlev;
  int ny;                 // rows per plane
  int ld;                 // physical row stride (reals)
  int wc;                 // work-buffer row stride (complex entries)
  int ncols;              // complex columns stored (r2c) / read (c2r), <= nx/2+1
  long pstride_phys;      // reals between consecutive planes of a physical field
  long pstride_work;      // complex entries between consecutive work planes
  const void* phys[JOB_MAXF];   // physical field base (plane 0)
  void* work[JOB_MAXF];         // work buffer base (plane 0)
  double scale[JOB_MAXF];       // r2c: multiply input by scale before the transform
  double div[JOB_MAXF];         // r2c: when non-zero, input is (x / div) * scale
  const double* off[JOB_MAXF];  // per-plane offsets: r2c subtracts off[plane] before
                                // scaling, c2r adds it to the output (null: none)
  int rpc;                      // rows per CTA (0: default for the size)
  FastDiv dnc;                  // ncols
};

// Spectral coefficient codes for the column operator.
enum ColCoef {
  CC_NONE = 0,
  CC_ONE = 1,     // copy
  CC_G = 2,       // x G_test       (test_filtermodule.f90:247)
  CC_GG = 3,      // x G_test_test
  CC_IKX = 4,     // x i kx         (ddx.f90:152)
  CC_IKY = 5,     // x i ky         (ddy.f90:183)
  CC_KILL = 6,    // copy with the Nyquist row/column zeroed (filt_da.f90:114-115)
  CC_MASK = 7,    // G_test / (1/(nx*ny)): pass where G_test != 0 (input already scaled)
  CC_MASK4 = 8,   // G_test_test / (1/(nx*ny))
  CC_MIKY = 9     // x (-i ky): with CC_IKX on a second input, the vertical vorticity dv/dx - du/dy
};
enum ColMap { MAP_SAME = 0, MAP_PAD = 1, MAP_UNPAD = 2 };
enum ColDir { DIR_FWD = 1, DIR_INV = 2, DIR_BOTH = 3 };

constexpr int COL_MAXI = 4;
constexpr int COL_MAXO = 6;

struct ColJob {
  int nin, nout, nlev;
  int nf;                 // independent field sets (grid z); set f uses
  long fs_in, fs_out;     // in[i] + f*fs_in and out[o] + f*fs_out
  int ny_in, ny_out;      // transform lengths
  int map, dir;           // dir & DIR_FWD: forward y pass on the inputs
  unsigned inv_mask;      // bit o: inverse y pass on output o (else the spectrum is stored)
  int ncols;              // kx columns processed
  int ny_small;           // ny of the small grid (pad/unpad mapping)
  int wc_in, wc_out;      // row strides (complex)
  long ps_in, ps_out;     // plane strides (complex)
  int coef[COL_MAXO][COL_MAXI];
  const void* in[COL_MAXI];
  void* out[COL_MAXO];
  const double* kx;       // (lh,ny) wavenumber tables of the small grid
  const double* ky;
  const double* G;        // G_test (lh,ny)
  const double* GG;       // G_test_test
  const float* kxf;       // the same tables in FP32 for FP32 kernels
  const float* kyf;
  const float* Gf;
  const float* GGf;
  const float2* kxd;      // kx, ky as float-float pairs (float-float kernels)
  const float2* kyd;
  int lh;                 // row stride of the (lh,ny) tables
  int tx;                 // kx columns per CTA (0: default for the precision)
};

}  // namespace les
