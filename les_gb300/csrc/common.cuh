// Shared device/host helpers for the GB300 LES core.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#define LES_PI 3.1415926535897932384626433   /* param.f90:51 */
#define LES_BOGUS (-1234567890.0)              /* param.f90:50 */

namespace les {

// Complex type traits for the two arithmetic precisions.
template <typename T> struct CT;
template <> struct CT<double> { typedef double2 type; };
template <> struct CT<float> { typedef float2 type; };

template <typename T> __host__ __device__ __forceinline__ typename CT<T>::type mk(T a, T b) {
  typename CT<T>::type r; r.x = a; r.y = b; return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) { a.x *= s; a.y *= s; return a; }
// i * a
template <typename C> __device__ __forceinline__ C cmuli(C a) { C r; r.x = -a.y; r.y = a.x; return r; }
// -i * a
template <typename C> __device__ __forceinline__ C cmulmi(C a) { C r; r.x = a.y; r.y = -a.x; return r; }
template <typename C> __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }

// eye * k * f = (-k f.im, k f.re), the reference's spectral derivative
// (ddx.f90:152, filt_da.f90:117-118).
template <typename C, typename T> __device__ __forceinline__ C ik(C f, T k) {
  C r; r.x = -(k * f.y); r.y = k * f.x; return r;
}

// FP32 truncation max(real(a), real(b)) of the reference's default-real MAX.
__device__ __forceinline__ double fmax32(double a, double b) {
  float fa = __double2float_rn(a), fb = __double2float_rn(b);
  return (double)(fa > fb ? fa : fb);
}

// IEEE-754 binary32 <-> binary64 conversions done with integer operations.
// On this part a hardware float<->double conversion issues on the FP64 pipe,
// which is as scarce as FP64 arithmetic; these run on the integer pipe for
// the normal range and zeros, and fall back to the hardware conversion for
// the rest (subnormals, overflow, infinities, NaN).  Results are identical
// to the hardware's: exact widening; narrowing rounds to nearest, ties to
// even, from the definition of the two formats.
__device__ __forceinline__ double cvt_f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) {
    if ((u << 1) == 0u) return __longlong_as_double((long long)((unsigned long long)u << 32));  // +-0
    return (double)f;
  }
  const unsigned long long d = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(e + 896u) << 52) |
                               ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)d);
}
__device__ __forceinline__ float cvt_d2f(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
  const int fe = (int)((b >> 52) & 0x7ffu) - 896;  // binary32 biased exponent
  if (fe <= 0 || fe >= 255) {
    if ((b << 1) == 0ull) return __uint_as_float(sgn);  // +-0
    return (float)x;
  }
  const unsigned m23 = (unsigned)(b >> 29) & 0x7fffffu;
  const unsigned rem = (unsigned)b & 0x1fffffffu;  // the 29 dropped mantissa bits
  unsigned r = sgn | ((unsigned)fe << 23) | m23;
  if (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) r += 1u;  // a carry rounds into the exponent
  return __uint_as_float(r);
}
// Float-float number ("double-single"): value hi + lo with |lo| <= ulp(hi)/2,
// about 48 significant bits, computed on the FP32 pipe with error-free
// transformations (Knuth's two-sum for additions, products through fused
// multiply-add, Dekker).  The mixed form runs its projection-path transforms
// in it: FP64-like accuracy at FP32-pipe throughput.
struct __align__(8) dfloat {
  float hi, lo;
  __host__ __device__ dfloat() {}
  __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dfloat(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr dfloat(int i) : hi((float)i), lo(0.f) {}
};
struct __align__(16) dcomplex {
  dfloat x, y;
};
template <> struct CT<dfloat> { typedef dcomplex type; };
__device__ __forceinline__ dfloat df_quick(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return dfloat(s, b - (s - a));
}
// Sums and products are left unnormalised (hi = the rounded leading term,
// lo = its exact error plus the low parts, |lo| a few ulp(hi) at most): the
// next operation's two-sum / FMA product absorbs it, and a conversion to
// FP64 adds the two.  Saves the quick-two-sum on the FP32 pipe.
__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb) + (a.lo + b.lo);
  return dfloat(s, e);
}
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return dfloat(p, e);
}
__device__ __forceinline__ dfloat operator/(dfloat a, dfloat b) {
  const float q1 = a.hi / b.hi;
  const dfloat r = a - b * dfloat(q1, 0.f);
  const float q2 = r.hi / b.hi;
  return df_quick(q1, q2);
}
__device__ __forceinline__ dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }
__device__ __forceinline__ dfloat& operator*=(dfloat& a, dfloat b) { return a = a * b; }
__device__ __forceinline__ bool operator!=(dfloat a, dfloat b) { return a.hi != b.hi || a.lo != b.lo; }

// element conversions between a transform's precision and the storage type
template <typename To, typename From> __device__ __forceinline__ To cvt(From v) { return (To)v; }
template <> __device__ __forceinline__ double cvt<double, float>(float v) { return cvt_f2d(v); }
template <> __device__ __forceinline__ float cvt<float, double>(double v) { return cvt_d2f(v); }
template <> __device__ __forceinline__ dfloat cvt<dfloat, double>(double v) {
  const float h = cvt_d2f(v);
  return dfloat(h, cvt_d2f(v - cvt_f2d(h)));
}
template <> __device__ __forceinline__ double cvt<double, dfloat>(dfloat v) { return cvt_f2d(v.hi) + cvt_f2d(v.lo); }
template <> __device__ __forceinline__ dfloat cvt<dfloat, dfloat>(dfloat v) { return v; }
__device__ __forceinline__ double2 to_d2(double2 v) { return v; }
__device__ __forceinline__ double2 to_d2(dcomplex v) { return make_double2(cvt<double>(v.x), cvt<double>(v.y)); }
template <typename CO> __device__ __forceinline__ CO from_d2(double2 v);
template <> __device__ __forceinline__ double2 from_d2<double2>(double2 v) { return v; }
template <> __device__ __forceinline__ dcomplex from_d2<dcomplex>(double2 v) {
  dcomplex r;
  r.x = cvt<dfloat>(v.x);
  r.y = cvt<dfloat>(v.y);
  return r;
}

}  // namespace les

#define LES_CUDA_CHECK(expr)                                                           \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess) {                                                           \
      les_set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(_e)); \
      return LES_ERR_CUDA;                                                             \
    }                                                                                  \
  } while (0)

void les_set_error(const char* fmt, ...);

// Number of kernels this library has launched (diagnostic counter).
extern unsigned long long g_les_launches;
#define LES_COUNT_LAUNCH() (++g_les_launches)

namespace les {
// Measurement hook (les_profile_begin/end): while a session is open, every
// launch of one kernel family on the session's stream is bracketed by CUDA
// events and its algorithmic bytes (inputs read once + outputs written once)
// are summed.  Families: 1 FP64 y-pass, 2 FP32 y-pass, 3 FP64 x-pass,
// 4 FP32 x-pass (forward and inverse).
enum ProfFamily { PROF_COLS64 = 1, PROF_COLS32 = 2, PROF_ROWS64 = 3, PROF_ROWS32 = 4 };
struct ProfSession {
  int family = 0;
  cudaStream_t stream = nullptr;
  int n = 0, cap = 0;
  cudaEvent_t* ev = nullptr;
  double bytes = 0.0;
};
extern ProfSession* g_prof;
bool prof_mark(int family, cudaStream_t s);         // true: the launch that follows is measured
void prof_done(cudaStream_t s, double bytes);       // after that launch
}  // namespace les
