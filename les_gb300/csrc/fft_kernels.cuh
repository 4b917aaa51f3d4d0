// Batched plane FFT kernel templates (rows_r2c, cols, rows_c2r), shared by
// the runtime-length instantiations (fft_kernels.cu) and the fixed-length
// FP32 instantiations (fft_fixed.cu).
#pragma once
#include "fft.cuh"

namespace les {

template <typename T> __device__ __forceinline__ typename CT<T>::type rw(const RealPlanDev& P, int k);
template <> __device__ __forceinline__ double2 rw<double>(const RealPlanDev& P, int k) { return __ldg(&P.w[k]); }
template <> __device__ __forceinline__ float2 rw<float>(const RealPlanDev& P, int k) { return __ldg(&P.wf[k]); }
template <> __device__ __forceinline__ dcomplex rw<dfloat>(const RealPlanDev& P, int k) {
  const float4 v = __ldg(&P.wd[k]);
  dcomplex r;
  r.x = dfloat(v.x, v.y);
  r.y = dfloat(v.z, v.w);
  return r;
}

// spectral coefficient tables in the kernel's precision
template <typename T> struct Tab;
template <> struct Tab<double> {
  static __device__ __forceinline__ double kx(const ColJob& J, size_t i) { return J.kx[i]; }
  static __device__ __forceinline__ double ky(const ColJob& J, size_t i) { return J.ky[i]; }
  static __device__ __forceinline__ double G(const ColJob& J, size_t i) { return J.G[i]; }
  static __device__ __forceinline__ double GG(const ColJob& J, size_t i) { return J.GG[i]; }
};
template <> struct Tab<dfloat> {
  static __device__ __forceinline__ dfloat kx(const ColJob& J, size_t i) { const float2 v = __ldg(&J.kxd[i]); return dfloat(v.x, v.y); }
  static __device__ __forceinline__ dfloat ky(const ColJob& J, size_t i) { const float2 v = __ldg(&J.kyd[i]); return dfloat(v.x, v.y); }
  static __device__ __forceinline__ dfloat G(const ColJob& J, size_t i) { return cvt<dfloat>(J.G[i]); }
  static __device__ __forceinline__ dfloat GG(const ColJob& J, size_t i) { return cvt<dfloat>(J.GG[i]); }
};
template <> struct Tab<float> {
  static __device__ __forceinline__ float kx(const ColJob& J, size_t i) { return J.kxf[i]; }
  static __device__ __forceinline__ float ky(const ColJob& J, size_t i) { return J.kyf[i]; }
  static __device__ __forceinline__ float G(const ColJob& J, size_t i) { return J.Gf[i]; }
  static __device__ __forceinline__ float GG(const ColJob& J, size_t i) { return J.GGf[i]; }
};

// x f - off(plane) rounded to the transform precision: an FP64 input is
// shifted in FP64 before rounding (the mean leaves FP32 transforms of u, v,
// w, theta with the fluctuation's precision); an FP32 input is shifted by the
// plane constant rounded to FP32 (the derivatives of a plane constant are
// zero, so any constant near the mean serves), with no FP64 arithmetic.
template <typename T, typename TIn> __device__ __forceinline__ T sub_off(TIn x, double off) {
  if constexpr (std::is_same<TIn, float>::value) return cvt<T, float>(x - cvt_d2f(off));
  else return cvt<T, double>(cvt<double, TIn>(x) - off);
}

// ---------------------------------------------------------------------------
// rows_r2c: x-transform of `rpc` rows per CTA.  grid = (ceil(ny/rpc), nlev, nfield)
// NF > 0: the half length m = nx/2 is NF at compile time (fixed-length
// transform, twiddles staged in shared memory after the work buffers).
template <typename T, typename TIn, int NF>
__global__ void __launch_bounds__(256) k_rows_r2c(RowJob J, RealPlanDev P, int rpc) {
  typedef typename CT<T>::type C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* A = reinterpret_cast<C*>(smraw);
  const int m = NF > 0 ? NF : P.nx / 2;
  const int rs = NF > 0 ? skn(NF) : m;  // row stride of A, B (skewed when NF > 0)
  C* B = A + rpc * rs;
  C* tws = B + rpc * rs;  // NF > 0: unit-circle table (NF) then post-processing twiddles (NF + 1)
  if constexpr (NF > 0) {
    for (int t = threadIdx.x; t < NF; t += 256) tws[t] = UnitSel<T>::get(P.c, t);
    for (int t = threadIdx.x; t <= NF; t += 256) tws[NF + t] = rw<T>(P, t);
  }
  const int f = blockIdx.z, lev = blockIdx.y;
  const int row0 = blockIdx.x * rpc;
  const int nrow = min(rpc, J.ny - row0);
  const TIn* src = reinterpret_cast<const TIn*>(J.phys[f]) + (size_t)lev * J.pstride_phys;
  const T s = (T)J.scale[f];
  const T dv = (T)J.div[f];
  const T sd = (T)(J.div[f] != 0.0 ? J.scale[f] / J.div[f] : J.scale[f]);
  const double off = J.off[f] ? J.off[f][lev] : 0.0;
  for (int t = threadIdx.x; t < nrow * m; t += blockDim.x) {
    const int r = NF > 0 ? t / NF : (int)P.dm.div((unsigned)t), k = t - r * m;
    const TIn* row = src + (size_t)(row0 + r) * J.ld;
    // the pair (2k, 2k+1) in one access: rows start on even offsets
    const typename CT<TIn>::type pr = reinterpret_cast<const typename CT<TIn>::type*>(row)[k];
    T a, b;
    if (J.off[f]) {
      a = sub_off<T, TIn>(pr.x, off);
      b = sub_off<T, TIn>(pr.y, off);
    } else {
      a = cvt<T, TIn>(pr.x);
      b = cvt<T, TIn>(pr.y);
    }
    if constexpr (std::is_same<T, double>::value) {  // the reference's division, then the scale
      if (dv != (T)0) { a = a / dv; b = b / dv; }
      A[r * rs + (NF > 0 ? sk(k) : k)] = mk<T>(a * s, b * s);
    } else {  // FP32 / float-float: one product with scale/div (formed in FP64)
      A[r * rs + (NF > 0 ? sk(k) : k)] = mk<T>(a * sd, b * sd);
    }
  }
  __syncthreads();
  C* Z;
  if constexpr (NF > 0) Z = fft_ct<T, false, NF, 1, -1, 256, CT_MAXR_ROWS>(A, B, tws, nrow);
  else Z = fft_smem<T, false>(A, B, nrow, m, P.c, -1);
  C* out = reinterpret_cast<C*>(J.work[f]) + (size_t)lev * J.pstride_work;
  for (int t = threadIdx.x; t < nrow * J.ncols; t += blockDim.x) {
    const int r = (int)J.dnc.div((unsigned)t), k = t - r * J.ncols;
    const C* z = Z + r * rs;
    C X;
    if (k == 0 || k == m) {
      const C z0 = z[0];
      X = mk<T>(k == 0 ? z0.x + z0.y : z0.x - z0.y, (T)0);
    } else {
      const C a = z[NF > 0 ? sk(k) : k];
      const C b = cconj(z[NF > 0 ? sk(m - k) : m - k]);
      const C e = cscale(cadd(a, b), (T)0.5);
      const C d = cscale(csub(a, b), (T)0.5);
      const C o = cmulmi(d);  // d / i
      X = cadd(e, cmul(NF > 0 ? tws[NF + k] : rw<T>(P, k), o));
    }
    out[(size_t)(row0 + r) * J.wc + k] = X;
  }
}

// rows_c2r: inverse x-transform.  Reads J.ncols complex columns (rest zero).
template <typename T, typename TOut, int NF>
__global__ void __launch_bounds__(256) k_rows_c2r(RowJob J, RealPlanDev P, int rpc) {
  typedef typename CT<T>::type C;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int m = NF > 0 ? NF : P.nx / 2;
  const int rs = NF > 0 ? skn(NF) : m;  // row stride of A, B (skewed when NF > 0)
  C* X = reinterpret_cast<C*>(smraw);  // rpc x (m+1)
  C* A = X + rpc * (m + 1);
  C* B = A + rpc * rs;
  C* tws = B + rpc * rs;  // NF > 0: unit-circle table (NF) then post-processing twiddles (NF + 1)
  if constexpr (NF > 0) {
    for (int t = threadIdx.x; t < NF; t += 256) tws[t] = UnitSel<T>::get(P.c, t);
    for (int t = threadIdx.x; t <= NF; t += 256) tws[NF + t] = rw<T>(P, t);
  }
  const int f = blockIdx.z, lev = blockIdx.y;
  const int row0 = blockIdx.x * rpc;
  const int nrow = min(rpc, J.ny - row0);
  const C* in = reinterpret_cast<const C*>(J.work[f]) + (size_t)lev * J.pstride_work;
  for (int t = threadIdx.x; t < nrow * (m + 1); t += blockDim.x) {
    const int r = NF > 0 ? t / (NF + 1) : (int)P.dm1.div((unsigned)t), k = t - r * (m + 1);
    C v = k < J.ncols ? in[(size_t)(row0 + r) * J.wc + k] : mk<T>((T)0, (T)0);
    if (k == 0 || k == m) v.y = (T)0;  // halfcomplex pass ignores these imaginary parts
    X[t] = v;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nrow * m; t += blockDim.x) {
    const int r = NF > 0 ? t / NF : (int)P.dm.div((unsigned)t), k = t - r * m;
    const C a = X[r * (m + 1) + k];
    const C b = cconj(X[r * (m + 1) + (m - k)]);
    const C e = cadd(a, b);
    const C d = cmul(csub(a, b), cconj(NF > 0 ? tws[NF + k] : rw<T>(P, k)));  // x exp(+2 pi i k/nx)
    A[r * rs + (NF > 0 ? sk(k) : k)] = cadd(e, cmuli(d));
  }
  __syncthreads();
  C* Z;
  if constexpr (NF > 0) Z = fft_ct<T, false, NF, 1, +1, 256, CT_MAXR_ROWS>(A, B, tws, nrow);
  else Z = fft_smem<T, false>(A, B, nrow, m, P.c, +1);
  TOut* dst = reinterpret_cast<TOut*>(const_cast<void*>(J.phys[f])) + (size_t)lev * J.pstride_phys;
  const double off = J.off[f] ? J.off[f][lev] : 0.0;
  for (int t = threadIdx.x; t < nrow * (m + 1); t += blockDim.x) {
    const int r = NF > 0 ? t / (NF + 1) : (int)P.dm1.div((unsigned)t), k = t - r * (m + 1);
    typename CT<TOut>::type* row = reinterpret_cast<typename CT<TOut>::type*>(dst + (size_t)(row0 + r) * J.ld);
    typename CT<TOut>::type pw;
    if (k < m) {
      const C z = Z[r * rs + (NF > 0 ? sk(k) : k)];
      if (J.off[f]) {
        pw.x = cvt<TOut, double>(cvt<double, T>(z.x) + off);
        pw.y = cvt<TOut, double>(cvt<double, T>(z.y) + off);
      } else {
        pw.x = cvt<TOut, T>(z.x);
        pw.y = cvt<TOut, T>(z.y);
      }
    } else {  // padding columns ld-1:ld
      pw.x = (TOut)0;
      pw.y = (TOut)0;
    }
    row[k] = pw;  // the pair (2k, 2k+1) in one access
  }
}

// Asynchronous 8-byte global -> shared copies (zero-filled when src_bytes is 0).
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Warp-local staging of the inverse x pass's rows: the TT threads of a row
// are lanes of one warp, so warp w copies its 32/TT rows (nc <= M + 1
// complex each, M + 1 <= MS) into those rows' slots of the exchange buffer
// with coalesced 8-byte cp.async copies: every element is read from global
// memory once (the Hermitian pre-processing reads X[k] and X[M - k]) and all
// of a thread's copies are in flight together.  __syncwarp makes them
// visible to the row's lanes.
template <typename C, int TT, int RPB, int MS, int M>
__device__ __forceinline__ void stage_rows_warp(C* S, const C* base, size_t wc, int row0, int ny, int nc) {
  static_assert(sizeof(C) == 8 && 32 % TT == 0 && MS >= M + 1, "8-byte elements, rows within one warp");
  constexpr int RPW = 32 / TT, KMAX = (M + 1 + 31) / 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = nc < M + 1 ? nc : M + 1;
#pragma unroll
  for (int rr = 0; rr < RPW; ++rr) {
    const int rl = w * RPW + rr, row = row0 + rl;
    if (rl < RPB && row < ny) {
      const C* src = base + (size_t)row * wc;
#pragma unroll
      for (int kk = 0; kk < KMAX; ++kk) {
        const int k = lane + 32 * kk;
        if (k < n) cp_async8(&S[rl * MS + k], src + k, 8);
      }
    }
  }
  cp_async_commit();
  cp_async_wait_all();
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Register-resident x pass, half length M = N1 * N2.  A row is served by
// TT = max(N1, N2) threads.  Forward (r2c): n = n1 + N1 n2, k = k2 + N2 k1;
// thread n1 loads the pairs z[n1 + N1 n2] straight from the row, DFT_N2 in
// registers, twiddle W_M^(n1 k2), one exchange through shared memory
// (element (n1, k2) at k2 (N1 + 1) + n1: conflict-free both ways), DFT_N1 in
// registers; the Hermitian post-processing pairs Z[k] with Z[M - k] through a
// second, natural-order trip.  Inverse (c2r): thread k1 forms the
// pre-processed A[k1 + N1 k2] from X[k] and X[M - k] read from the work
// buffer, inverse DFT_N2, twiddle, exchange, inverse DFT_N1, and thread n2
// writes the real pairs n2 + N2 n1 of the row.
template <typename T, typename TIn, int N1, int N2, int NT>
__global__ void __launch_bounds__(NT) k_r2c_reg(RowJob J, RealPlanDev P) {
  typedef typename CT<T>::type C;
  typedef typename CT<TIn>::type CI;
  constexpr int M = N1 * N2, TT = N1 > N2 ? N1 : N2, RPB = NT / TT, MS = N2 * (N1 + 1);
  extern __shared__ __align__(16) unsigned char smraw[];
  C* S = reinterpret_cast<C*>(smraw);  // RPB rows x MS
  C* tw = S + RPB * MS;                // exp(-2 pi i j / M), j < M
  C* wr = tw + M;                      // exp(-2 pi i k / nx), k <= M
  for (int t = threadIdx.x; t < M; t += NT) tw[t] = UnitSel<T>::get(P.c, t);
  for (int t = threadIdx.x; t <= M; t += NT) wr[t] = rw<T>(P, t);
  const int q = threadIdx.x % TT, r = threadIdx.x / TT;
  const int f = blockIdx.z, lev = blockIdx.y;
  const int row = blockIdx.x * RPB + r;
  const bool rowok = r < RPB && row < J.ny;
  C* Sr = S + (r < RPB ? r : 0) * MS;
  C v[TT];
  // FP32 input: the rows (M pairs each) are staged once through their
  // exchange slots (stage_rows_warp); an FP64 row does not fit its slot and
  // is read straight from global memory
  constexpr bool STAGED = sizeof(CI) == sizeof(C);
  const TIn* plane = reinterpret_cast<const TIn*>(J.phys[f]) + (size_t)lev * J.pstride_phys;
  if constexpr (STAGED)
    stage_rows_warp<C, TT, RPB, MS, M>(S, reinterpret_cast<const C*>(plane), J.ld / 2, blockIdx.x * RPB, J.ny, M);
  if (q < N1) {
    const T sd = (T)(J.div[f] != 0.0 ? J.scale[f] / J.div[f] : J.scale[f]);  // scale/div, one product
    const bool hasoff = J.off[f] != nullptr;
    const double off = hasoff ? J.off[f][lev] : 0.0;
    const CI* src = STAGED ? reinterpret_cast<const CI*>(Sr) + q
                           : reinterpret_cast<const CI*>(plane + (size_t)(rowok ? row : 0) * J.ld) + q;
#pragma unroll
    for (int i = 0; i < N2; ++i) {
      v[i] = mk<T>((T)0, (T)0);
      if (rowok) {
        const CI pr = src[N1 * i];
        T a, b;
        if (hasoff) {
          a = sub_off<T, TIn>(pr.x, off);
          b = sub_off<T, TIn>(pr.y, off);
        } else {
          a = cvt<T, TIn>(pr.x);
          b = cvt<T, TIn>(pr.y);
        }
        v[i] = mk<T>(a * sd, b * sd);
      }
    }
  }
  __syncthreads();  // tables
  if (q < N1) {
    dft_n<T, N2>(v, -1);  // over n2: v[i] = y[n1 = q][k2 = i]
#pragma unroll
    for (int i = 1; i < N2; ++i) v[i] = cmul(v[i], tw[q * i]);
    if (r < RPB) {
#pragma unroll
      for (int i = 0; i < N2; ++i) Sr[i * (N1 + 1) + q] = v[i];
    }
  }
  __syncthreads();
  if (q < N2 && r < RPB) {
#pragma unroll
    for (int i = 0; i < N1; ++i) v[i] = Sr[q * (N1 + 1) + i];
    dft_n<T, N1>(v, -1);  // over n1: v[i] = Z[q + N2 i]
  }
  __syncthreads();
  if (q < N2 && r < RPB) {
#pragma unroll
    for (int i = 0; i < N1; ++i) Sr[q + N2 * i] = v[i];  // natural order
  }
  __syncthreads();
  if (q < N2 && rowok) {
    C* out = reinterpret_cast<C*>(J.work[f]) + (size_t)lev * J.pstride_work + (size_t)row * J.wc;
    const int nc = J.ncols;
#pragma unroll
    for (int i = 0; i < N1; ++i) {
      const int k = q + N2 * i;
      const C a = v[i];
      C X;
      if (k == 0) {
        X = mk<T>(a.x + a.y, (T)0);
        if (M < nc) out[M] = mk<T>(a.x - a.y, (T)0);
      } else {
        const C b = cconj(Sr[M - k]);
        const C e = cscale(cadd(a, b), (T)0.5);
        const C d = cscale(csub(a, b), (T)0.5);
        X = cadd(e, cmul(wr[k], cmulmi(d)));  // (d / i) x exp(-2 pi i k / nx)
      }
      if (k < nc) out[k] = X;
    }
  }
}

template <typename T, typename TOut, int N1, int N2, int NT>
__global__ void __launch_bounds__(NT) k_c2r_reg(RowJob J, RealPlanDev P) {
  typedef typename CT<T>::type C;
  typedef typename CT<TOut>::type CO;
  constexpr int M = N1 * N2, TT = N1 > N2 ? N1 : N2, RPB = NT / TT, MS = N2 * (N1 + 1);
  extern __shared__ __align__(16) unsigned char smraw[];
  C* S = reinterpret_cast<C*>(smraw);  // RPB rows x MS
  // twiddles exp(-2 pi i j / M) and exp(-2 pi i k / nx) straight from their
  // (cached) global tables: a block issues its row loads without first
  // waiting for a table fill and a barrier
  const int q = threadIdx.x % TT, r = threadIdx.x / TT;
  const int f = blockIdx.z, lev = blockIdx.y;
  const int row = blockIdx.x * RPB + r;
  const bool rowok = r < RPB && row < J.ny;
  C* Sr = S + (r < RPB ? r : 0) * MS;
  C v[TT];
  const int nc = J.ncols;
  stage_rows_warp<C, TT, RPB, MS, M>(S, reinterpret_cast<const C*>(J.work[f]) + (size_t)lev * J.pstride_work, J.wc,
                                     blockIdx.x * RPB, J.ny, nc);
  if (q < N1) {
#pragma unroll
    for (int i = 0; i < N2; ++i) {
      const int k = q + N1 * i, km = M - k;
      C a = mk<T>((T)0, (T)0), bb = mk<T>((T)0, (T)0);
      if (rowok) {
        if (k < nc) a = Sr[k];
        if (km < nc) bb = Sr[km];
      }
      if (k == 0) { a.y = (T)0; bb.y = (T)0; }  // the halfcomplex pass ignores Im of X[0], X[M]
      const C b = cconj(bb);
      const C e = cadd(a, b);
      const C d = cmul(csub(a, b), cconj(rw<T>(P, k)));  // x exp(+2 pi i k / nx)
      v[i] = cadd(e, cmuli(d));
    }
  }
  __syncwarp();  // the row's staged input is read before its exchange slots are written
  if (q < N1) {
    dft_n<T, N2>(v, +1);  // over k2: v[i] = y[k1 = q][n2 = i]
#pragma unroll
    for (int i = 1; i < N2; ++i) v[i] = cmul(v[i], cconj(UnitSel<T>::get(P.c, q * i)));
    if (r < RPB) {
#pragma unroll
      for (int i = 0; i < N2; ++i) Sr[i * (N1 + 1) + q] = v[i];
    }
  }
  __syncthreads();
  if (q < N2 && rowok) {
#pragma unroll
    for (int i = 0; i < N1; ++i) v[i] = Sr[q * (N1 + 1) + i];
    dft_n<T, N1>(v, +1);  // over k1: v[i] = z[q + N2 i]
    TOut* dst = reinterpret_cast<TOut*>(const_cast<void*>(J.phys[f])) + (size_t)lev * J.pstride_phys +
                (size_t)row * J.ld;
    CO* pairs = reinterpret_cast<CO*>(dst);
    const bool hasoff = J.off[f] != nullptr;
    const double off = hasoff ? J.off[f][lev] : 0.0;
#pragma unroll
    for (int i = 0; i < N1; ++i) {
      const C z = v[i];
      CO pw;
      if (hasoff) {
        pw.x = cvt<TOut, double>(cvt<double, T>(z.x) + off);
        pw.y = cvt<TOut, double>(cvt<double, T>(z.y) + off);
      } else {
        pw.x = cvt<TOut, T>(z.x);
        pw.y = cvt<TOut, T>(z.y);
      }
      pairs[q + N2 * i] = pw;
    }
    if (q == 0) {  // padding columns ld-1:ld
      CO pz;
      pz.x = (TOut)0;
      pz.y = (TOut)0;
      pairs[M] = pz;
    }
  }
}

// The same x pass with TT threads per row, TT dividing N1 and N2: thread q
// takes the N1/TT first-step transforms n1 = q + TT j and the N2/TT
// second-step transforms k2 = q + TT j, so every lane works in both steps
// and in the Hermitian pre/post-processing (half length 128 = 16 x 8 with
// eight threads per row).
template <typename T, typename TIn, int N1, int N2, int TT, int NT>
__global__ void __launch_bounds__(NT, 5) k_r2c_reg2(RowJob J, RealPlanDev P) {
  typedef typename CT<T>::type C;
  typedef typename CT<TIn>::type CI;
  static_assert(N1 % TT == 0 && N2 % TT == 0 && NT % TT == 0, "thread split");
  constexpr int M = N1 * N2, RPB = NT / TT, MS = N2 * (N1 + 1), J1 = N1 / TT, J2 = N2 / TT;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* S = reinterpret_cast<C*>(smraw);  // RPB rows x MS
  C* tw = S + RPB * MS;                // exp(-2 pi i j / M), j < M
  C* wr = tw + M;                      // exp(-2 pi i k / nx), k <= M
  for (int t = threadIdx.x; t < M; t += NT) tw[t] = UnitSel<T>::get(P.c, t);
  for (int t = threadIdx.x; t <= M; t += NT) wr[t] = rw<T>(P, t);
  const int q = threadIdx.x % TT, r = threadIdx.x / TT;
  const int f = blockIdx.z, lev = blockIdx.y;
  const int row = blockIdx.x * RPB + r;
  const bool rowok = row < J.ny;
  C* Sr = S + r * MS;
  const T sd = (T)(J.div[f] != 0.0 ? J.scale[f] / J.div[f] : J.scale[f]);  // scale/div, one product
  const bool hasoff = J.off[f] != nullptr;
  const double off = hasoff ? J.off[f][lev] : 0.0;
  // FP32 input staged as in k_r2c_reg
  constexpr bool STAGED = sizeof(CI) == sizeof(C);
  const TIn* plane = reinterpret_cast<const TIn*>(J.phys[f]) + (size_t)lev * J.pstride_phys;
  if constexpr (STAGED)
    stage_rows_warp<C, TT, RPB, MS, M>(S, reinterpret_cast<const C*>(plane), J.ld / 2, blockIdx.x * RPB, J.ny, M);
  const CI* src = STAGED ? reinterpret_cast<const CI*>(Sr)
                         : reinterpret_cast<const CI*>(plane + (size_t)(rowok ? row : 0) * J.ld);
  C v[J1][N2];
#pragma unroll
  for (int j = 0; j < J1; ++j)
#pragma unroll
    for (int i = 0; i < N2; ++i) {
      v[j][i] = mk<T>((T)0, (T)0);
      if (rowok) {
        const CI pr = src[q + TT * j + N1 * i];
        T a, b;
        if (hasoff) {
          a = sub_off<T, TIn>(pr.x, off);
          b = sub_off<T, TIn>(pr.y, off);
        } else {
          a = cvt<T, TIn>(pr.x);
          b = cvt<T, TIn>(pr.y);
        }
        v[j][i] = mk<T>(a * sd, b * sd);
      }
    }
  __syncthreads();  // tables
#pragma unroll
  for (int j = 0; j < J1; ++j) {
    const int n1 = q + TT * j;
    dft_n<T, N2>(v[j], -1);  // over n2: v[j][i] = y[n1][k2 = i]
#pragma unroll
    for (int i = 1; i < N2; ++i) v[j][i] = cmul(v[j][i], tw[n1 * i]);
#pragma unroll
    for (int i = 0; i < N2; ++i) Sr[i * (N1 + 1) + n1] = v[j][i];
  }
  __syncthreads();
  C w[J2][N1];
#pragma unroll
  for (int j = 0; j < J2; ++j) {
    const int k2 = q + TT * j;
#pragma unroll
    for (int i = 0; i < N1; ++i) w[j][i] = Sr[k2 * (N1 + 1) + i];
    dft_n<T, N1>(w[j], -1);  // over n1: w[j][i] = Z[k2 + N2 i]
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < J2; ++j)
#pragma unroll
    for (int i = 0; i < N1; ++i) Sr[q + TT * j + N2 * i] = w[j][i];  // natural order
  __syncthreads();
  if (rowok) {
    C* out = reinterpret_cast<C*>(J.work[f]) + (size_t)lev * J.pstride_work + (size_t)row * J.wc;
    const int nc = J.ncols;
#pragma unroll
    for (int j = 0; j < J2; ++j)
#pragma unroll
      for (int i = 0; i < N1; ++i) {
        const int k = q + TT * j + N2 * i;
        const C a = w[j][i];
        C X;
        if (k == 0) {
          X = mk<T>(a.x + a.y, (T)0);
          if (M < nc) out[M] = mk<T>(a.x - a.y, (T)0);
        } else {
          const C b = cconj(Sr[M - k]);
          const C e = cscale(cadd(a, b), (T)0.5);
          const C d = cscale(csub(a, b), (T)0.5);
          X = cadd(e, cmul(wr[k], cmulmi(d)));  // (d / i) x exp(-2 pi i k / nx)
        }
        if (k < nc) out[k] = X;
      }
  }
}

template <typename T, typename TOut, int N1, int N2, int TT, int NT>
__global__ void __launch_bounds__(NT, 5) k_c2r_reg2(RowJob J, RealPlanDev P) {
  typedef typename CT<T>::type C;
  typedef typename CT<TOut>::type CO;
  static_assert(N1 % TT == 0 && N2 % TT == 0 && NT % TT == 0, "thread split");
  constexpr int M = N1 * N2, RPB = NT / TT, MS = N2 * (N1 + 1), J1 = N1 / TT, J2 = N2 / TT;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* S = reinterpret_cast<C*>(smraw);  // RPB rows x MS
  // twiddles from their cached global tables (no table fill and barrier
  // ahead of the row loads)
  const int q = threadIdx.x % TT, r = threadIdx.x / TT;
  const int f = blockIdx.z, lev = blockIdx.y;
  const int row = blockIdx.x * RPB + r;
  const bool rowok = row < J.ny;
  C* Sr = S + r * MS;
  const int nc = J.ncols;
  stage_rows_warp<C, TT, RPB, MS, M>(S, reinterpret_cast<const C*>(J.work[f]) + (size_t)lev * J.pstride_work, J.wc,
                                     blockIdx.x * RPB, J.ny, nc);
  C v[J1][N2];
#pragma unroll
  for (int j = 0; j < J1; ++j) {
    const int k1 = q + TT * j;
#pragma unroll
    for (int i = 0; i < N2; ++i) {
      const int k = k1 + N1 * i, km = M - k;
      C a = mk<T>((T)0, (T)0), bb = mk<T>((T)0, (T)0);
      if (rowok) {
        if (k < nc) a = Sr[k];
        if (km < nc) bb = Sr[km];
      }
      if (k == 0) { a.y = (T)0; bb.y = (T)0; }  // the halfcomplex pass ignores Im of X[0], X[M]
      const C b = cconj(bb);
      const C e = cadd(a, b);
      const C d = cmul(csub(a, b), cconj(rw<T>(P, k)));  // x exp(+2 pi i k / nx)
      v[j][i] = cadd(e, cmuli(d));
    }
  }
  __syncwarp();  // the row's staged input is read before its exchange slots are written
#pragma unroll
  for (int j = 0; j < J1; ++j) {
    const int k1 = q + TT * j;
    dft_n<T, N2>(v[j], +1);  // over k2: v[j][i] = y[k1][n2 = i]
#pragma unroll
    for (int i = 1; i < N2; ++i) v[j][i] = cmul(v[j][i], cconj(UnitSel<T>::get(P.c, k1 * i)));
#pragma unroll
    for (int i = 0; i < N2; ++i) Sr[i * (N1 + 1) + k1] = v[j][i];
  }
  __syncthreads();
  if (rowok) {
    TOut* dst = reinterpret_cast<TOut*>(const_cast<void*>(J.phys[f])) + (size_t)lev * J.pstride_phys +
                (size_t)row * J.ld;
    CO* pairs = reinterpret_cast<CO*>(dst);
    const bool hasoff = J.off[f] != nullptr;
    const double off = hasoff ? J.off[f][lev] : 0.0;
#pragma unroll
    for (int j = 0; j < J2; ++j) {
      const int n2 = q + TT * j;
      C w[N1];
#pragma unroll
      for (int i = 0; i < N1; ++i) w[i] = Sr[n2 * (N1 + 1) + i];
      dft_n<T, N1>(w, +1);  // over k1: w[i] = z[n2 + N2 i]
#pragma unroll
      for (int i = 0; i < N1; ++i) {
        const C z = w[i];
        CO pw;
        if (hasoff) {
          pw.x = cvt<TOut, double>(cvt<double, T>(z.x) + off);
          pw.y = cvt<TOut, double>(cvt<double, T>(z.y) + off);
        } else {
          pw.x = cvt<TOut, T>(z.x);
          pw.y = cvt<TOut, T>(z.y);
        }
        pairs[n2 + N2 * i] = pw;
      }
    }
    if (q == 0) {  // padding columns ld-1:ld
      CO pz;
      pz.x = (TOut)0;
      pz.y = (TOut)0;
      pairs[M] = pz;
    }
  }
}

// ---------------------------------------------------------------------------
// cols: y-transform of TX kx columns per CTA, all fields of the job.
// grid = (ceil(ncols/TX), nlev, nf)
template <typename T>
__device__ __forceinline__ typename CT<T>::type apply_coef(int code, typename CT<T>::type v, int jx,
                                                           int js, const ColJob& J) {
  typedef typename CT<T>::type C;
  const size_t ki = (size_t)jx + (size_t)J.lh * js;
  switch (code) {
    case CC_ONE: return v;
    case CC_G: return cscale(v, Tab<T>::G(J, ki));
    case CC_GG: return cscale(v, Tab<T>::GG(J, ki));
    case CC_IKX: return ik(v, Tab<T>::kx(J, ki));
    case CC_IKY: return ik(v, Tab<T>::ky(J, ki));
    case CC_MIKY: return ik(v, -Tab<T>::ky(J, ki));
    case CC_KILL: {
      const int lhm1 = J.lh - 1;
      if (jx == lhm1 || js == J.ny_small / 2) return mk<T>((T)0, (T)0);
      return v;
    }
    case CC_MASK: return Tab<T>::G(J, ki) != (T)0 ? v : mk<T>((T)0, (T)0);
    case CC_MASK4: return Tab<T>::GG(J, ki) != (T)0 ? v : mk<T>((T)0, (T)0);
    default: return mk<T>((T)0, (T)0);
  }
}

// i kx, i ky and -i ky without a (lh, ny) table load per element: the
// tables hold kx by column and ky by row, zeroed on the column kx = nx/2 and
// the row ky = ny/2 (fft.f90:54-81), so kx(jx, js) is row 0's entry (kxc,
// held by the column's thread) but zero on row ny/2, and ky(jx, js) column
// 0's entry (kys, a shared-memory copy of that column) but zero on column
// lh - 1: the same values as the table.  Other codes read the tables.
template <typename T>
__device__ __forceinline__ typename CT<T>::type apply_coef_k(int code, typename CT<T>::type v, int jx, int js,
                                                             T kxc, const T* kys, const ColJob& J) {
  switch (code) {
    case CC_IKX: return ik(v, js == J.ny_small / 2 ? (T)0 : kxc);
    case CC_IKY: return ik(v, jx == J.lh - 1 ? (T)0 : kys[js]);
    case CC_MIKY: return ik(v, -(jx == J.lh - 1 ? (T)0 : kys[js]));
    default: return apply_coef<T>(code, v, jx, js, J);
  }
}

// Runtime lengths (plans Pin, Pout): the fixed-length kernels below cover
// the lengths the workloads use.
template <typename T, int TX, typename CIn>
__global__ void __launch_bounds__(256) k_cols(ColJob J, FftPlanDev Pin, FftPlanDev Pout) {
  typedef typename CT<T>::type C;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ny_in = J.ny_in, ny_out = J.ny_out;
  const int nymax = max(ny_in, ny_out);
  C* IN = reinterpret_cast<C*>(smraw);
  C* A = IN + J.nin * ny_in * TX;
  C* B = A + nymax * TX;
  const int jx0 = blockIdx.x * TX;
  const int lev = blockIdx.y;
  for (int i = 0; i < J.nin; ++i) {
    const CIn* src = reinterpret_cast<const CIn*>(J.in[i]) + (size_t)lev * J.ps_in + (size_t)blockIdx.z * J.fs_in;
    for (int t = threadIdx.x; t < ny_in * TX; t += blockDim.x) {
      const int row = t / TX, b = t - row * TX;
      const int jx = jx0 + b;
      C v = mk<T>((T)0, (T)0);
      if (jx < J.ncols) {
        const CIn x = src[(size_t)row * J.wc_in + jx];
        v = mk<T>(cvt<T, decltype(x.x)>(x.x), cvt<T, decltype(x.y)>(x.y));
      }
      IN[i * ny_in * TX + row * TX + b] = v;
    }
  }
  __syncthreads();
  if (J.dir & DIR_FWD) {
    for (int i = 0; i < J.nin; ++i) {
      C* xi = IN + i * ny_in * TX;
      C* r = fft_smem<T, true>(xi, A, TX, 0, Pin, -1);
      if (r != xi) {
        for (int t = threadIdx.x; t < ny_in * TX; t += blockDim.x) xi[t] = r[t];
        __syncthreads();
      }
    }
  }
  const int nys = J.ny_small;
  const int nyb = (J.map == MAP_SAME) ? nys : (J.map == MAP_PAD ? ny_out : ny_in);
  for (int o = 0; o < J.nout; ++o) {
    for (int t = threadIdx.x; t < ny_out * TX; t += blockDim.x) {
      const int row = t / TX, b = t - row * TX;
      const int jx = jx0 + b;
      int rin, js;
      if (J.map == MAP_SAME) { rin = row; js = row; }
      else if (J.map == MAP_PAD) {  // padd.f90:123-133
        if (row < nys / 2) rin = row;
        else if (row > nyb - nys / 2) rin = row - (nyb - nys);
        else rin = -1;
        js = rin;
      } else {  // unpadd.f90:143-155
        if (row < nys / 2) rin = row;
        else if (row == nys / 2) rin = -1;
        else rin = row + (nyb - nys);
        js = row;
      }
      C acc = mk<T>((T)0, (T)0);
      if (rin >= 0 && jx < J.ncols) {
        for (int i = 0; i < J.nin; ++i) {
          const int code = J.coef[o][i];
          if (code != CC_NONE) acc = cadd(acc, apply_coef<T>(code, IN[i * ny_in * TX + rin * TX + b], jx, js, J));
        }
      }
      A[row * TX + b] = acc;
    }
    __syncthreads();
    C* r = A;
    if ((J.inv_mask >> o) & 1u) r = fft_smem<T, true>(A, B, TX, 0, Pout, +1);
    C* dst = reinterpret_cast<C*>(J.out[o]) + (size_t)lev * J.ps_out + (size_t)blockIdx.z * J.fs_out;
    for (int t = threadIdx.x; t < ny_out * TX; t += blockDim.x) {
      const int row = t / TX, b = t - row * TX;
      const int jx = jx0 + b;
      if (jx < J.ncols) dst[(size_t)row * J.wc_out + jx] = r[row * TX + b];
    }
    __syncthreads();
  }
}


// Fixed-length y pass (NIN, NOUT at compile time).  Thread t owns column
// b = t % TX of the tile and the rows r0 = t / TX + k * (256 / TX): global
// loads and stores walk the column by pointer increments, the row map of
// padd/unpadd follows from NIN, NOUT, and for single-input jobs the
// coefficient code is dispatched once per output instead of per element.
template <typename T, int CODE>
__device__ __forceinline__ typename CT<T>::type apply_coef_ct(typename CT<T>::type v, int jx, int js,
                                                              const ColJob& J) {
  typedef typename CT<T>::type C;
  const size_t ki = (size_t)jx + (size_t)J.lh * js;
  if constexpr (CODE == CC_ONE) return v;
  else if constexpr (CODE == CC_G) return cscale(v, Tab<T>::G(J, ki));
  else if constexpr (CODE == CC_GG) return cscale(v, Tab<T>::GG(J, ki));
  else if constexpr (CODE == CC_IKX) return ik(v, Tab<T>::kx(J, ki));
  else if constexpr (CODE == CC_IKY) return ik(v, Tab<T>::ky(J, ki));
  else if constexpr (CODE == CC_MIKY) return ik(v, -Tab<T>::ky(J, ki));
  else if constexpr (CODE == CC_KILL) {
    if (jx == J.lh - 1 || js == J.ny_small / 2) return mk<T>((T)0, (T)0);
    return v;
  } else if constexpr (CODE == CC_MASK) return Tab<T>::G(J, ki) != (T)0 ? v : mk<T>((T)0, (T)0);
  else if constexpr (CODE == CC_MASK4) return Tab<T>::GG(J, ki) != (T)0 ? v : mk<T>((T)0, (T)0);
  else return mk<T>((T)0, (T)0);
}
template <int NIN, int NOUT>
__device__ __forceinline__ void row_map(int row, int nys, int& rin, int& js) {
  if constexpr (NIN == NOUT) {
    rin = row; js = row;
  } else if constexpr (NOUT > NIN) {  // padd.f90:123-133
    if (row < nys / 2) rin = row;
    else if (row > NOUT - nys / 2) rin = row - (NOUT - nys);
    else rin = -1;
    js = rin;
  } else {  // unpadd.f90:143-155
    if (row < nys / 2) rin = row;
    else if (row == nys / 2) rin = -1;
    else rin = row + (NIN - nys);
    js = row;
  }
}
template <typename T, int TX, int NIN, int NOUT, int CODE>
__device__ __forceinline__ void coef_rows(const typename CT<T>::type* __restrict__ in, typename CT<T>::type* a,
                                          int b, int r0, int jx, bool colok, const ColJob& J) {
  typedef typename CT<T>::type C;
  constexpr int RS = 256 / TX;
  for (int row = r0; row < NOUT; row += RS) {
    int rin, js;
    row_map<NIN, NOUT>(row, J.ny_small, rin, js);
    C v = mk<T>((T)0, (T)0);
    if (rin >= 0 && colok) v = apply_coef_ct<T, CODE>(in[sk(rin) * TX + b], jx, js, J);
    a[sk(row) * TX + b] = v;
  }
}
template <typename T, int TX, typename CIn, int NIN, int NOUT>
__global__ void __launch_bounds__(256) k_colsf(ColJob J, FftPlanDev Pin, FftPlanDev Pout) {
  typedef typename CT<T>::type C;
  static_assert(256 % TX == 0, "tile width divides the block");
  constexpr int RS = 256 / TX;
  constexpr int PIN = skn(NIN), PMAX = skn(NIN > NOUT ? NIN : NOUT);
  extern __shared__ __align__(16) unsigned char smraw[];
  C* IN = reinterpret_cast<C*>(smraw);
  C* A = IN + J.nin * PIN * TX;
  C* B = A + PMAX * TX;
  C* twi = B + PMAX * TX;
  C* two = twi + NIN;
  for (int t = threadIdx.x; t < NIN; t += 256) twi[t] = UnitSel<T>::get(Pin, t);
  for (int t = threadIdx.x; t < NOUT; t += 256) two[t] = UnitSel<T>::get(Pout, t);
  const int b = threadIdx.x % TX, r0 = threadIdx.x / TX;
  const int jx = blockIdx.x * TX + b;
  const bool colok = jx < J.ncols;
  const int lev = blockIdx.y;
  for (int i = 0; i < J.nin; ++i) {
    const CIn* src = reinterpret_cast<const CIn*>(J.in[i]) + (size_t)lev * J.ps_in + (size_t)blockIdx.z * J.fs_in +
                     jx + (size_t)r0 * J.wc_in;
    const int step = RS * J.wc_in;
    C* xi = IN + i * PIN * TX;
    for (int row = r0; row < NIN; row += RS, src += step) {
      C v = mk<T>((T)0, (T)0);
      if (colok) {
        const CIn x = *src;
        v = mk<T>(cvt<T, decltype(x.x)>(x.x), cvt<T, decltype(x.y)>(x.y));
      }
      xi[sk(row) * TX + b] = v;
    }
  }
  __syncthreads();
  if (J.dir & DIR_FWD) {
    for (int i = 0; i < J.nin; ++i) {
      C* xi = IN + i * PIN * TX;
      C* r = fft_ct<T, true, NIN, TX, -1, 256, CtMaxR<T>::v>(xi, A, twi, TX);
      if (r != xi) {
        for (int t = threadIdx.x; t < PIN * TX; t += 256) xi[t] = r[t];
        __syncthreads();
      }
    }
  }
  for (int o = 0; o < J.nout; ++o) {
    // single-input jobs: the coefficient dispatched once per output; any code
    // not listed (and every multi-input job) takes the per-element dispatch
    bool done = J.nin == 1;
    if (J.nin == 1) {
      switch (J.coef[o][0]) {
        case CC_NONE: coef_rows<T, TX, NIN, NOUT, CC_NONE>(IN, A, b, r0, jx, colok, J); break;
        case CC_ONE: coef_rows<T, TX, NIN, NOUT, CC_ONE>(IN, A, b, r0, jx, colok, J); break;
        case CC_G: coef_rows<T, TX, NIN, NOUT, CC_G>(IN, A, b, r0, jx, colok, J); break;
        case CC_GG: coef_rows<T, TX, NIN, NOUT, CC_GG>(IN, A, b, r0, jx, colok, J); break;
        case CC_IKX: coef_rows<T, TX, NIN, NOUT, CC_IKX>(IN, A, b, r0, jx, colok, J); break;
        case CC_IKY: coef_rows<T, TX, NIN, NOUT, CC_IKY>(IN, A, b, r0, jx, colok, J); break;
        case CC_MIKY: coef_rows<T, TX, NIN, NOUT, CC_MIKY>(IN, A, b, r0, jx, colok, J); break;
        case CC_KILL: coef_rows<T, TX, NIN, NOUT, CC_KILL>(IN, A, b, r0, jx, colok, J); break;
        case CC_MASK: coef_rows<T, TX, NIN, NOUT, CC_MASK>(IN, A, b, r0, jx, colok, J); break;
        case CC_MASK4: coef_rows<T, TX, NIN, NOUT, CC_MASK4>(IN, A, b, r0, jx, colok, J); break;
        default: done = false; break;
      }
    }
    if (!done) {
      for (int row = r0; row < NOUT; row += RS) {
        int rin, js;
        row_map<NIN, NOUT>(row, J.ny_small, rin, js);
        C acc = mk<T>((T)0, (T)0);
        if (rin >= 0 && colok) {
          for (int i = 0; i < J.nin; ++i) {
            const int code = J.coef[o][i];
            if (code != CC_NONE) acc = cadd(acc, apply_coef<T>(code, IN[i * PIN * TX + sk(rin) * TX + b], jx, js, J));
          }
        }
        A[sk(row) * TX + b] = acc;
      }
    }
    __syncthreads();
    C* r = A;
    if ((J.inv_mask >> o) & 1u) r = fft_ct<T, true, NOUT, TX, +1, 256, CtMaxR<T>::v>(A, B, two, TX);
    if (colok) {
      C* dst = reinterpret_cast<C*>(J.out[o]) + (size_t)lev * J.ps_out + (size_t)blockIdx.z * J.fs_out + jx +
               (size_t)r0 * J.wc_out;
      const int step = RS * J.wc_out;
      for (int row = r0; row < NOUT; row += RS, dst += step) *dst = r[sk(row) * TX + b];
    }
    __syncthreads();
  }
}

// Register-resident y pass for one input and same-length outputs, N = R * R
// (R = 16: 256 points; R = 8: 64).  Four-step split n = n1 + R n2,
// k = k2 + R k1: thread q of a column holds the R elements x[q + R i]
// (n1 = q) or X[q + R i] (k2 = q), so global loads and stores touch rows
// q + R i in both layouts.  Forward: DFT_R over n2 in registers, twiddle
// W_N^(n1 k2), one exchange through shared memory, DFT_R over n1; the
// spectrum then sits in registers, the coefficient of each output is
// applied there, and the inverse runs the same steps in reverse order
// (DFT_R over k1, twiddle, exchange, DFT_R over k2).  Two trips through
// shared memory per transform instead of one per radix pass; every thread
// has its R loads in flight at once.
template <typename T, int R>
__device__ __forceinline__ void dft_r(typename CT<T>::type* v, int sign) {
  typedef typename CT<T>::type C;
  if constexpr (R == 16) dft16<C, T>(v, sign);
  else if constexpr (R == 8) dft8<C, T>(v, sign);
  else dft4(v, sign);
}

// Persistent form: a CTA walks the (kx tile, level, field set) items of the
// job with stride gridDim.x; each thread stages its R input elements of the
// next item into shared memory with cp.async while the current item is
// transformed, so the loads of one item overlap the arithmetic of the
// previous one.  A thread reads back only what it staged itself, so the
// staging needs no barrier.  8-byte elements (FP32 complex).
template <typename T, int TX, typename CIn, int R>
__global__ void __launch_bounds__(TX * R, 3) k_colsr(ColJob J, FftPlanDev P, int ntile, int nitems) {
  typedef typename CT<T>::type C;
  static_assert(sizeof(CIn) == 8 && sizeof(C) == 8, "8-byte complex elements");
  constexpr int N = R * R;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* S = reinterpret_cast<C*>(smraw);          // exchange: element (i, q) of column b at (i * R + q) * TX + b
  CIn* G = reinterpret_cast<CIn*>(S + N * TX);  // staged input, same index
  C* tw = reinterpret_cast<C*>(G + N * TX);    // exp(-2 pi i m / N), m < N
  T* kys = reinterpret_cast<T*>(tw + N);        // ky of row js (column 0 of the table), js < N
  for (int t = threadIdx.x; t < N; t += TX * R) {
    tw[t] = UnitSel<T>::get(P, t);
    kys[t] = Tab<T>::ky(J, (size_t)J.lh * t);
  }
  const int b = threadIdx.x % TX, q = threadIdx.x / TX;
  const int nlev = J.nlev;
  auto stage = [&](int item) {
    const int tile = item % ntile, rest = item / ntile;
    const int lev = rest % nlev, z = rest / nlev;
    const int jx = tile * TX + b;
    const bool ok = jx < J.ncols;
    const CIn* src = reinterpret_cast<const CIn*>(J.in[0]) + (size_t)lev * J.ps_in + (size_t)z * J.fs_in +
                     (ok ? jx : 0) + (size_t)q * J.wc_in;
    const size_t step = (size_t)R * J.wc_in;
#pragma unroll
    for (int i = 0; i < R; ++i) cp_async8(&G[(i * R + q) * TX + b], src + i * step, ok ? 8 : 0);
    cp_async_commit();
  };
  if ((int)blockIdx.x < nitems) stage(blockIdx.x);
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int tile = item % ntile, rest = item / ntile;
    const int lev = rest % nlev, z = rest / nlev;
    const int jx = tile * TX + b;
    const bool colok = jx < J.ncols;
    C v[R];
    cp_async_wait_all();
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const CIn x = G[(i * R + q) * TX + b];
      v[i] = mk<T>(x.x, x.y);
    }
    if (item + (int)gridDim.x < nitems) stage(item + gridDim.x);
    __syncthreads();  // the previous item's readers of S are done (and the twiddle table is in place)
    if (J.dir & DIR_FWD) {
      dft_r<T, R>(v, -1);  // over n2: v[i] = y[n1 = q][k2 = i]
#pragma unroll
      for (int i = 1; i < R; ++i) v[i] = cmul(v[i], tw[q * i]);
#pragma unroll
      for (int i = 0; i < R; ++i) S[(i * R + q) * TX + b] = v[i];
      __syncthreads();
#pragma unroll
      for (int i = 0; i < R; ++i) v[i] = S[(q * R + i) * TX + b];  // y[n1 = i][k2 = q]
      dft_r<T, R>(v, -1);  // over n1: v[i] = X[q + R i]
    }
    const T kxc = colok ? Tab<T>::kx(J, (size_t)jx) : (T)0;  // row 0: kx of the column
    for (int o = 0; o < J.nout; ++o) {
      C y[R];
      const int code = J.coef[o][0];
#pragma unroll
      for (int i = 0; i < R; ++i)
        y[i] = colok ? apply_coef_k<T>(code, v[i], jx, q + R * i, kxc, kys, J) : mk<T>((T)0, (T)0);
      if ((J.inv_mask >> o) & 1u) {
        dft_r<T, R>(y, +1);  // over k1: y[i] = z[k2 = q][n1 = i]
#pragma unroll
        for (int i = 1; i < R; ++i) y[i] = cmul(y[i], cconj(tw[q * i]));
        __syncthreads();  // earlier readers of S are done
#pragma unroll
        for (int i = 0; i < R; ++i) S[(i * R + q) * TX + b] = y[i];
        __syncthreads();
#pragma unroll
        for (int i = 0; i < R; ++i) y[i] = S[(q * R + i) * TX + b];  // z[k2 = i][n1 = q]
        dft_r<T, R>(y, +1);  // over k2: y[i] = x[q + R i]
      }
      if (colok) {
        C* dst = reinterpret_cast<C*>(J.out[o]) + (size_t)lev * J.ps_out + (size_t)z * J.fs_out + jx +
                 (size_t)q * J.wc_out;
        const size_t step = (size_t)R * J.wc_out;
#pragma unroll
        for (int i = 0; i < R; ++i) dst[i * step] = y[i];
      }
    }
  }
  cp_async_wait_all();  // nothing in flight at exit
}

// Register-resident 3/2 padding and truncation (one input, one output, unit
// coefficient): small length NS = 16 A, big length NB = 16 B, B = 3A/2.  A
// transform of length N = 16 L splits as n = n1 + L n2, k = k2 + 16 k1, so
// thread q < 16 of a column holds the spectral rows q + 16 k1 (k1 < L) and
// thread t < L the physical rows t + L n2 (n2 < 16); one exchange through
// shared memory turns one layout into the other.  In the spectral layout
// the padding and truncation maps (padd.f90:123-133, unpadd.f90:143-155)
// stay inside a thread: small row q + 16 i is big row q + 16 i for i < A/2
// and q + 16 (i + B - A) for i >= A/2, and the small Nyquist row (q = 0,
// i = A/2) is dropped.  The padded spectrum's zero rows are never loaded.
template <typename T, int TX, int L, int M>
__device__ __forceinline__ void fwd_16l(typename CT<T>::type (&v)[M], typename CT<T>::type* S,
                                        const typename CT<T>::type* tw, int r, int b) {
  // on entry thread r < L holds x[r + L n2] in v[n2]; on exit thread r < 16
  // holds X[r + 16 k1] in v[k1]
  __syncthreads();  // the twiddle table is in place and earlier readers of S are done
  if (r < L) {
    dft_n<T, 16>(v, -1);  // over n2: v[k2] = y[n1 = r][k2]
#pragma unroll
    for (int k2 = 1; k2 < 16; ++k2) v[k2] = cmul(v[k2], tw[r * k2]);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) S[(r * 16 + k2) * TX + b] = v[k2];
  }
  __syncthreads();
  if (r < 16) {
#pragma unroll
    for (int n1 = 0; n1 < L; ++n1) v[n1] = S[(n1 * 16 + r) * TX + b];
    dft_n<T, L>(v, -1);  // over n1: v[k1] = X[r + 16 k1]
  }
}
template <typename T, int TX, int L, int M>
__device__ __forceinline__ void inv_16l(typename CT<T>::type (&v)[M], typename CT<T>::type* S,
                                        const typename CT<T>::type* tw, int r, int b) {
  // unnormalised inverse: on entry thread r < 16 holds X[r + 16 k1] in
  // v[k1]; on exit thread r < L holds x[r + L n2] in v[n2]
  __syncthreads();
  if (r < 16) {
    dft_n<T, L>(v, +1);  // over k1: v[n1] = z[k2 = r][n1]
#pragma unroll
    for (int n1 = 1; n1 < L; ++n1) v[n1] = cmul(v[n1], cconj(tw[r * n1]));
#pragma unroll
    for (int n1 = 0; n1 < L; ++n1) S[(n1 * 16 + r) * TX + b] = v[n1];
  }
  __syncthreads();
  if (r < L) {
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) v[k2] = S[(r * 16 + k2) * TX + b];
    dft_n<T, 16>(v, +1);  // over k2: v[n2] = x[r + L n2]
  }
}
template <int NIN, int NOUT> struct PadShape {
  static constexpr bool pad = NOUT > NIN;
  static constexpr int ns = pad ? NIN : NOUT, nb = pad ? NOUT : NIN, a = ns / 16, b = nb / 16;
  static constexpr int tt = b > 16 ? b : 16;  // threads per column (and register array length)
};
template <typename T, int TX, typename CIn, int NIN, int NOUT>
__global__ void __launch_bounds__(TX * PadShape<NIN, NOUT>::tt, 2) k_colsr_pad(ColJob J, FftPlanDev Pin,
                                                                                 FftPlanDev Pout) {
  typedef typename CT<T>::type C;
  typedef PadShape<NIN, NOUT> PS;
  constexpr int A = PS::a, B = PS::b, NS = PS::ns, NB = PS::nb, TT = PS::tt;
  static_assert(NS == 16 * A && NB == 16 * B && 2 * B == 3 * A && A % 2 == 0, "3/2 padding of 16 A rows");
  extern __shared__ __align__(16) unsigned char smraw[];
  C* S = reinterpret_cast<C*>(smraw);  // element (n1, k2) of column b at (n1 * 16 + k2) * TX + b
  C* tws = S + 16 * B * TX;            // exp(-2 pi i m / NS), m < NS
  C* twb = tws + NS;                   // exp(-2 pi i m / NB), m < NB
  for (int t = threadIdx.x; t < NS; t += TX * TT) tws[t] = UnitSel<T>::get(PS::pad ? Pin : Pout, t);
  for (int t = threadIdx.x; t < NB; t += TX * TT) twb[t] = UnitSel<T>::get(PS::pad ? Pout : Pin, t);
  const int b = threadIdx.x % TX, r = threadIdx.x / TX;
  const int jx = blockIdx.x * TX + b;
  const bool colok = jx < J.ncols;
  const CIn* src = reinterpret_cast<const CIn*>(J.in[0]) + (size_t)blockIdx.y * J.ps_in +
                   (size_t)blockIdx.z * J.fs_in + (colok ? jx : 0);
  C* dst = reinterpret_cast<C*>(J.out[0]) + (size_t)blockIdx.y * J.ps_out + (size_t)blockIdx.z * J.fs_out + jx;
  auto load = [&](C& d, int row) {
    const CIn x = src[(size_t)row * J.wc_in];
    d = mk<T>(cvt<T, decltype(x.x)>(x.x), cvt<T, decltype(x.y)>(x.y));
  };
  C v[TT];
  if constexpr (PS::pad) {
    if (J.dir & DIR_FWD) {
      if (r < A) {
#pragma unroll
        for (int n2 = 0; n2 < 16; ++n2) load(v[n2], r + A * n2);
      }
      fwd_16l<T, TX, A>(v, S, tws, r, b);
    } else if constexpr (sizeof(CIn) > 8) {
      // 16-byte inputs: every thread row loads (about NS / TT rows each) and
      // stages them in S, so the loads in flight fit the register budget
#pragma unroll
      for (int k = 0; k < (NS + TT - 1) / TT; ++k) {
        const int row = r + k * TT;
        if (row < NS) {
          C x;
          load(x, row);
          S[row * TX + b] = x;
        }
      }
      __syncthreads();
      if (r < 16) {
#pragma unroll
        for (int i = 0; i < A; ++i) v[i] = S[(r + 16 * i) * TX + b];
      }
    } else if (r < 16) {
#pragma unroll
      for (int i = 0; i < A; ++i) load(v[i], r + 16 * i);
    }
    if (r < 16) {  // v[m] = padded X[r + 16 m], m < B
#pragma unroll
      for (int i = A / 2; i < A; ++i) v[i + B - A] = v[i];
#pragma unroll
      for (int m = A / 2; m < B - A / 2; ++m) v[m] = mk<T>((T)0, (T)0);
      if (r == 0) v[B - A / 2] = mk<T>((T)0, (T)0);
    }
    inv_16l<T, TX, B>(v, S, twb, r, b);
    if (colok && r < B) {
#pragma unroll
      for (int n2 = 0; n2 < 16; ++n2) dst[(size_t)(r + B * n2) * J.wc_out] = v[n2];
    }
  } else {
    if (r < B) {
#pragma unroll
      for (int n2 = 0; n2 < 16; ++n2) load(v[n2], r + B * n2);
    }
    fwd_16l<T, TX, B>(v, S, twb, r, b);
    if (r < 16) {  // v[i] = truncated X[r + 16 i], i < A
#pragma unroll
      for (int i = A / 2; i < A; ++i) v[i] = v[i + B - A];
      if (r == 0) v[A / 2] = mk<T>((T)0, (T)0);
    }
    inv_16l<T, TX, A>(v, S, tws, r, b);
    if (colok && r < A) {
#pragma unroll
      for (int n2 = 0; n2 < 16; ++n2) dst[(size_t)(r + A * n2) * J.wc_out] = v[n2];
    }
  }
}

// Several inputs summed per output (the stress and flux divergences:
// out_o = sum_i coef(o,i) * in_i), at most NO outputs: each input is loaded
// and transformed in turn and its contributions are accumulated in shared
// memory (each thread owns its accumulator slots, so no barrier guards
// them), so every input is read once and no spectrum goes through global
// memory.  Same four-step split and exchange as k_colsr.
template <typename T, int TX, typename CIn, int R, int NO>
__global__ void __launch_bounds__(TX * R, 2) k_colsr_sum(ColJob J, FftPlanDev P) {
  typedef typename CT<T>::type C;
  constexpr int N = R * R;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* S = reinterpret_cast<C*>(smraw);  // exchange: element (i, q) of column b at (i * R + q) * TX + b
  C* A = S + N * TX;                   // NO accumulators, same index
  C* tw = A + NO * N * TX;             // exp(-2 pi i m / N), m < N
  T* kys = reinterpret_cast<T*>(tw + N);  // ky of row js (column 0 of the table), js < N
  for (int t = threadIdx.x; t < N; t += TX * R) {
    tw[t] = UnitSel<T>::get(P, t);
    kys[t] = Tab<T>::ky(J, (size_t)J.lh * t);
  }
  const int b = threadIdx.x % TX, q = threadIdx.x / TX;
  const int jx = blockIdx.x * TX + b;
  const bool colok = jx < J.ncols;
  const T kxc = colok ? Tab<T>::kx(J, (size_t)jx) : (T)0;  // row 0: kx of the column
  const int lev = blockIdx.y;
#pragma unroll
  for (int o = 0; o < NO; ++o)
#pragma unroll
    for (int i = 0; i < R; ++i) A[o * N * TX + (i * R + q) * TX + b] = mk<T>((T)0, (T)0);
  for (int in = 0; in < J.nin; ++in) {
    C v[R];
    const CIn* src = reinterpret_cast<const CIn*>(J.in[in]) + (size_t)lev * J.ps_in + (size_t)blockIdx.z * J.fs_in +
                     (colok ? jx : 0) + (size_t)q * J.wc_in;
    const size_t step = (size_t)R * J.wc_in;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      v[i] = mk<T>((T)0, (T)0);
      if (colok) {
        const CIn x = src[i * step];
        v[i] = mk<T>(cvt<T, decltype(x.x)>(x.x), cvt<T, decltype(x.y)>(x.y));
      }
    }
    __syncthreads();  // the previous input's readers of S are done (and the twiddle table is in place)
    if (J.dir & DIR_FWD) {
      dft_r<T, R>(v, -1);
#pragma unroll
      for (int i = 1; i < R; ++i) v[i] = cmul(v[i], tw[q * i]);
#pragma unroll
      for (int i = 0; i < R; ++i) S[(i * R + q) * TX + b] = v[i];
      __syncthreads();
#pragma unroll
      for (int i = 0; i < R; ++i) v[i] = S[(q * R + i) * TX + b];
      dft_r<T, R>(v, -1);  // v[i] = X_in[q + R i]
    }
    if (colok) {
#pragma unroll 1
      for (int o = 0; o < NO; ++o) {
        const int code = o < J.nout ? J.coef[o][in] : CC_NONE;
        if (code != CC_NONE) {
          C* a = A + o * N * TX + q * TX + b;
#pragma unroll
          for (int i = 0; i < R; ++i)
            a[i * R * TX] = cadd(a[i * R * TX], apply_coef_k<T>(code, v[i], jx, q + R * i, kxc, kys, J));
        }
      }
    }
  }
  for (int o = 0; o < J.nout && o < NO; ++o) {
    C y[R];
#pragma unroll
    for (int i = 0; i < R; ++i) y[i] = A[o * N * TX + (i * R + q) * TX + b];
    if ((J.inv_mask >> o) & 1u) {
      dft_r<T, R>(y, +1);
#pragma unroll
      for (int i = 1; i < R; ++i) y[i] = cmul(y[i], cconj(tw[q * i]));
      __syncthreads();
#pragma unroll
      for (int i = 0; i < R; ++i) S[(i * R + q) * TX + b] = y[i];
      __syncthreads();
#pragma unroll
      for (int i = 0; i < R; ++i) y[i] = S[(q * R + i) * TX + b];
      dft_r<T, R>(y, +1);
    }
    if (colok) {
      C* dst = reinterpret_cast<C*>(J.out[o]) + (size_t)lev * J.ps_out + (size_t)blockIdx.z * J.fs_out + jx +
               (size_t)q * J.wc_out;
      const size_t step = (size_t)R * J.wc_out;
#pragma unroll
      for (int i = 0; i < R; ++i) dst[i * step] = y[i];
    }
  }
}

// rows per CTA of the x-pass kernels (default when a job gives none)
template <typename T>
inline int rows_pc(int nx) {
  const int m = nx / 2;
  int r = 256 / (m / 4 > 0 ? m / 4 : 1);
  if (r < 1) r = 1;
  if (r > 16) r = 16;
  return r;
}

// fixed-length launchers (fft_fixed.cu): true when the job's length has a
// fixed-length instantiation and it was launched
template <typename T, typename TIn>
bool launch_rows_r2c_fixed(const RowJob& J, const RealPlanDev& P, int rpc, size_t sm, cudaStream_t s);
template <typename T, typename TOut>
bool launch_rows_c2r_fixed(const RowJob& J, const RealPlanDev& P, int rpc, size_t sm, cudaStream_t s);
template <typename T, int TX, typename CIn>
bool launch_cols_fixed(const ColJob& J, const FftPlanDev& Pin, const FftPlanDev& Pout, size_t sm, dim3 grid,
                       cudaStream_t s);

}  // namespace les
