// Line-FFT engine for the pseudo-spectral Navier-Stokes kernels (sm_103a).
//
// A "line" is one 1-D transform of length N (a power of two, 16..1024).  A
// group of G = N/E lanes of one warp owns a line; every lane keeps E = 16 (or
// 32 for N = 1024) complex values in registers and the line is exchanged
// between radix passes through a padded shared-memory buffer.  The passes are
// the Stockham autosort formulation (Govindaraju et al., "High performance
// discrete Fourier transforms on graphics processors", SC'08): for pass
// (Ns, R) the butterfly j reads x[j + r N/R], multiplies by W_{Ns R}^{r (j mod
// Ns)}, does a radix-R DFT in registers and writes x'[(j - j mod Ns) R + j mod
// Ns + r Ns].  Radices are 16,16,...,N/16^a.  Twiddles come from a table
// generated in FP64 on the host and rounded to the working precision.
//
// Sign convention: S = -1 forward (exp(-2 pi i nk/N)), S = +1 inverse
// (unnormalised).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sdns {

template <typename R> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) x, decltype(C::x) y) { C c; c.x = x; c.y = y; return c; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return mk<C>(a.x, -a.y); }
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) { return mk<C>(a.x * s, a.y * s); }
// multiply by S*i  (S=-1: -i z, S=+1: i z)
template <int S, typename C> __device__ __forceinline__ C mul_si(C a) {
  return S < 0 ? mk<C>(a.y, -a.x) : mk<C>(-a.y, a.x);
}
// multiply by the constant (cr + S*ci*i)
template <int S, typename C> __device__ __forceinline__ C mulc(C a, double cr, double ci) {
  using T = decltype(C::x);
  const T r = (T)cr, i = (T)(S * ci);
  return mk<C>(a.x * r - a.y * i, a.x * i + a.y * r);
}

// constants cos(pi/8), sin(pi/8), sqrt(1/2)
#define SDNS_C8 0.92387953251128675613
#define SDNS_S8 0.38268343236508977173
#define SDNS_R2 0.70710678118654752440

template <int S, typename C> __device__ __forceinline__ void dft2(C& a, C& b) {
  C t = a; a = cadd(t, b); b = csub(t, b);
}
template <int S, typename C> __device__ __forceinline__ void dft4(C& a, C& b, C& c, C& d) {
  C t0 = cadd(a, c), t1 = csub(a, c), t2 = cadd(b, d), t3 = mul_si<S>(csub(b, d));
  a = cadd(t0, t2); c = csub(t0, t2); b = cadd(t1, t3); d = csub(t1, t3);
}
template <int S, typename C> __device__ __forceinline__ void dft8(C* v) {
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<S>(e0, e1, e2, e3);
  dft4<S>(o0, o1, o2, o3);
  o1 = mulc<S>(o1, SDNS_R2, SDNS_R2);   // W8^1
  o2 = mul_si<S>(o2);                   // W8^2
  o3 = mulc<S>(o3, -SDNS_R2, SDNS_R2);  // W8^3
  v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1); v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2); v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3); v[7] = csub(e3, o3);
}
// W16^m = (cos(pi m/8), S sin(pi m/8))
template <int S, typename C> __device__ __forceinline__ void dft16(C* v) {
  // n = 4 n1 + n2 ; k = k1 + 4 k2
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4<S>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
  // now v[4 k1 + n2] holds y[n2][k1]; twiddle by W16^{n2 k1}
  v[4 * 1 + 1] = mulc<S>(v[4 * 1 + 1], SDNS_C8, SDNS_S8);    // m=1
  v[4 * 2 + 1] = mulc<S>(v[4 * 2 + 1], SDNS_R2, SDNS_R2);    // m=2
  v[4 * 3 + 1] = mulc<S>(v[4 * 3 + 1], SDNS_S8, SDNS_C8);    // m=3
  v[4 * 1 + 2] = mulc<S>(v[4 * 1 + 2], SDNS_R2, SDNS_R2);    // m=2
  v[4 * 2 + 2] = mul_si<S>(v[4 * 2 + 2]);                     // m=4
  v[4 * 3 + 2] = mulc<S>(v[4 * 3 + 2], -SDNS_R2, SDNS_R2);   // m=6
  v[4 * 1 + 3] = mulc<S>(v[4 * 1 + 3], SDNS_S8, SDNS_C8);    // m=3
  v[4 * 2 + 3] = mulc<S>(v[4 * 2 + 3], -SDNS_R2, SDNS_R2);   // m=6
  v[4 * 3 + 3] = mulc<S>(v[4 * 3 + 3], -SDNS_C8, -SDNS_S8);  // m=9
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4<S>(v[4 * k1 + 0], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
  // v[4 k1 + k2] holds X[k1 + 4 k2]; transpose to natural order
  C t[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = t[i];
}

// cos(pi k/16) for k = 0..8; sin(pi k/16) = cos(pi (8-k)/16)
__host__ __device__ constexpr double c16(int k) {
  return k == 0 ? 1.0 : k == 1 ? 0.98078528040323044913 : k == 2 ? SDNS_C8 : k == 3 ? 0.83146961230254523708
       : k == 4 ? SDNS_R2 : k == 5 ? 0.55557023301960222474 : k == 6 ? SDNS_S8 : k == 7 ? 0.19509032201612826785
       : 0.0;
}
__host__ __device__ constexpr double cos16(int k) { return k <= 8 ? c16(k) : -c16(16 - k); }  // k = 0..15

// 32-point DFT in registers: radix 2 over two 16-point DFTs (even / odd inputs),
// X[k] = E[k] + W32^k O[k], X[k+16] = E[k] - W32^k O[k]; natural order out.
template <int S, typename C> __device__ __forceinline__ void dft32(C* v) {
  C e[16], o[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) { e[m] = v[2 * m]; o[m] = v[2 * m + 1]; }
  dft16<S>(e);
  dft16<S>(o);
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    C t = o[k];
    if (k == 8) t = mul_si<S>(t);
    else if (k != 0) t = mulc<S>(t, cos16(k), k < 8 ? c16(8 - k) : c16(k - 8));
    v[k] = cadd(e[k], t);
    v[k + 16] = csub(e[k], t);
  }
}

template <int R, int S, typename C> __device__ __forceinline__ void dftR(C* v) {
  if constexpr (R == 2) dft2<S>(v[0], v[1]);
  else if constexpr (R == 4) dft4<S>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 8) dft8<S>(v);
  else if constexpr (R == 16) dft16<S>(v);
  else dft32<S>(v);
}

// padded shared-memory index of line position p (breaks stride-16 bank conflicts)
__device__ __forceinline__ int padp(int p) { return p + (p >> 4); }
__host__ __device__ inline int line_ld(int n) {
  int ld = n + ((n - 1) >> 4);
  return (ld & 1) ? ld : ld + 1;
}
// twiddle table length for an axis of n points: sum over passes of R*Ns
__host__ __device__ inline int tw_len(int n) {
  int len = 0, ns = 1;
  while (ns < n) { int r = (n / ns) >= 16 ? 16 : n / ns; len += r * ns; ns *= r; }
  return len;
}

// Each axis's table ends with the full table W_n^m, m = 0..n-1 (forward), which
// the two-pass radix-32 transforms index directly.
__host__ __device__ inline int tw_total(int n) { return tw_len(n) + n; }

// One Stockham pass of radix R on a line held in `buf` (padded positions).
template <int R, int E, int S, typename C>
__device__ __forceinline__ void stockham_pass(C* buf, int g, int G, int N, int Ns, const C* __restrict__ tw) {
  constexpr int NB = E / R;
  const int NR = N / R;
  C v[E];
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = buf[padp(j + r * NR)];
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
    const int k = j & (Ns - 1);
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        C w = tw[r * Ns + k];
        if (S > 0) w.y = -w.y;
        v[q * R + r] = cmul(v[q * R + r], w);
      }
    }
    dftR<R, S>(&v[q * R]);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
    const int k = j & (Ns - 1);
    const int idx = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) buf[padp(idx + r * Ns)] = v[q * R + r];
  }
  __syncwarp();
}

// Full in-place transform of a line in `buf` (natural order in and out).
// All 32 lanes of the warp must call this (it uses __syncwarp).
template <int E, int S, typename C>
__device__ __forceinline__ void line_fft(C* buf, int g, int N, const C* __restrict__ tw) {
  const int G = N / E;
  int Ns = 1, off = 0;
  while (Ns < N) {
    const int R = (N / Ns) >= 16 ? 16 : N / Ns;
    switch (R) {
      case 16: stockham_pass<16, E, S>(buf, g, G, N, Ns, tw + off); break;
      case 8: stockham_pass<8, E, S>(buf, g, G, N, Ns, tw + off); break;
      case 4: stockham_pass<4, E, S>(buf, g, G, N, Ns, tw + off); break;
      default: stockham_pass<2, E, S>(buf, g, G, N, Ns, tw + off); break;
    }
    off += R * Ns;
    Ns *= R;
  }
}

// First pass (Ns = 1, radix 16) reading its inputs through a loader
// functor ld(position) instead of from `buf`; the result is written to `buf`
// in natural order.  The loader may read memory that overlaps `buf`: every
// lane loads before any lane stores.
template <int E, int S, typename C, typename Loader>
__device__ __forceinline__ void stockham_first16(C* buf, int g, int G, int N, Loader& ld) {
  constexpr int R = 16, NB = E / R;
  const int NR = N / R;
  C v[E];
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = ld(j + r * NR);
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < NB; ++q) dftR<R, S>(&v[q * R]);
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
#pragma unroll
    for (int r = 0; r < R; ++r) buf[padp(j * R + r)] = v[q * R + r];
  }
  __syncwarp();
}

template <int E, int S, typename C, typename Loader>
__device__ __forceinline__ void line_fft_ld(C* buf, int g, int N, const C* __restrict__ tw, Loader& ld) {
  const int G = N / E;
  stockham_first16<E, S>(buf, g, G, N, ld);
  int Ns = 16, off = 16;
  while (Ns < N) {
    const int R = (N / Ns) >= 16 ? 16 : N / Ns;
    switch (R) {
      case 16: stockham_pass<16, E, S>(buf, g, G, N, Ns, tw + off); break;
      case 8: stockham_pass<8, E, S>(buf, g, G, N, Ns, tw + off); break;
      case 4: stockham_pass<4, E, S>(buf, g, G, N, Ns, tw + off); break;
      default: stockham_pass<2, E, S>(buf, g, G, N, Ns, tw + off); break;
    }
    off += R * Ns;
    Ns *= R;
  }
}

// ---------------------------------------------------------------------------
// Passes with the line length N and the stride Ns known at compile time.
// For p = a + 16 m the padded index is padp(a) + 17 m, so an access pattern
// j + r*D with D a multiple of 16 needs one padded base per butterfly and
// constant offsets r*(D + D/16) instead of a shift and an add per access.
// ---------------------------------------------------------------------------
template <int D> __device__ __forceinline__ constexpr int pstride() { return D + D / 16; }

// padded index of j = g + G q
template <int G> __device__ __forceinline__ int padq(int g, int q) {
  if constexpr (G % 16 == 0) return padp(g) + q * pstride<G>();
  else return padp(g + G * q);
}

// position j + r*D, r = 0..R-1, of a line in `buf` (padded); pj = padp(j)
template <int R, int D, typename C>
__device__ __forceinline__ void load_r(const C* buf, int j, int pj, C* v) {
  if constexpr (D % 16 == 0) {
    const C* b = buf + pj;
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = b[r * pstride<D>()];
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = buf[padp(j + r * D)];
  }
}
template <int R, int D, typename C>
__device__ __forceinline__ void store_r(C* buf, int j, const C* v) {
  if constexpr (D % 16 == 0) {
    C* b = buf + padp(j);
#pragma unroll
    for (int r = 0; r < R; ++r) b[r * pstride<D>()] = v[r];
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r) buf[padp(j + r * D)] = v[r];
  }
}

// Twiddles of a pass from few table loads (FP32: the loads, not the
// arithmetic, are the scarce resource of the shared-memory-bound sweeps).
// Radix 16: w^r for r = 1..15 from the loaded w^1, w^2, w^4, w^8, each product
// at most three multiplications deep.
template <typename C>
__device__ __forceinline__ void powers16(const C* t, int Ns, C (&w)[16]) {
  w[1] = t[Ns]; w[2] = t[2 * Ns]; w[4] = t[4 * Ns]; w[8] = t[8 * Ns];
  w[3] = cmul(w[1], w[2]); w[5] = cmul(w[1], w[4]); w[6] = cmul(w[2], w[4]); w[7] = cmul(w[3], w[4]);
#pragma unroll
  for (int r = 9; r < 16; ++r) w[r] = cmul(w[r - 8], w[8]);
}
// exp(-2 pi i q/16) = (cos(pi q/8), -sin(pi q/8)), q = 0..7
__device__ __forceinline__ constexpr double w16c(int q) {
  return q == 0 ? 1.0 : q == 1 ? SDNS_C8 : q == 2 ? SDNS_R2 : q == 3 ? SDNS_S8 : q == 4 ? 0.0 : q == 5 ? -SDNS_S8
       : q == 6 ? -SDNS_R2 : -SDNS_C8;
}
__device__ __forceinline__ constexpr double w16s(int q) {
  return q == 0 ? 0.0 : q == 1 ? SDNS_S8 : q == 2 ? SDNS_R2 : q == 3 ? SDNS_C8 : q == 4 ? 1.0 : q == 5 ? SDNS_C8
       : q == 6 ? SDNS_R2 : SDNS_S8;
}

template <int R, int E, int S, int N, int Ns, typename C>
__device__ __forceinline__ void stockham_pass_c(C* buf, int g, const C* __restrict__ tw) {
  constexpr int G = N / E, NB = E / R, NR = N / R;
  C v[E];
#pragma unroll
  for (int q = 0; q < NB; ++q) load_r<R, NR>(buf, g + G * q, padq<G>(g, q), &v[q * R]);
  __syncwarp();
  constexpr bool f32 = sizeof(C) == 8;
  // last radix-2 pass of the compact sweeps: the twiddle of butterfly j = g + G q is
  // W_N^g * exp(-2 pi i q/16) (G = N/16): one load per lane
  constexpr bool tw_const = f32 && R == 2 && E == 16 && 2 * Ns == N && NB > 1;
  C w0 = mk<C>(0, 0);
  if constexpr (tw_const) w0 = tw[Ns + g];
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
    const int k = j & (Ns - 1);
    if constexpr (Ns > 1) {
      const C* t = tw + k;
      if constexpr (f32 && R == 16) {
        C w[16];
        powers16(t, Ns, w);
#pragma unroll
        for (int r = 1; r < R; ++r) v[q * R + r] = cmul(v[q * R + r], S > 0 ? cconj(w[r]) : w[r]);
      } else if constexpr (tw_const) {
        C w = mulc<-1>(w0, w16c(q), w16s(q));
        if (S > 0) w.y = -w.y;
        v[q * R + 1] = cmul(v[q * R + 1], w);
      } else {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          C w = t[r * Ns];
          if (S > 0) w.y = -w.y;
          v[q * R + r] = cmul(v[q * R + r], w);
        }
      }
    }
    dftR<R, S>(&v[q * R]);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
    const int k = j & (Ns - 1);
    store_r<R, Ns>(buf, (j - k) * R + k, &v[q * R]);
  }
  __syncwarp();
}

template <int R, int E, int S, int N, int Ns, typename C>
__device__ __forceinline__ void last_pass_regs_c(const C* buf, int g, const C* __restrict__ tw, C (&x)[E]) {
  constexpr int G = N / E, NB = E / R, NR = N / R;
  C v[E];
#pragma unroll
  for (int q = 0; q < NB; ++q) load_r<R, NR>(buf, g + G * q, padq<G>(g, q), &v[q * R]);
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const C* t = tw + (g + G * q);  // j < Ns in the last pass, so (j mod Ns) = j
#pragma unroll
    for (int r = 1; r < R; ++r) {
      C w = t[r * Ns];
      if (S > 0) w.y = -w.y;
      v[q * R + r] = cmul(v[q * R + r], w);
    }
    dftR<R, S>(&v[q * R]);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r) x[q + r * NB] = v[q * R + r];
}

// Pruned inverse transforms: with the 2/3 rule the kept input positions are
// p <= kc and p >= N - kc, and kc < 6N/16, so the first pass's inputs
// j + r*N/16 with r = 6..9 are zero for every j.  PR = true skips them (the
// radix-16 butterfly then folds the zeros away).
__host__ __device__ constexpr bool prunable(int n, int kc) { return kc >= 0 && kc < 6 * (n / 16); }
__host__ __device__ constexpr bool pruned_r(int r) { return r >= 6 && r <= 9; }

// first radix-16 pass fed by a loader; result written in natural order
template <int E, int S, int N, bool PR = false, typename C, typename Loader>
__device__ __forceinline__ void first16_c(C* buf, int g, Loader& ld) {
  constexpr int R = 16, NB = E / R, NR = N / R, G = N / E;
  C v[E];
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = (PR && pruned_r(r)) ? mk<C>(0, 0) : ld(j + r * NR);
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < NB; ++q) dftR<R, S>(&v[q * R]);
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    C* b = buf + 17 * (g + G * q);  // padp(16 j + r) = 17 j + r for r < 16
#pragma unroll
    for (int r = 0; r < R; ++r) b[r] = v[q * R + r];
  }
  __syncwarp();
}

// first radix-16 pass reading the line from `buf` itself (in place)
template <int E, int S, int N, bool PR = false, typename C>
__device__ __forceinline__ void first16_buf(C* buf, int g) {
  constexpr int R = 16, NB = E / R, NR = N / R, G = N / E;
  C v[E];
  if constexpr (PR && NR % 16 == 0) {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const C* b = buf + padq<G>(g, q);
#pragma unroll
      for (int r = 0; r < R; ++r) v[q * R + r] = pruned_r(r) ? mk<C>(0, 0) : b[r * pstride<NR>()];
    }
  } else if constexpr (PR) {
#pragma unroll
    for (int q = 0; q < NB; ++q)
#pragma unroll
      for (int r = 0; r < R; ++r) v[q * R + r] = pruned_r(r) ? mk<C>(0, 0) : buf[padp(g + G * q + r * NR)];
  } else {
#pragma unroll
    for (int q = 0; q < NB; ++q) load_r<R, NR>(buf, g + G * q, padq<G>(g, q), &v[q * R]);
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < NB; ++q) dftR<R, S>(&v[q * R]);
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    C* b = buf + 17 * (g + G * q);
#pragma unroll
    for (int r = 0; r < R; ++r) b[r] = v[q * R + r];
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Two-pass transforms of N = 512 (32 x 16) and N = 1024 (32 x 32) lines with
// E = 32 values per lane (G = N/32 lanes per line): a radix-32 first pass and
// a radix-N/32 last pass.  One shared-memory round trip fewer than 16,16,2 /
// 16,16,4, so fewer shared-memory instructions and a shorter dependency chain.
// The last pass reads its twiddles W_N^{r k} from the full table `twf`
// (FP32: the powers of k from log2(R) loads; FP64: one load each).
// ---------------------------------------------------------------------------
template <int N, int S, bool PR, typename C>
__device__ __forceinline__ void first32_buf(C* buf, int g) {
  constexpr int NR = N / 32;  // 16 or 32: a multiple of 16
  static_assert(NR % 16 == 0, "radix-32 first pass for N = 512, 1024");
  C v[32];
  const C* b = buf + padp(g);
#pragma unroll
  for (int r = 0; r < 32; ++r) v[r] = (PR && r >= 12 && r <= 19) ? mk<C>(0, 0) : b[r * pstride<NR>()];
  __syncwarp();
  dft32<S>(v);
  C* o = buf + 34 * g;  // padp(32 g + r) = 34 g + r + r/16
#pragma unroll
  for (int r = 0; r < 32; ++r) o[r + (r >> 4)] = v[r];
  __syncwarp();
}

template <int N, int S, typename C>
__device__ __forceinline__ void last32_buf(C* buf, int g, const C* __restrict__ twf) {
  constexpr int R = N / 32, E = 32, NB = E / R, NR = N / R, G = N / 32, Ns = 32;
  C v[E];
#pragma unroll
  for (int q = 0; q < NB; ++q) load_r<R, NR>(buf, g + G * q, padq<G>(g, q), &v[q * R]);
  __syncwarp();
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int k = (g + G * q) & (Ns - 1);
    C w[R];
    if constexpr (sizeof(C) == 8) {
#pragma unroll
      for (int b = 1; b < R; b <<= 1) w[b] = twf[k * b];
#pragma unroll
      for (int r = 3; r < R; ++r) {
        if ((r & (r - 1)) == 0) continue;
        int hb = 1;
        while (hb * 2 <= r) hb *= 2;
        w[r] = cmul(w[r - hb], w[hb]);
      }
    } else {
#pragma unroll
      for (int r = 1; r < R; ++r) w[r] = twf[k * r];
    }
#pragma unroll
    for (int r = 1; r < R; ++r) v[q * R + r] = cmul(v[q * R + r], S > 0 ? cconj(w[r]) : w[r]);
    dftR<R, S>(&v[q * R]);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;  // j < Ns: the output block starts at j
    store_r<R, Ns>(buf, j, &v[q * R]);
  }
  __syncwarp();
}

template <int N, int S, bool PR, typename C>
__device__ __forceinline__ void line_fft_r32(C* buf, int g, const C* __restrict__ tw) {
  first32_buf<N, S, PR>(buf, g);
  last32_buf<N, S>(buf, g, tw + tw_len(N));
}

// Same transform with the line length N fixed at compile time: the pass
// sequence, the strides and the twiddle offsets are constants, so the index
// arithmetic of every pass folds into immediate offsets.
template <int N, int E, int S, int Ns, typename C>
__device__ __forceinline__ void passes_t(C* buf, int g, const C* __restrict__ tw, int off) {
  if constexpr (Ns < N) {
    constexpr int R = (N / Ns) >= 16 ? 16 : N / Ns;
    stockham_pass_c<R, E, S, N, Ns>(buf, g, tw + off);
    passes_t<N, E, S, Ns * R>(buf, g, tw, off + R * Ns);
  }
}
template <int N, int E, int S, bool PR = false, typename C, typename Loader>
__device__ __forceinline__ void line_fft_ld_t(C* buf, int g, const C* __restrict__ tw, Loader& ld) {
  first16_c<E, S, N, PR>(buf, g, ld);
  passes_t<N, E, S, 16>(buf, g, tw, 16);
}
// in-place transform of a line held in natural order in `buf`
template <int N, int E, int S, bool PR = false, typename C>
__device__ __forceinline__ void line_fft_t(C* buf, int g, const C* __restrict__ tw) {
  first16_buf<E, S, N, PR>(buf, g);
  passes_t<N, E, S, 16>(buf, g, tw, 16);
}

// ---------------------------------------------------------------------------
// Register-resident ends of a line transform.  After the last Stockham pass
// the lane g of a group holds the outputs of positions g + G*m, m = 0..E-1,
// in x[m]; the first radix-16 pass reads exactly the same positions.  A
// transform can therefore start from, or end in, registers, and pointwise
// work between an inverse and a forward transform needs no shared memory.
// ---------------------------------------------------------------------------
template <int R, int E, int S, typename C>
__device__ __forceinline__ void last_pass_regs(const C* buf, int g, int G, int N, int Ns, const C* __restrict__ tw,
                                               C (&x)[E]) {
  constexpr int NB = E / R;
  const int NR = N / R;
  C v[E];
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = buf[padp(j + r * NR)];
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;  // j < Ns in the last pass, so (j mod Ns) = j
#pragma unroll
    for (int r = 1; r < R; ++r) {
      C w = tw[r * Ns + j];
      if (S > 0) w.y = -w.y;
      v[q * R + r] = cmul(v[q * R + r], w);
    }
    dftR<R, S>(&v[q * R]);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r) x[q + r * NB] = v[q * R + r];
}

// passes 2.. of a transform whose first pass has been written to `buf`;
// the result ends in registers x[m] (position g + G*m)
template <int E, int S, typename C>
__device__ __forceinline__ void fft_tail_regs(C* buf, int g, int G, int N, const C* __restrict__ tw, C (&x)[E]) {
  int Ns = 16, off = 16;
  while (Ns * 16 < N) {
    stockham_pass<16, E, S>(buf, g, G, N, Ns, tw + off);
    off += 16 * Ns;
    Ns *= 16;
  }
  switch (N / Ns) {
    case 16: last_pass_regs<16, E, S>(buf, g, G, N, Ns, tw + off, x); break;
    case 8: last_pass_regs<8, E, S>(buf, g, G, N, Ns, tw + off, x); break;
    case 4: last_pass_regs<4, E, S>(buf, g, G, N, Ns, tw + off, x); break;
    default: last_pass_regs<2, E, S>(buf, g, G, N, Ns, tw + off, x); break;
  }
}

// transform with a loader-fed first pass, ending in registers (E == 16 when N == 16)
template <int E, int S, typename C, typename Loader>
__device__ __forceinline__ void fft_ld_regs(C* buf, int g, int N, const C* __restrict__ tw, Loader& ld, C (&x)[E]) {
  const int G = N / E;
  if (N == 16) {
#pragma unroll
    for (int r = 0; r < 16; ++r) x[r] = ld(r);
    dft16<S>(x);
    return;
  }
  stockham_first16<E, S>(buf, g, G, N, ld);
  fft_tail_regs<E, S>(buf, g, G, N, tw, x);
}

// transform starting from registers x[m] (position g + G*m), ending in y[m]
template <int E, int S, typename C>
__device__ __forceinline__ void fft_regs_regs(C* buf, int g, int N, const C* __restrict__ tw, const C (&x)[E],
                                              C (&y)[E]) {
  const int G = N / E;
  constexpr int NB = E / 16;
  C v[E];
#pragma unroll
  for (int q = 0; q < NB; ++q)
#pragma unroll
    for (int r = 0; r < 16; ++r) v[q * 16 + r] = x[q + r * NB];
#pragma unroll
  for (int q = 0; q < NB; ++q) dft16<S>(&v[q * 16]);
  if (N == 16) {
#pragma unroll
    for (int r = 0; r < E; ++r) y[r] = v[r];
    return;
  }
  __syncwarp();  // earlier readers of buf are done
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
#pragma unroll
    for (int r = 0; r < 16; ++r) buf[padp(j * 16 + r)] = v[q * 16 + r];
  }
  __syncwarp();
  fft_tail_regs<E, S>(buf, g, G, N, tw, y);
}

// ---------------------------------------------------------------------------
// Forward transform of a line of compile-time length N (16..512, E = 16)
// held in registers: x[m] is position g + G*m on entry and holds the output
// of position g + G*m on exit.  The pass structure is fixed at compile time,
// so one instance is small enough to stay resident in the instruction cache
// when it is reused for several transforms (inverse transforms use
// conj(fwd(conj(.)))).
// ---------------------------------------------------------------------------
template <int N, int Ns, typename C>
__device__ __forceinline__ void fwd_passes_const(C* buf, int g, const C* __restrict__ tw, int off, C (&x)[16]) {
  constexpr int G = N / 16;
  constexpr int R = (N / Ns) >= 16 ? 16 : N / Ns;
  if constexpr (Ns * R == N) {
    last_pass_regs_c<R, 16, -1, N, Ns>(buf, g, tw + off, x);
  } else {
    stockham_pass_c<R, 16, -1, N, Ns>(buf, g, tw + off);
    fwd_passes_const<N, Ns * R>(buf, g, tw, off + R * Ns, x);
  }
}

template <int N, typename C>
__device__ __forceinline__ void fwd_line_regs(C* buf, int g, const C* __restrict__ tw, C (&x)[16]) {
  dft16<-1>(x);
  if constexpr (N > 16) {
    __syncwarp();  // earlier readers of buf are done
    C* b = buf + 17 * g;  // padp(16 g + r) = 17 g + r
#pragma unroll
    for (int r = 0; r < 16; ++r) b[r] = x[r];
    __syncwarp();
    fwd_passes_const<N, 16>(buf, g, tw, 16, x);
  }
}

// ---------------------------------------------------------------------------
// L independent lines transformed together (line l in buf + l*ldb): every
// pass loads all L lines, applies each twiddle factor to all of them and
// stores all of them, so the L dependency chains interleave and one twiddle
// load serves L lines.  Forward sign; x[l][m] is position g + G*m.
// ---------------------------------------------------------------------------
template <int R, int N, int Ns, int L, typename C>
__device__ __forceinline__ void stockham_pass_fL(C* buf, int ldb, int g, const C* __restrict__ tw) {
  constexpr int E = 16, G = N / E, NB = E / R, NR = N / R;
  C v[L][E];
#pragma unroll
  for (int q = 0; q < NB; ++q)
#pragma unroll
    for (int l = 0; l < L; ++l) load_r<R, NR>(buf + l * ldb, g + G * q, padq<G>(g, q), &v[l][q * R]);
  __syncwarp();
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
    const int k = j & (Ns - 1);
    const C* t = tw + k;
#pragma unroll
    for (int r = 1; r < R; ++r) {
      const C w = t[r * Ns];
#pragma unroll
      for (int l = 0; l < L; ++l) v[l][q * R + r] = cmul(v[l][q * R + r], w);
    }
#pragma unroll
    for (int l = 0; l < L; ++l) dftR<R, -1>(&v[l][q * R]);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = g + G * q;
    const int k = j & (Ns - 1);
#pragma unroll
    for (int l = 0; l < L; ++l) store_r<R, Ns>(buf + l * ldb, (j - k) * R + k, &v[l][q * R]);
  }
  __syncwarp();
}

template <int R, int N, int Ns, int L, typename C>
__device__ __forceinline__ void last_pass_fL(const C* buf, int ldb, int g, const C* __restrict__ tw, C (&x)[L][16]) {
  constexpr int E = 16, G = N / E, NB = E / R, NR = N / R;
  C v[L][E];
#pragma unroll
  for (int q = 0; q < NB; ++q)
#pragma unroll
    for (int l = 0; l < L; ++l) load_r<R, NR>(buf + l * ldb, g + G * q, padq<G>(g, q), &v[l][q * R]);
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const C* t = tw + (g + G * q);  // j < Ns in the last pass
#pragma unroll
    for (int r = 1; r < R; ++r) {
      const C w = t[r * Ns];
#pragma unroll
      for (int l = 0; l < L; ++l) v[l][q * R + r] = cmul(v[l][q * R + r], w);
    }
#pragma unroll
    for (int l = 0; l < L; ++l) dftR<R, -1>(&v[l][q * R]);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int l = 0; l < L; ++l) x[l][q + r * NB] = v[l][q * R + r];
}

template <int N, int Ns, int L, typename C>
__device__ __forceinline__ void fwd_passes_L(C* buf, int ldb, int g, const C* __restrict__ tw, int off,
                                             C (&x)[L][16]) {
  constexpr int R = (N / Ns) >= 16 ? 16 : N / Ns;
  if constexpr (Ns * R == N) {
    last_pass_fL<R, N, Ns, L>(buf, ldb, g, tw + off, x);
  } else {
    stockham_pass_fL<R, N, Ns, L>(buf, ldb, g, tw + off);
    fwd_passes_L<N, Ns * R, L>(buf, ldb, g, tw, off + R * Ns, x);
  }
}

// forward transforms of L lines of compile-time length N (16..512) held in
// registers (x[l][m] = position g + G*m in and out); buf holds L lines of ldb
template <int N, int L, typename C>
__device__ __forceinline__ void fwd_lines_regs(C* buf, int ldb, int g, const C* __restrict__ tw, C (&x)[L][16]) {
#pragma unroll
  for (int l = 0; l < L; ++l) dft16<-1>(x[l]);
  if constexpr (N > 16) {
    __syncwarp();  // earlier readers of buf are done
#pragma unroll
    for (int l = 0; l < L; ++l) {
      C* b = buf + l * ldb + 17 * g;  // padp(16 g + r) = 17 g + r
#pragma unroll
      for (int r = 0; r < 16; ++r) b[r] = x[l][r];
    }
    __syncwarp();
    fwd_passes_L<N, 16, L>(buf, ldb, g, tw, 16, x);
  }
}

// Ampere-style asynchronous global->shared copies (LDGSTS); the data does not
// pass through registers, so a whole tile can be in flight per thread block.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
template <int BYTES> __device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  if constexpr (BYTES == 16) cp_async16(smem, gmem);
  else cp_async8(smem, gmem);
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

}  // namespace sdns
