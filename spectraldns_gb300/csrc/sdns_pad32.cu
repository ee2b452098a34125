// 3/2-rule (padded) right-hand side of the pseudo-spectral Navier-Stokes
// solver: spectralDNS/solvers/NS.py:29-31 with padding_factor = 1.5, and the
// velocity-vorticity form of spectralDNS/solvers/VV.py on the same transforms.
//
// The N modes of each axis (Nyquist excluded) are placed in a spectral array
// of M = 3N/2 points per axis, transformed to the padded physical grid, the
// cross product u x w is formed there, transformed back and truncated to the
// N modes, so the quadratic term carries no aliasing error.  The transform
// lengths 3 * 2^k are handled by a generic mixed-radix (4, 2, 3) Stockham
// line FFT on shared-memory tiles (radix-2^k sweeps of the 2/3-rule path do
// not cover them).  This path is for the 3/2-rule contexts; the fused
// 2/3-rule sweeps remain the fast path.
#include <cuda_runtime.h>

#include <type_traits>

#include "sdns_fft.cuh"
#include "sdns_internal.h"

namespace sdns {
namespace {

template <typename C> __device__ __forceinline__ C cz() { return mk<C>(0, 0); }
// multiply by +i (s > 0) or -i (s < 0)
template <typename C> __device__ __forceinline__ C mul_i(C a, int s) { return s > 0 ? mk<C>(-a.y, a.x) : mk<C>(a.y, -a.x); }

template <typename C>
__device__ __forceinline__ void dft_small(C* v, int r, int s) {
  using Real = decltype(C::x);
  if (r == 2) {
    const C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if (r == 4) {
    const C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    const C c = cadd(v[1], v[3]), d = mul_i(csub(v[1], v[3]), s);
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, d);
    v[3] = csub(b, d);
  } else {  // r == 3: X1,2 = x0 - (x1+x2)/2 +- s i sqrt(3)/2 (x1 - x2)
    const Real h = (Real)0.86602540378443864676;
    const C sum = cadd(v[1], v[2]);
    const C t = mk<C>(v[0].x - (Real)0.5 * sum.x, v[0].y - (Real)0.5 * sum.y);
    const C d = mul_i(mk<C>(h * (v[1].x - v[2].x), h * (v[1].y - v[2].y)), s);
    v[0] = cadd(v[0], sum);
    v[1] = cadd(t, d);
    v[2] = csub(t, d);
  }
}

// Stockham autosort FFT (Govindaraju et al., SC'08) of W lines of length N
// (pitch N + 1) held in shared memory, ping-ponging between a and b; returns
// the buffer holding the result.  The radix sequence (4s, then a 2, then a 3)
// and every stride are compile-time constants.  tw[j] = exp(-2 pi i j / N)
// (FP64, rounded); s = -1 forward, +1 inverse (unnormalised).
template <int N, int NS> struct pass_radix {
  static constexpr int rem = N / NS;
  static constexpr int value = rem % 4 == 0 ? 4 : (rem % 2 == 0 ? 2 : 3);
};

template <typename C, int N, int NS>
__device__ __forceinline__ C* fft_passes(C* in, C* out, int W, int s, const C* __restrict__ tw) {
  if constexpr (NS >= N) {
    return in;
  } else {
    constexpr int R = pass_radix<N, NS>::value, NB = N / R, TS = N / (NS * R), LD = N + 1;
    for (int t = threadIdx.x; t < W * NB; t += blockDim.x) {
      const int w = t / NB, j = t - w * NB;
      const int k = j % NS;
      const C* x = in + w * LD;
      C* y = out + w * LD;
      C v[4];
#pragma unroll
      for (int m = 0; m < R; ++m) v[m] = x[j + m * NB];
#pragma unroll
      for (int m = 1; m < R; ++m) {
        C wv = tw[TS * k * m];
        if (s > 0) wv.y = -wv.y;
        v[m] = cmul(v[m], wv);
      }
      dft_small(v, R, s);
      const int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int m = 0; m < R; ++m) y[base + m * NS] = v[m];
    }
    __syncthreads();
    return fft_passes<C, N, NS * R>(out, in, W, s, tw);
  }
}

template <typename C, int N>
__device__ __forceinline__ C* smem_fft(C* a, C* b, int W, int s, const C* __restrict__ tw) {
  return fft_passes<C, N, 1>(a, b, W, s, tw);
}

// Is line l of a padded axis sweep one that can hold nonzero data?  Lines are
// (a, kz) with a = l / ld2 and kz = l % ld2: kz must be below kzmax and, when
// na > 0, a must be one of the N-grid wave numbers of an axis of length ma
// (a < na/2 or a > ma - na/2).  Lines that cannot are all zero on input (the
// inverse sweeps) or never read (the forward sweeps) and are skipped.
__device__ __forceinline__ bool line_live(long long l, const Pad32Axis& ax) {
  if (ax.ld2 <= 0) return true;
  const long long a = l / ax.ld2;
  const int kz = (int)(l - a * ax.ld2);
  if (kz >= ax.kzmax) return false;
  return ax.na <= 0 || 2 * a < ax.na || 2 * (ax.ma - a) < ax.na;
}

// C2C along a strided axis, in place: line l of field f starts at
// f*fs + (l / B)*ss + (l % B), position p adds p*rs.  A block transforms W
// adjacent lines (coalesced rows of W values); tiles without a live line return.
template <typename C, int N>
__global__ void __launch_bounds__(256) k_fft_axis(C* data, Pad32Axis ax, int s, double scale, const C* tw) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int n = N, ld = N + 1;
  const int W = ax.W;
  C* a = reinterpret_cast<C*>(smraw);
  C* b = a + (size_t)W * ld;
  const long long l0 = (long long)blockIdx.x * W;
  const long long nl = ax.nlines;
  {
    bool any = false;
    for (int w = 0; w < W; ++w)
      if (l0 + w < nl && line_live(l0 + w, ax)) { any = true; break; }
    if (!any) return;
  }
  // every row of the tile is in flight at once (cp.async), then one wait
  for (int idx = threadIdx.x; idx < W * n; idx += blockDim.x) {
    const int w = idx % W, p = idx / W;
    const long long l = l0 + w;
    if (l < nl) {
      const long long f = blockIdx.y;
      const long long o = f * ax.fs + (l / ax.B) * ax.ss + (l % ax.B) + (long long)p * ax.rs;
      cp_async<sizeof(C)>(&a[w * ld + p], &data[o]);
    } else {
      a[w * ld + p] = cz<C>();
    }
  }
  cp_commit();
  cp_wait_all();
  __syncthreads();
  const C* res = smem_fft<C, N>(a, b, W, s, tw);
  using Real = decltype(C::x);
  const Real sc = (Real)scale;
  for (int idx = threadIdx.x; idx < W * n; idx += blockDim.x) {
    const int w = idx % W, p = idx / W;
    const long long l = l0 + w;
    if (l < nl) {
      const long long f = blockIdx.y;
      const long long o = f * ax.fs + (l / ax.B) * ax.ss + (l % ax.B) + (long long)p * ax.rs;
      const C v = res[w * ld + p];
      data[o] = mk<C>(v.x * sc, v.y * sc);
    }
  }
}

// C2R (dir > 0) or R2C (dir < 0) along the contiguous last axis.  Spectral
// lines have nh = n/2 + 1 values (pitch nh), physical lines n values.  C2R
// drops the imaginary parts of the k = 0 and k = n/2 coefficients.
template <typename C, int N>
__global__ void __launch_bounds__(256) k_fft_z(C* spec, void* physv, long long nlines, int W, int dir, double scale,
                                               const C* tw) {
  using Real = decltype(C::x);
  Real* phys = reinterpret_cast<Real*>(physv);
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int n = N, nh = N / 2 + 1, ld = N + 1;
  C* a = reinterpret_cast<C*>(smraw);
  C* b = a + (size_t)W * ld;
  const long long l0 = (long long)blockIdx.x * W;
  if (dir > 0) {
    // stage the half spectra (cp.async, all in flight), then form the Hermitian lines
    for (int idx = threadIdx.x; idx < W * nh; idx += blockDim.x) {
      const int w = idx / nh, k = idx - w * nh;
      const long long l = l0 + w;
      if (l < nlines) cp_async<sizeof(C)>(&a[w * ld + k], &spec[l * nh + k]);
      else a[w * ld + k] = cz<C>();
    }
    cp_commit();
    cp_wait_all();
    __syncthreads();
    for (int idx = threadIdx.x; idx < W * nh; idx += blockDim.x) {
      const int w = idx / nh, k = idx - w * nh;
      C v = a[w * ld + k];
      if (k == 0 || 2 * k == n) {
        v.y = 0;
        a[w * ld + k] = v;
      } else {
        a[w * ld + n - k] = mk<C>(v.x, -v.y);
      }
    }
  } else {
    // real lines: eight independent loads per thread before the shared-memory stores
    constexpr int U = 8;
    for (int base = threadIdx.x; base < W * n; base += U * blockDim.x) {
      Real r[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int idx = base + u * blockDim.x;
        const int w = idx / n;
        r[u] = (idx < W * n && l0 + w < nlines) ? phys[(l0 + w) * n + (idx - w * n)] : (Real)0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int idx = base + u * blockDim.x;
        if (idx < W * n) {
          const int w = idx / n;
          a[w * ld + idx - w * n] = mk<C>(r[u], (Real)0);
        }
      }
    }
  }
  __syncthreads();
  const C* res = smem_fft<C, N>(a, b, W, dir > 0 ? 1 : -1, tw);
  const Real sc = (Real)scale;
  if (dir > 0) {
    for (int idx = threadIdx.x; idx < W * n; idx += blockDim.x) {
      const int w = idx / n, j = idx - w * n;
      const long long l = l0 + w;
      if (l < nlines) phys[l * n + j] = res[w * ld + j].x * sc;
    }
  } else {
    for (int idx = threadIdx.x; idx < W * nh; idx += blockDim.x) {
      const int w = idx / nh, k = idx - w * nh;
      const long long l = l0 + w;
      if (l < nlines) {
        const C v = res[w * ld + k];
        spec[l * nh + k] = mk<C>(v.x * sc, v.y * sc);
      }
    }
  }
}

__device__ __forceinline__ int wave_of(int p, int n) { return p < (n + 1) / 2 ? p : p - n; }

// caller-layout vector (3, N0, N1, N2/2+1) -> the six padded spectral fields
// [6][M0][M1][M2/2+1]: NS u_hat and i K x u_hat; VV i K x w_hat / K^2 and
// w_hat.  Modes outside the N-mode box and the Nyquist modes are zero.
template <typename C>
__global__ void k_pad_fields(const C* u, C* spec, Pad32 p) {
  using Real = decltype(C::x);
  const int M0 = p.M[0], M1 = p.M[1], M2h = p.M[2] / 2 + 1, N2h = p.N[2] / 2 + 1;
  const long long n1 = (long long)M0 * M1 * M2h;
  const long long f1 = (long long)p.N[0] * p.N[1] * N2h;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n1; i += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(i % M2h);
    const int p1 = (int)((i / M2h) % M1), p0 = (int)(i / ((long long)M2h * M1));
    const int k0 = wave_of(p0, M0), k1 = wave_of(p1, M1);
    const bool in = 2 * k0 < p.N[0] && 2 * k0 > -p.N[0] && 2 * k1 < p.N[1] && 2 * k1 > -p.N[1] && 2 * kz < p.N[2];
    C o[6];
    for (int q = 0; q < 6; ++q) o[q] = cz<C>();
    if (in) {
      const int n0 = k0 >= 0 ? k0 : p.N[0] + k0, n1i = k1 >= 0 ? k1 : p.N[1] + k1;
      const long long s = ((long long)n0 * p.N[1] + n1i) * N2h + kz;
      const C a = u[s], b = u[f1 + s], c = u[2 * f1 + s];
      const double K0 = p.ks[0] * k0, K1 = p.ks[1] * k1, K2 = p.ks[2] * kz;
      const double q2 = K0 * K0 + K1 * K1 + K2 * K2;
      const double sc = p.vv ? (q2 > 0.0 ? 1.0 / q2 : 0.0) : 1.0;
      // i K x v (scaled by sc)
      const double xr = sc * (K1 * c.x - K2 * b.x), xi = sc * (K1 * c.y - K2 * b.y);
      const double yr = sc * (K2 * a.x - K0 * c.x), yi = sc * (K2 * a.y - K0 * c.y);
      const double zr = sc * (K0 * b.x - K1 * a.x), zi = sc * (K0 * b.y - K1 * a.y);
      const C cx = mk<C>((Real)(-xi), (Real)xr), cy = mk<C>((Real)(-yi), (Real)yr), cw = mk<C>((Real)(-zi), (Real)zr);
      if (p.vv) {
        o[0] = cx; o[1] = cy; o[2] = cw; o[3] = a; o[4] = b; o[5] = c;
      } else {
        o[0] = a; o[1] = b; o[2] = c; o[3] = cx; o[4] = cy; o[5] = cw;
      }
    }
    for (int q = 0; q < 6; ++q) spec[q * n1 + i] = o[q];
  }
}

// u x w on the padded physical grid: fields 0..2 <- (0..2) x (3..5)
template <typename Real>
__global__ void k_cross6(Real* ph, long long np) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < np; i += (long long)gridDim.x * blockDim.x) {
    const Real u0 = ph[i], u1 = ph[np + i], u2 = ph[2 * np + i];
    const Real w0 = ph[3 * np + i], w1 = ph[4 * np + i], w2 = ph[5 * np + i];
    ph[i] = u1 * w2 - u2 * w1;
    ph[np + i] = u2 * w0 - u0 * w2;
    ph[2 * np + i] = u0 * w1 - u1 * w0;
  }
}

// truncate the padded nonlinear term to the N modes (Nyquist masked,
// NS.py:253-254) and assemble the right-hand side: NS projection and diffusion
// (NS.py:203-217), VV curl and diffusion (VV.py:103-110), plus Source
template <typename C>
__global__ void k_rhs32(const C* spec, const C* u, const C* src, C* rhs, C* phat, Pad32 p) {
  using Real = decltype(C::x);
  const int M0 = p.M[0], M1 = p.M[1], M2h = p.M[2] / 2 + 1, N2h = p.N[2] / 2 + 1;
  const long long nm = (long long)M0 * M1 * M2h;
  const long long f1 = (long long)p.N[0] * p.N[1] * N2h;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < f1; i += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(i % N2h);
    const int n1 = (int)((i / N2h) % p.N[1]), n0 = (int)(i / ((long long)N2h * p.N[1]));
    const int k0 = wave_of(n0, p.N[0]), k1 = wave_of(n1, p.N[1]);
    const bool nyq = 2 * n0 == p.N[0] || 2 * n1 == p.N[1] || 2 * kz == p.N[2];
    double nr[3] = {0, 0, 0}, ni[3] = {0, 0, 0};
    if (!nyq) {
      const long long q = ((long long)(k0 >= 0 ? k0 : M0 + k0) * M1 + (k1 >= 0 ? k1 : M1 + k1)) * M2h + kz;
      for (int c = 0; c < 3; ++c) {
        const C v = spec[c * nm + q];
        nr[c] = v.x;
        ni[c] = v.y;
      }
    }
    const double K[3] = {p.ks[0] * k0, p.ks[1] * k1, p.ks[2] * kz};
    const double q2 = K[0] * K[0] + K[1] * K[1] + K[2] * K[2];
    const double nuK2 = p.nu * q2;
    double cr[3], ci[3];
    if (p.vv) {
      for (int c = 0; c < 3; ++c) {
        const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
        cr[c] = -(K[c1] * ni[c2] - K[c2] * ni[c1]);
        ci[c] = K[c1] * nr[c2] - K[c2] * nr[c1];
      }
    } else {
      const double iq = q2 > 0.0 ? 1.0 / q2 : 0.0;
      const double Pr = (nr[0] * K[0] + nr[1] * K[1] + nr[2] * K[2]) * iq;
      const double Pi = (ni[0] * K[0] + ni[1] * K[1] + ni[2] * K[2]) * iq;
      if (phat) phat[i] = mk<C>((Real)Pr, (Real)Pi);
      for (int c = 0; c < 3; ++c) {
        cr[c] = nr[c] - Pr * K[c];
        ci[c] = ni[c] - Pi * K[c];
      }
    }
    for (int c = 0; c < 3; ++c) {
      const C uv = u[c * f1 + i];
      double xr = cr[c] - nuK2 * uv.x, xi = ci[c] - nuK2 * uv.y;
      if (src) {
        const C sv = src[c * f1 + i];
        xr += sv.x;
        xi += sv.y;
      }
      rhs[c * f1 + i] = mk<C>((Real)xr, (Real)xi);
    }
  }
}

inline unsigned grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 16) b = 152LL * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

// lines per tile of length n (two ping-pong buffers of pitch n + 1 in shared memory)
inline int tile_lines(int n, size_t csz) {
  int W = 16;
  while (W > 1 && (size_t)2 * W * (n + 1) * csz > 200 * 1024) W >>= 1;
  return W;
}

// launch a kernel instance templated on the padded length M in {24, ..., 1536}
template <typename F> int by_length(int n, F&& f) {
  switch (n) {
    case 24: return f(std::integral_constant<int, 24>());
    case 48: return f(std::integral_constant<int, 48>());
    case 96: return f(std::integral_constant<int, 96>());
    case 192: return f(std::integral_constant<int, 192>());
    case 384: return f(std::integral_constant<int, 384>());
    case 768: return f(std::integral_constant<int, 768>());
    case 1536: return f(std::integral_constant<int, 1536>());
    default: return (int)cudaErrorInvalidValue;
  }
}

template <typename C> int rhs_t(const Pad32& p, const void* u_hat, const void* src, void* rhs, void* phat,
                                cudaStream_t s) {
  using Real = decltype(C::x);
  const int M0 = p.M[0], M1 = p.M[1], M2 = p.M[2], M2h = M2 / 2 + 1;
  const long long nm = (long long)M0 * M1 * M2h, np = (long long)M0 * M1 * M2;
  C* spec = reinterpret_cast<C*>(p.spec);
  Real* ph = reinterpret_cast<Real*>(p.phys);
  const C* tw0 = reinterpret_cast<const C*>(p.tw[0]);
  const C* tw1 = reinterpret_cast<const C*>(p.tw[1]);
  const C* tw2 = reinterpret_cast<const C*>(p.tw[2]);
  k_pad_fields<C><<<grid_for(nm), 256, 0, s>>>(reinterpret_cast<const C*>(u_hat), spec, p);
  int err = 0;
  // lines (a, kz) of the x sweeps: a = k1 position; of the y sweeps: a = k0 position (any)
  auto axis = [&](int n, long long nlines, long long B, long long fs, long long ss, long long rs, int nf, int sign,
                  double scale, const C* tw, int na, int ma) {
    Pad32Axis ax;
    ax.n = n; ax.nlines = nlines; ax.B = B; ax.fs = fs; ax.ss = ss; ax.rs = rs;
    ax.ld2 = M2h; ax.kzmax = p.N[2] / 2; ax.na = na; ax.ma = ma;
    ax.W = tile_lines(n, sizeof(C));
    const size_t sm = (size_t)2 * ax.W * (n + 1) * sizeof(C);
    const dim3 grid((unsigned)((nlines + ax.W - 1) / ax.W), (unsigned)nf);
    const int e = by_length(n, [&](auto L) {
      k_fft_axis<C, decltype(L)::value><<<grid, 256, sm, s>>>(spec, ax, sign, scale, tw);
      return (int)cudaGetLastError();
    });
    if (e && !err) err = e;
  };
  auto zpass = [&](int nf, int dir) {
    const int W = tile_lines(M2, sizeof(C));
    const size_t sm = (size_t)2 * W * (M2 + 1) * sizeof(C);
    const long long nl = (long long)nf * M0 * M1;
    const int e = by_length(M2, [&](auto L) {
      k_fft_z<C, decltype(L)::value><<<(unsigned)((nl + W - 1) / W), 256, sm, s>>>(spec, ph, nl, W, dir, 1.0, tw2);
      return (int)cudaGetLastError();
    });
    if (e && !err) err = e;
  };
  // inverse: x (lines M1*M2h, rows stride M1*M2h), y (lines M0*M2h in runs of M2h), z C2R
  axis(M0, (long long)M1 * M2h, (long long)M1 * M2h, nm, 0, (long long)M1 * M2h, 6, +1, 1.0, tw0, p.N[1], M1);
  axis(M1, (long long)M0 * M2h, M2h, nm, (long long)M1 * M2h, M2h, 6, +1, 1.0, tw1, 0, M0);
  zpass(6, +1);
  k_cross6<Real><<<grid_for(np), 256, 0, s>>>(ph, np);
  zpass(3, -1);
  axis(M1, (long long)M0 * M2h, M2h, nm, (long long)M1 * M2h, M2h, 3, -1, 1.0, tw1, 0, M0);
  axis(M0, (long long)M1 * M2h, (long long)M1 * M2h, nm, 0, (long long)M1 * M2h, 3, -1,
       1.0 / ((double)M0 * M1 * M2), tw0, p.N[1], M1);
  if (err) return err;
  const long long f1 = (long long)p.N[0] * p.N[1] * (p.N[2] / 2 + 1);
  k_rhs32<C><<<grid_for(f1), 256, 0, s>>>(spec, reinterpret_cast<const C*>(u_hat), reinterpret_cast<const C*>(src),
                                          reinterpret_cast<C*>(rhs), reinterpret_cast<C*>(phat), p);
  return (int)cudaGetLastError();
}

template <typename C> cudaError_t optin(int dev) {
  int mx = 0;
  cudaError_t e = cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  for (int n : {24, 48, 96, 192, 384, 768, 1536}) {
    by_length(n, [&](auto L) {
      constexpr int NL = decltype(L)::value;
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k_fft_axis<C, NL>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k_fft_z<C, NL>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
      return 0;
    });
  }
  return e;
}

}  // namespace

int pad32_rhs(const Pad32& p, const void* u_hat, const void* src, void* rhs, void* phat, cudaStream_t s) {
  return p.dbl ? rhs_t<double2>(p, u_hat, src, rhs, phat, s) : rhs_t<float2>(p, u_hat, src, rhs, phat, s);
}

int pad32_smem_optin(int dev, bool dbl) { return (int)(dbl ? optin<double2>(dev) : optin<float2>(dev)); }

}  // namespace sdns
