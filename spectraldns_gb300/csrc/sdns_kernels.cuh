// Transform sweeps of one RK4 stage of the pseudo-spectral Navier-Stokes
// solver (spectralDNS solvers/NS.py:191-261 restated for sm_103a).
//
// The velocity lives in HBM only inside the 2/3-rule set, as a "compact"
// array [3][K0][K1][Kzp] (K0 = 2 kc0 + 1, K1 = 2 kc1 + 1, Kz = kc2 + 1, Kzp =
// Kz rounded up to 8).  One stage is five sweeps over HBM:
//   x^-1 (+ curl)  [3][K0][K1][Kzp]   -> [6][N0][K1][Kzp]
//   y^-1           [6][N0][K1][Kzp]   -> [6][N0][N1][Kzp]
//   z: C2R(6) -> u x w -> R2C(3)      -> [3][N0][N1][Kzp]   (in place)
//   y             [3][N0][N1][Kzp]   -> [3][N0][K1][Kzp]
//   x + projection + diffusion + source + RK4 update -> compact state
// The pruned inverse transforms read only the kept rows and zero the rest in
// shared memory; the pruned forward transforms store only the kept rows
// (which is the 2/3-rule mask of the nonlinear term).
#pragma once
#include "sdns_fft.cuh"
#include "sdns_internal.h"

namespace sdns {

template <typename C> __device__ __forceinline__ C czero() { return mk<C>(0, 0); }

// ---------------------------------------------------------------------------
// strided axis sweep: MODE 0 plain copy prologue, MODE 1 curl prologue
// ---------------------------------------------------------------------------
template <typename Real, int E, int S, int MODE>
__global__ void __launch_bounds__(256) k_axis(AxisArgs a) {
  using C = typename cplx_of<Real>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int N = a.min.n;
  const int G = N / E;
  const int W = blockDim.x / G;
  const int LD = line_ld(N);
  C* sm = reinterpret_cast<C*>(smraw);
  long long* cin = reinterpret_cast<long long*>(sm + (size_t)W * LD);
  long long* cout = cin + W;
  Real* ck = reinterpret_cast<Real*>(cout + W);  // k1, kz per column (curl)
  const int f = blockIdx.y;
  const long long l0 = (long long)blockIdx.x * W;
  const int tid = threadIdx.x, nth = blockDim.x;

  for (int w = tid; w < W; w += nth) {
    const long long l = l0 + w;
    long long bi = -1, bo = -1;
    if (l < a.nlines) {
      const long long slab = l / a.B, b = l - slab * a.B;
      bi = slab * a.in_ss + b;
      bo = slab * a.out_ss + b;
      if (MODE == 1) {
        const int k1row = (int)(b / a.Kzp), kz = (int)(b - (long long)k1row * a.Kzp);
        ck[2 * w] = (Real)(a.kscale[1] * a.m1.wave(k1row));
        ck[2 * w + 1] = (Real)(a.kscale[2] * kz);
      }
    }
    cin[w] = bi;
    cout[w] = bo;
  }
  __syncthreads();

  const int rin = a.min.rows();
  const C* in = reinterpret_cast<const C*>(a.in);
  for (int i = tid; i < rin * W; i += nth) {
    const int r = i / W, w = i - r * W;
    const long long bi = cin[w];
    C v = czero<C>();
    if (bi >= 0) {
      if (MODE == 0) {
        v = in[f * a.in_fs + r * a.in_rs + bi];
      } else {
        const long long o = r * a.in_rs + bi;
        if (f < 3) {
          v = in[f * a.in_fs + o];
        } else {
          const Real k0 = (Real)(a.kscale[0] * a.min.wave(r));
          const Real k1 = ck[2 * w], k2 = ck[2 * w + 1];
          C t;
          if (f == 3) {        // i (k1 uz - kz uy)
            const C uy = in[1 * a.in_fs + o], uz = in[2 * a.in_fs + o];
            t = mk<C>(k1 * uz.x - k2 * uy.x, k1 * uz.y - k2 * uy.y);
          } else if (f == 4) { // i (kz ux - k0 uz)
            const C ux = in[o], uz = in[2 * a.in_fs + o];
            t = mk<C>(k2 * ux.x - k0 * uz.x, k2 * ux.y - k0 * uz.y);
          } else {             // i (k0 uy - k1 ux)
            const C ux = in[o], uy = in[1 * a.in_fs + o];
            t = mk<C>(k0 * uy.x - k1 * ux.x, k0 * uy.y - k1 * ux.y);
          }
          v = mk<C>(-t.y, t.x);
        }
      }
    }
    sm[w * LD + padp(a.min.pos(r))] = v;
  }
  if (a.min.kc >= 0) {
    const int nz = N - rin;
    for (int i = tid; i < nz * W; i += nth) {
      const int q = i / W, w = i - q * W;
      sm[w * LD + padp(a.min.kc + 1 + q)] = czero<C>();
    }
  }
  __syncthreads();
  {
    const int lane = tid & 31, warp = tid >> 5;
    const int w = warp * (32 / G) + lane / G;
    line_fft<E, S>(sm + w * LD, lane % G, N, reinterpret_cast<const C*>(a.tw));
  }
  __syncthreads();
  const int rout = a.mout.rows();
  C* out = reinterpret_cast<C*>(a.out);
  const Real sc = (Real)a.scale;
  for (int i = tid; i < rout * W; i += nth) {
    const int r = i / W, w = i - r * W;
    const long long bo = cout[w];
    if (bo >= 0) {
      const C v = sm[w * LD + padp(a.mout.pos(r))];
      out[f * a.out_fs + r * a.out_rs + bo] = mk<C>(v.x * sc, v.y * sc);
    }
  }
}

// ---------------------------------------------------------------------------
// z-line sweeps (R2C axis): one group of G = n/E lanes per line
// ---------------------------------------------------------------------------
// Pack the Hermitian half-spectra A, B of two real lines into the full
// spectrum of a + i b (the imaginary part of the kz=0 and kz=n/2 coefficients
// is dropped, as a C2R transform does).
template <typename C>
__device__ __forceinline__ void pack_pair(C* cb, const C* pa, const C* pb, int Kz, int n, int g, int G, bool valid) {
  for (int kz = g; kz < Kz; kz += G) {
    C A = (valid && pa) ? pa[kz] : czero<C>();
    C B = (valid && pb) ? pb[kz] : czero<C>();
    if (kz == 0 || 2 * kz == n) { A.y = 0; B.y = 0; }
    cb[padp(kz)] = mk<C>(A.x - B.y, A.y + B.x);
    if (kz > 0 && 2 * kz < n) cb[padp(n - kz)] = mk<C>(A.x + B.y, B.x - A.y);
  }
  for (int q = Kz + g; q <= n - Kz; q += G) cb[padp(q)] = czero<C>();
}

// MODE 0: NS (6 fields -> cross -> 3 fields), 1: C2R only, 2: R2C only
template <typename Real, int E, int MODE>
__global__ void __launch_bounds__(128) k_zline(ZArgs a) {
  using C = typename cplx_of<Real>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int N = a.n, G = N / E, LPW = 32 / G, LD = line_ld(N);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G, g = lane % G;
  const long long line = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * LPW + sub;
  const bool valid = line < a.nlines;
  const int NB = (MODE == 0) ? 3 : 2;
  C* buf = sm + (size_t)((warp * LPW + sub) * NB) * LD;
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const long long fs = a.nlines * a.Kzp;
  const C* in = reinterpret_cast<const C*>(a.in);
  const long long lo = line * a.Kzp;
  const int npair = (MODE == 0) ? 3 : (a.nf + 1) / 2;

  if (MODE == 0 || MODE == 1) {
    for (int p = 0; p < npair; ++p) {
      const int fa = 2 * p, fb = 2 * p + 1;
      const int nfin = (MODE == 0) ? 6 : a.nf;
      pack_pair(buf + p * LD, in + fa * fs + lo, fb < nfin ? in + fb * fs + lo : (const C*)nullptr,
                a.Kz, N, g, G, valid);
    }
    __syncwarp();
    for (int p = 0; p < npair; ++p) line_fft<E, +1>(buf + p * LD, g, N, tw);
  }
  if (MODE == 1) {
    Real* ph = reinterpret_cast<Real*>(a.phys);
    const long long pfs = a.nlines * (long long)N;
    if (valid) {
      for (int m = 0; m < E; ++m) {
        const int n = g + G * m;
        for (int p = 0; p < npair; ++p) {
          const C c = buf[p * LD + padp(n)];
          ph[(2 * p) * pfs + line * N + n] = c.x;
          if (2 * p + 1 < a.nf) ph[(2 * p + 1) * pfs + line * N + n] = c.y;
        }
      }
    }
    return;
  }
  if (MODE == 0) {
    double rmax = 0.0;
#pragma unroll 4
    for (int m = 0; m < E; ++m) {
      const int n = padp(g + G * m);
      const C c0 = buf[n], c1 = buf[LD + n], c2 = buf[2 * LD + n];
      const Real u0 = c0.x, u1 = c0.y, u2 = c1.x, w0 = c1.y, w1 = c2.x, w2 = c2.y;
      if (a.cfl_rate)
        rmax = fmax(rmax, fabs((double)u0) * a.inv_dx[0] + fabs((double)u1) * a.inv_dx[1] + fabs((double)u2) * a.inv_dx[2]);
      buf[n] = mk<C>(u1 * w2 - u2 * w1, u2 * w0 - u0 * w2);
      buf[LD + n] = mk<C>(u0 * w1 - u1 * w0, (Real)0);
    }
    if (a.cfl_rate) {
      if (!valid) rmax = 0.0;
      for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
      if (lane == 0) atomicMax(reinterpret_cast<unsigned long long*>(a.cfl_rate), (unsigned long long)__double_as_longlong(rmax));
    }
  } else {  // MODE 2: load physical pairs
    const Real* ph = reinterpret_cast<const Real*>(a.phys);
    const long long pfs = a.nlines * (long long)N;
    for (int p = 0; p < npair; ++p) {
      for (int m = 0; m < E; ++m) {
        const int n = g + G * m;
        Real x = 0, y = 0;
        if (valid) {
          x = ph[(2 * p) * pfs + line * N + n];
          if (2 * p + 1 < a.nf) y = ph[(2 * p + 1) * pfs + line * N + n];
        }
        buf[p * LD + padp(n)] = mk<C>(x, y);
      }
    }
  }
  __syncwarp();
  const int nout = (MODE == 0) ? 3 : a.nf;
  const int nfwd = (nout + 1) / 2;
  for (int p = 0; p < nfwd; ++p) line_fft<E, -1>(buf + p * LD, g, N, tw);
  if (!valid) return;
  C* out = reinterpret_cast<C*>(a.out);
  for (int kz = g; kz < a.Kzp; kz += G) {
    for (int p = 0; p < nfwd; ++p) {
      const bool two = (2 * p + 1 < nout);
      C oa = czero<C>(), ob = czero<C>();
      if (kz < a.Kz) {
        const C X = buf[p * LD + padp(kz)];
        if (two) {
          const C Yc = buf[p * LD + padp((N - kz) & (N - 1))];
          oa = mk<C>((Real)0.5 * (X.x + Yc.x), (Real)0.5 * (X.y - Yc.y));
          ob = mk<C>((Real)0.5 * (X.y + Yc.y), (Real)0.5 * (Yc.x - X.x));
        } else {
          oa = X;
        }
      }
      out[(2 * p) * fs + lo + kz] = oa;
      if (two) out[(2 * p + 1) * fs + lo + kz] = ob;
    }
  }
}

// ---------------------------------------------------------------------------
// final x sweep + projection + diffusion + source + RK4 stage update
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 d2(double x, double y) { return make_double2(x, y); }

template <typename Real, int E>
__global__ void __launch_bounds__(256) k_axis_rk(RKArgs a) {
  using C = typename cplx_of<Real>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int N = a.m0.n, G = N / E, W = blockDim.x / G, LD = line_ld(N);
  C* sm = reinterpret_cast<C*>(smraw);
  int* ck1 = reinterpret_cast<int*>(sm + (size_t)3 * W * LD);
  int* ckz = ck1 + W;
  __shared__ double red[2][32];
  const long long l0 = (long long)blockIdx.x * W;
  const int tid = threadIdx.x, nth = blockDim.x;
  const long long nl = a.nlines;
  for (int w = tid; w < W; w += nth) {
    const long long l = l0 + w;
    if (l < nl) {
      const int k1row = (int)(l / a.Kzp);
      ck1[w] = k1row;
      ckz[w] = (int)(l - (long long)k1row * a.Kzp);
    } else {
      ck1[w] = -1;
      ckz[w] = -1;
    }
  }
  const C* in = reinterpret_cast<const C*>(a.in);
  for (int f = 0; f < 3; ++f) {
    for (int i = tid; i < N * W; i += nth) {
      const int r = i / W, w = i - r * W;
      const long long l = l0 + w;
      sm[(f * W + w) * LD + padp(r)] = (l < nl) ? in[((long long)f * N + r) * nl + l] : czero<C>();
    }
  }
  __syncthreads();
  {
    const int lane = tid & 31, warp = tid >> 5;
    const int w = warp * (32 / G) + lane / G;
    const C* tw = reinterpret_cast<const C*>(a.tw);
    for (int f = 0; f < 3; ++f) line_fft<E, -1>(sm + (f * W + w) * LD, lane % G, N, tw);
  }
  __syncthreads();

  const int K0 = a.m0.rows();
  const long long cs = (long long)K0 * nl;  // component stride of the compact layout
  const double dt = *a.dt;
  const double alpha = a.force_alpha ? *a.force_alpha : 0.0;
  C* Y = reinterpret_cast<C*>(a.Y);
  double e_sum = 0.0, z_sum = 0.0;
  for (int i = tid; i < K0 * W; i += nth) {
    const int r = i / W, w = i - r * W;
    const int k1row = ck1[w], kz = ckz[w];
    if (k1row < 0) continue;
    const long long o = (long long)r * nl + l0 + w;
    if (kz >= a.Kz) {  // padding of the R2C axis stays zero
      for (int c = 0; c < 3; ++c) {
        if (a.stage == 4) {
          reinterpret_cast<C*>(a.rhs_out)[c * cs + o] = czero<C>();
        } else {
          Y[c * cs + o] = czero<C>();
          if (a.stage == 3) a.S[c * cs + o] = d2(0, 0); else a.A[c * cs + o] = d2(0, 0);
        }
      }
      if (a.p_out) reinterpret_cast<C*>(a.p_out)[o] = czero<C>();
      continue;
    }
    const int p = a.m0.pos(r);
    const double k[3] = {a.kscale[0] * a.m0.wave(r), a.kscale[1] * a.m1.wave(k1row), a.kscale[2] * kz};
    const double K2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    const double iK2 = K2 > 0.0 ? 1.0 / K2 : 0.0;
    double2 nlv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C v = sm[(c * W + w) * LD + padp(p)];
      nlv[c] = d2((double)v.x * a.scale, (double)v.y * a.scale);
    }
    const double2 P = d2((nlv[0].x * k[0] + nlv[1].x * k[1] + nlv[2].x * k[2]) * iK2,
                         (nlv[0].y * k[0] + nlv[1].y * k[1] + nlv[2].y * k[2]) * iK2);
    if (a.p_out) reinterpret_cast<C*>(a.p_out)[o] = mk<C>((Real)P.x, (Real)P.y);
    const bool forced = a.force_alpha && K2 > 0.0 && K2 <= a.kf2;
    double2 snew[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long oc = c * cs + o;
      double2 u, s;
      if (a.stage == 0) {
        s = a.S[oc];
        u = s;
      } else {
        const C y = Y[oc];
        u = d2((double)y.x, (double)y.y);
        if (a.stage == 1 || a.stage == 2 || forced) s = a.S[oc];
      }
      double2 rhs = d2(nlv[c].x - P.x * k[c] - a.nu * K2 * u.x, nlv[c].y - P.y * k[c] - a.nu * K2 * u.y);
      if (a.source) { const double2 q = a.source[oc]; rhs.x += q.x; rhs.y += q.y; }
      if (forced) { rhs.x += alpha * s.x; rhs.y += alpha * s.y; }
      if (a.stage == 4) {
        reinterpret_cast<C*>(a.rhs_out)[oc] = mk<C>((Real)rhs.x, (Real)rhs.y);
      } else if (a.stage == 0) {
        Y[oc] = mk<C>((Real)(s.x + a.b * dt * rhs.x), (Real)(s.y + a.b * dt * rhs.y));
        a.A[oc] = d2(s.x + a.a * dt * rhs.x, s.y + a.a * dt * rhs.y);
      } else if (a.stage < 3) {
        const double2 acc = a.A[oc];
        Y[oc] = mk<C>((Real)(s.x + a.b * dt * rhs.x), (Real)(s.y + a.b * dt * rhs.y));
        a.A[oc] = d2(acc.x + a.a * dt * rhs.x, acc.y + a.a * dt * rhs.y);
      } else {
        const double2 acc = a.A[oc];
        const double2 sn = d2(acc.x + a.a * dt * rhs.x, acc.y + a.a * dt * rhs.y);
        a.S[oc] = sn;
        Y[oc] = mk<C>((Real)sn.x, (Real)sn.y);
        snew[c] = sn;
      }
    }
    if (a.stage == 3) {
      const double wz = (kz == 0) ? 0.5 : 1.0;  // 1/2 * Hermitian weight
      e_sum += wz * (snew[0].x * snew[0].x + snew[0].y * snew[0].y + snew[1].x * snew[1].x +
                     snew[1].y * snew[1].y + snew[2].x * snew[2].x + snew[2].y * snew[2].y);
      // |k x u|^2
      const double cx_r = k[1] * snew[2].x - k[2] * snew[1].x, cx_i = k[1] * snew[2].y - k[2] * snew[1].y;
      const double cy_r = k[2] * snew[0].x - k[0] * snew[2].x, cy_i = k[2] * snew[0].y - k[0] * snew[2].y;
      const double cz_r = k[0] * snew[1].x - k[1] * snew[0].x, cz_i = k[0] * snew[1].y - k[1] * snew[0].y;
      z_sum += wz * (cx_r * cx_r + cx_i * cx_i + cy_r * cy_r + cy_i * cy_i + cz_r * cz_r + cz_i * cz_i);
    }
  }
  if (a.stage == 3 && a.partials) {
    for (int o = 16; o > 0; o >>= 1) {
      e_sum += __shfl_xor_sync(0xffffffffu, e_sum, o);
      z_sum += __shfl_xor_sync(0xffffffffu, z_sum, o);
    }
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) { red[0][warp] = e_sum; red[1][warp] = z_sum; }
    __syncthreads();
    if (tid == 0) {
      double e = 0, z = 0;
      for (int q = 0; q < (nth + 31) / 32; ++q) { e += red[0][q]; z += red[1][q]; }
      a.partials[2 * blockIdx.x] = e;
      a.partials[2 * blockIdx.x + 1] = z;
    }
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
inline int elems_for(int n) { return n >= 1024 ? 32 : 16; }

template <typename Real>
static size_t axis_smem(int n, int W, bool curl) {
  using C = typename cplx_of<Real>::type;
  return (size_t)W * line_ld(n) * sizeof(C) + 2 * W * sizeof(long long) + (curl ? 2 * W * sizeof(Real) : 0) + 16;
}

template <typename Real, int E, int S, int MODE>
static int launch_axis(const AxisArgs& a, cudaStream_t s) {
  const int G = a.min.n / E;
  const int W = 256 / G;
  const size_t sm = axis_smem<Real>(a.min.n, W, MODE == 1);
  auto kern = k_axis<Real, E, S, MODE>;
  dim3 grid((unsigned)((a.nlines + W - 1) / W), (unsigned)a.nfield, 1);
  kern<<<grid, 256, sm, s>>>(a);
  return (int)cudaGetLastError();
}

template <typename Real>
int Kernels<Real>::axis_plain(const AxisArgs& a, int sign, cudaStream_t s) {
  const int E = elems_for(a.min.n);
  if (E == 16) return sign < 0 ? launch_axis<Real, 16, -1, 0>(a, s) : launch_axis<Real, 16, 1, 0>(a, s);
  return sign < 0 ? launch_axis<Real, 32, -1, 0>(a, s) : launch_axis<Real, 32, 1, 0>(a, s);
}

template <typename Real>
int Kernels<Real>::axis_curl_inv(const AxisArgs& a, cudaStream_t s) {
  const int E = elems_for(a.min.n);
  if (E == 16) return launch_axis<Real, 16, 1, 1>(a, s);
  return launch_axis<Real, 32, 1, 1>(a, s);
}

template <typename Real, int E, int MODE>
static int launch_z(const ZArgs& a, cudaStream_t s) {
  using C = typename cplx_of<Real>::type;
  const int G = a.n / E, LPW = 32 / G;
  const int NB = (MODE == 0) ? 3 : 2;
  const int warps = 4;
  const size_t sm = (size_t)warps * LPW * NB * line_ld(a.n) * sizeof(C);
  auto kern = k_zline<Real, E, MODE>;
  const long long per_block = (long long)warps * LPW;
  dim3 grid((unsigned)((a.nlines + per_block - 1) / per_block));
  kern<<<grid, warps * 32, sm, s>>>(a);
  return (int)cudaGetLastError();
}

template <typename Real>
int Kernels<Real>::zline_ns(const ZArgs& a, cudaStream_t s) {
  return elems_for(a.n) == 16 ? launch_z<Real, 16, 0>(a, s) : launch_z<Real, 32, 0>(a, s);
}
template <typename Real>
int Kernels<Real>::zline_c2r(const ZArgs& a, cudaStream_t s) {
  return elems_for(a.n) == 16 ? launch_z<Real, 16, 1>(a, s) : launch_z<Real, 32, 1>(a, s);
}
template <typename Real>
int Kernels<Real>::zline_r2c(const ZArgs& a, cudaStream_t s) {
  return elems_for(a.n) == 16 ? launch_z<Real, 16, 2>(a, s) : launch_z<Real, 32, 2>(a, s);
}

template <typename Real, int E>
static int launch_rk(const RKArgs& a, cudaStream_t s, int* nblocks) {
  using C = typename cplx_of<Real>::type;
  const int G = a.m0.n / E;
  int W = 256 / G;
  auto smsize = [&](int w) { return (size_t)3 * w * line_ld(a.m0.n) * sizeof(C) + 2 * w * sizeof(int) + 16; };
  while (W > 1 && smsize(W) > 200 * 1024) W /= 2;
  const size_t sm = smsize(W);
  auto kern = k_axis_rk<Real, E>;
  const unsigned nb = (unsigned)((a.nlines + W - 1) / W);
  if (nblocks) *nblocks = (int)nb;
  kern<<<nb, W * G, sm, s>>>(a);
  return (int)cudaGetLastError();
}

template <typename Real>
int Kernels<Real>::axis_rk(const RKArgs& a, cudaStream_t s, int* nblocks) {
  return elems_for(a.m0.n) == 16 ? launch_rk<Real, 16>(a, s, nblocks) : launch_rk<Real, 32>(a, s, nblocks);
}

// Allow the large dynamic shared-memory tiles once per device (outside any
// stream capture).
template <typename K> static cudaError_t optin_one(K kern, int optin) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

template <typename Real>
int Kernels<Real>::smem_optin(int dev) {
  int mx = 0;
  cudaError_t e = cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
#define SDNS_OPT(k) if (e == cudaSuccess) e = optin_one(k, mx)
  SDNS_OPT((k_axis<Real, 16, -1, 0>)); SDNS_OPT((k_axis<Real, 16, 1, 0>)); SDNS_OPT((k_axis<Real, 16, 1, 1>));
  SDNS_OPT((k_axis<Real, 32, -1, 0>)); SDNS_OPT((k_axis<Real, 32, 1, 0>)); SDNS_OPT((k_axis<Real, 32, 1, 1>));
  SDNS_OPT((k_zline<Real, 16, 0>)); SDNS_OPT((k_zline<Real, 16, 1>)); SDNS_OPT((k_zline<Real, 16, 2>));
  SDNS_OPT((k_zline<Real, 32, 0>)); SDNS_OPT((k_zline<Real, 32, 1>)); SDNS_OPT((k_zline<Real, 32, 2>));
  SDNS_OPT((k_axis_rk<Real, 16>)); SDNS_OPT((k_axis_rk<Real, 32>));
#undef SDNS_OPT
  return (int)e;
}

// number of CTAs axis_rk launches (for sizing the partials buffer)
template <typename Real>
inline long long rk_blocks(int n0, long long nlines) {
  using C = typename cplx_of<Real>::type;
  const int E = elems_for(n0), G = n0 / E;
  int W = 256 / G;
  while (W > 1 && (size_t)3 * W * line_ld(n0) * sizeof(C) + 2 * W * sizeof(int) + 16 > 200 * 1024) W /= 2;
  return (nlines + W - 1) / W;
}

}  // namespace sdns
