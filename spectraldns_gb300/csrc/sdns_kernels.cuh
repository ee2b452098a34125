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
// The pruned inverse transforms read only the kept rows (the rest of the line
// is zero); the pruned forward transforms store only the kept rows (which is
// the 2/3-rule mask of the nonlinear term).  Tiles are staged into shared
// memory with cp.async so that a whole tile is in flight per thread block.
#pragma once
#include "sdns_fft.cuh"
#include "sdns_internal.h"

namespace sdns {

template <typename C> __device__ __forceinline__ C czero() { return mk<C>(0, 0); }

// error-free float-float addition (Knuth TwoSum + renormalisation)
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  const float t = __fadd_rn(e, lo);
  hi = __fadd_rn(s, t);
  lo = __fsub_rn(t, __fsub_rn(hi, s));
}

// ---------------------------------------------------------------------------
// Persistent, double-buffered plain axis sweep (MODE 0 of k_axis).  A task is
// one tile of W adjacent lines of one field (tasks field-major, so blocks
// running at the same time stream neighbouring tiles of one field); each
// block walks tasks blockIdx.x, blockIdx.x + gridDim.x, ... and stages the
// next task's rows with cp.async while it transforms and stores the current
// one.  Every thread stages and stores one fixed column (line) of the tile,
// so the line bases are computed once per task.
// ---------------------------------------------------------------------------
template <int N> struct axis_e { static constexpr int value = N >= 1024 ? 32 : 16; };

// Pitch (in complex values) of a tile of W lines in shared memory, at least
// `minlen`.  The staging and store phases access the tile row by row, W
// lines wide; one shared-memory wavefront serves L = 128/csz lanes.  With
// W >= L the L lanes hit L lines of one row (odd pitch: distinct banks); with
// W < L they hit L/W rows of W lines, distinct when pitch = L/W (mod L).
__host__ __device__ inline int tile_pitch(int minlen, int W, int csz) {
  const int L = 128 / csz;
  int ld = minlen;
  if (W >= L) return ld | 1;
  const int want = L / W;
  while ((ld & (L - 1)) != want) ++ld;
  return ld;
}
__host__ __device__ inline int axis_ld(int n, int W, int csz) { return tile_pitch(n + ((n - 1) >> 4), W, csz); }

// FP32 lines of 512 and 1024 points use the two-pass radix-32 transforms
template <typename Real, int N> struct axis_r32 {
  static constexpr bool value = sizeof(Real) == 4 && (N == 512 || N == 1024);
};

template <typename Real, int N, int S>
__global__ void __launch_bounds__(256, axis_r32<Real, N>::value ? 2 : 3) k_axis_p(AxisArgs a) {
  using C = typename cplx_of<Real>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr bool R32 = axis_r32<Real, N>::value;
  constexpr int E = R32 ? 32 : axis_e<N>::value, G = N / E;
  const int W = blockDim.x / G, LD = axis_ld(N, W, (int)sizeof(C));
  const int wsh = __ffs(W) - 1;
  C* const bufs = reinterpret_cast<C*>(smraw);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wl = warp * (32 / G) + lane / G, g = lane % G;  // FFT phase: line of this lane
  const int wc = tid & (W - 1), r0 = tid >> wsh;            // staging phase: column, first row (step G)
  // 32-bit task bookkeeping (the launcher checks nlines * nfield < 2^31)
  const unsigned nlines = (unsigned)a.nlines, B = (unsigned)a.B;
  const unsigned ntile = (nlines + W - 1) / W;
  const unsigned ntask = ntile * (unsigned)a.nfield;
  const int rin = a.min.rows(), rout = a.mout.rows();
  const C* in = reinterpret_cast<const C*>(a.in);
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const Real sc = (Real)a.scale;
  // rows are staged at their line positions; the positions between the kept
  // rows of a pruned input (kc < p < N - kc) are written with zeros
  const int kcin = a.min.kc, shift = N - rin;
  const bool prune = prunable(N, kcin);
  auto issue = [&](unsigned f, unsigned tile, C* dst) {
    const unsigned l = tile * W + wc;
    if (l < nlines) {
      const unsigned slab = l / B;
      const C* src = in + (long long)f * a.in_fs + (long long)slab * a.in_ss + (l - slab * B) + (long long)r0 * a.in_rs;
      const long long step = (long long)G * a.in_rs;
      C* d = dst + wc * LD;
      if (kcin >= 0) {
        for (int r = r0; r < rin; r += G, src += step) cp_async<sizeof(C)>(d + padp(r <= kcin ? r : r + shift), src);
        if (prune) {  // positions 6N/16 .. 10N/16-1 are never read (pruned first pass)
          for (int p = kcin + 1 + r0; p < 6 * (N / 16); p += G) d[padp(p)] = czero<C>();
          for (int p = 10 * (N / 16) + r0; p < N - kcin; p += G) d[padp(p)] = czero<C>();
        } else {
          for (int p = kcin + 1 + r0; p < N - kcin; p += G) d[padp(p)] = czero<C>();
        }
      } else {
        for (int r = r0; r < rin; r += G, src += step) cp_async<sizeof(C)>(d + padp(r), src);
      }
    }
    cp_commit();
  };
  const unsigned gstep = gridDim.x;
  const bool dbuf = a.nbuf == 2;  // double buffering: the next tile is in flight during this one
  unsigned task = blockIdx.x;
  unsigned f = task / ntile, tile = task - f * ntile;
  int b = 0;
  if (task < ntask && dbuf) issue(f, tile, bufs);
  for (; task < ntask; task += gstep, b ^= (dbuf ? 1 : 0)) {
    C* const cur = bufs + (size_t)b * W * LD;
    unsigned nf = f, ntl = tile + gstep;
    while (ntl >= ntile) { ntl -= ntile; ++nf; }
    if (!dbuf) {
      issue(f, tile, cur);
      cp_wait_all();
    } else if (task + gstep < ntask) {
      issue(nf, ntl, bufs + (size_t)(b ^ 1) * W * LD);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      cp_wait_all();
    }
    __syncthreads();
    if constexpr (R32) {
      if (prune) line_fft_r32<N, S, true>(cur + wl * LD, g, tw);
      else line_fft_r32<N, S, false>(cur + wl * LD, g, tw);
    } else {
      if (prune) line_fft_t<N, E, S, true>(cur + wl * LD, g, tw);
      else line_fft_t<N, E, S, false>(cur + wl * LD, g, tw);
    }
    __syncthreads();
    {
      C* out = reinterpret_cast<C*>(a.out) + (long long)f * a.out_fs;
      if constexpr (sizeof(C) == 8) {
        // adjacent line pairs -> one 16-byte store; this thread: columns 2u, 2u+1
        const int Wh = W >> 1, u = tid % Wh;
        const unsigned l0 = tile * W + 2 * u;
        if (l0 < nlines) {
          const unsigned slab = l0 / B, rem = l0 - slab * B;
          const long long b0 = (long long)slab * a.out_ss + rem;
          const bool has1 = l0 + 1 < nlines;
          const long long b1 = (rem + 1 < B) ? b0 + 1 : (long long)(slab + 1) * a.out_ss;
          const bool pair = has1 && b1 == b0 + 1 && ((b0 & 1) == 0) && ((a.out_rs & 1) == 0);
          const C* c0 = cur + (2 * u) * LD;
          for (int r = tid / Wh; r < rout; r += nth / Wh) {
            const int pp = padp(a.mout.pos(r));
            const C v0 = c0[pp];
            const long long o = r * a.out_rs + b0;
            if (pair) {
              const C v1 = c0[LD + pp];
              reinterpret_cast<float4*>(out)[o >> 1] = make_float4(v0.x * sc, v0.y * sc, v1.x * sc, v1.y * sc);
            } else {
              out[o] = mk<C>(v0.x * sc, v0.y * sc);
              if (has1) {
                const C v1 = c0[LD + pp];
                out[r * a.out_rs + b1] = mk<C>(v1.x * sc, v1.y * sc);
              }
            }
          }
        }
      } else {
        const unsigned l = tile * W + wc;
        if (l < nlines) {
          const unsigned slab = l / B;
          const long long bo = (long long)slab * a.out_ss + (l - slab * B);
          const C* c0 = cur + wc * LD;
          for (int r = r0; r < rout; r += G) {
            const C v = c0[padp(a.mout.pos(r))];
            out[r * a.out_rs + bo] = mk<C>(v.x * sc, v.y * sc);
          }
        }
      }
    }
    __syncthreads();  // cur is refilled (double buffering: two tasks ahead)
    f = nf;
    tile = ntl;
  }
}

// x^-1 sweep with the curl: one block stages the three velocity components of
// a tile of W lines once and produces all six output fields from them (u_hat
// and i K x u_hat), one line transform per warp and field.  With VV the staged
// vector is the vorticity w_hat and the six fields are the velocity
// i K x w_hat / K^2 (spectralDNS/solvers/VV.py:52-67, K_over_K2 with K2 = 0 -> 1)
// and w_hat itself (VV.py:97-98).
__host__ __device__ inline int staged_rows(int rin, int W, int csz) {
  return tile_pitch((rin - 1) + ((rin - 1) >> 4) + 1, W, csz);
}

template <typename Real, int N, bool VV = false>
__global__ void __launch_bounds__(512, 1) k_axis_curl6(AxisArgs a) {
  using C = typename cplx_of<Real>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int E = axis_e<N>::value, G = N / E;
  const int W = blockDim.x / G, LD = axis_ld(N, W, (int)sizeof(C));
  const int wsh = __ffs(W) - 1;
  const int rin = a.min.rows(), rout = a.mout.rows();
  const int PR = staged_rows(rin, W, (int)sizeof(C));
  C* const comp = reinterpret_cast<C*>(smraw);    // [3][W][PR] staged components
  C* const work = comp + (size_t)3 * W * PR;       // [W][LD] transform buffers
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wl = warp * (32 / G) + lane / G, g = lane % G;
  const int wc = tid & (W - 1), r0 = tid >> wsh;
  const long long tile = blockIdx.x;
  const C* in = reinterpret_cast<const C*>(a.in);
  const C* tw = reinterpret_cast<const C*>(a.tw);
  {
    const long long l = tile * W + wc;
    if (l < a.nlines) {
      const long long step = (long long)G * a.in_rs;
#pragma unroll 1
      for (int c = 0; c < 3; ++c) {
        const C* src = in + c * a.in_fs + l + (long long)r0 * a.in_rs;
        C* d = comp + (size_t)(c * W + wc) * PR;
        for (int r = r0; r < rin; r += G, src += step) cp_async<sizeof(C)>(d + padp(r), src);
      }
    }
    cp_commit();
  }
  // wave numbers of this lane's line: b = k1row * Kzp + kz
  Real k1 = 0, kz = 0;
  {
    const long long l = tile * W + wl;
    if (l < a.nlines) {
      const int k1row = (int)(l / a.Kzp);
      k1 = (Real)(a.kscale[1] * a.m1.wave(k1row));
      kz = (Real)(a.kscale[2] * (double)(l - (long long)k1row * a.Kzp));
    }
  }
  const Real ks0 = (Real)a.kscale[0];
  const RowMap mi = a.min;
  cp_wait_all();
  __syncthreads();
#pragma unroll 1
  for (int f = 0; f < 6; ++f) {
    C* line = work + wl * LD;
    // cross-product field: NS fields 3..5, VV fields 0..2; cf = its component
    const bool crossf = VV ? (f < 3) : (f >= 3);
    const int cf = f < 3 ? f : f - 3;
    int c1 = cf, c2 = 0;
    if (crossf) {
      if (cf == 0) { c1 = 2; c2 = 1; }       // i (k1 uz - kz uy)
      else if (cf == 1) { c1 = 0; c2 = 2; }  // i (kz ux - k0 uz)
      else { c1 = 1; c2 = 0; }               // i (k0 uy - k1 ux)
    }
    const C* s1 = comp + (size_t)(c1 * W + wl) * PR;
    const C* s2 = comp + (size_t)(c2 * W + wl) * PR;
    auto ld = [&](int p) -> C {
      int r = p;
      if (mi.kc >= 0) {
        if (p > mi.kc && p < N - mi.kc) return czero<C>();
        if (p > mi.kc) r = p - N + 2 * mi.kc + 1;
      }
      const C v1 = s1[padp(r)];
      if (!crossf) return v1;
      const C v2 = s2[padp(r)];
      C t;
      if (cf == 0 && !VV) {
        t = mk<C>(k1 * v1.x - kz * v2.x, k1 * v1.y - kz * v2.y);
      } else {
        const Real k0 = ks0 * (Real)mi.wave(r);
        if (cf == 0) t = mk<C>(k1 * v1.x - kz * v2.x, k1 * v1.y - kz * v2.y);
        else if (cf == 1) t = mk<C>(kz * v1.x - k0 * v2.x, kz * v1.y - k0 * v2.y);
        else t = mk<C>(k0 * v1.x - k1 * v2.x, k0 * v1.y - k1 * v2.y);
        if constexpr (VV) {
          const Real K2 = k0 * k0 + k1 * k1 + kz * kz;
          const Real iK2 = K2 > (Real)0 ? (Real)1 / K2 : (Real)0;
          t = mk<C>(t.x * iK2, t.y * iK2);
        }
      }
      return mk<C>(-t.y, t.x);
    };
    if (prunable(N, mi.kc)) line_fft_ld_t<N, E, 1, true>(line, g, tw, ld);
    else line_fft_ld_t<N, E, 1, false>(line, g, tw, ld);
    __syncthreads();
    C* out = reinterpret_cast<C*>(a.out) + f * a.out_fs;
    if constexpr (sizeof(C) == 8) {
      const int Wh = W >> 1, u = tid % Wh;
      const long long l0 = tile * W + 2 * u;
      if (l0 < a.nlines) {
        const bool pair = l0 + 1 < a.nlines;  // l0 even, a.B = nlines and out_rs even: 16-byte aligned pair
        const C* c0 = work + (2 * u) * LD;
        for (int r = tid / Wh; r < rout; r += nth / Wh) {
          const int pp = padp(a.mout.pos(r));
          const C v0 = c0[pp];
          const long long o = r * a.out_rs + l0;
          if (pair) {
            const C v1 = c0[LD + pp];
            reinterpret_cast<float4*>(out)[o >> 1] = make_float4(v0.x, v0.y, v1.x, v1.y);
          } else {
            out[o] = v0;
          }
        }
      }
    } else {
      const long long l = tile * W + wc;
      if (l < a.nlines) {
        const C* c0 = work + wc * LD;
        for (int r = r0; r < rout; r += G) out[r * a.out_rs + l] = c0[padp(a.mout.pos(r))];
      }
    }
    __syncthreads();
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

// extract the half spectra of the two real lines packed in X (forward FFT of a + i b)
template <typename C, typename Real>
__device__ __forceinline__ void unpack_pair(const C* buf, int kz, int N, C& oa, C& ob) {
  const C X = buf[padp(kz)];
  const C Yc = buf[padp((N - kz) & (N - 1))];
  oa = mk<C>((Real)0.5 * (X.x + Yc.x), (Real)0.5 * (X.y - Yc.y));
  ob = mk<C>((Real)0.5 * (X.y + Yc.y), (Real)0.5 * (Yc.x - X.x));
}

// Fused NS z sweep (persistent warps).  Per line: stage the 6 spectral rows
// (u_hat, w_hat after the x and y inverse sweeps) with cp.async, pack pairs,
// 3 inverse FFTs, u x w (+ CFL maximum), 2 forward FFTs, store 3 rows.  The
// staging area is refilled with the next line while the current one is
// transformed.
// complex values of shared memory per warp of k_zline_ns (kept even so that
// every warp block starts on a 16-byte boundary)
__host__ __device__ inline size_t zns_per_warp(int LD, int Kzp, int LPW) {
  const size_t n = (size_t)LPW * ((size_t)6 * Kzp + (size_t)3 * LD);
  return (n + 1) & ~(size_t)1;
}

template <typename Real, int E>
__global__ void __launch_bounds__(64) k_zline_ns(ZArgs a) {
  using C = typename cplx_of<Real>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int N = a.n, G = N / E, LPW = 32 / G, LD = line_ld(N);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G, g = lane % G;
  const int Kzp = a.Kzp;
  // per warp: LPW staging areas of 6 rows of Kzp (16-byte aligned: Kzp is a
  // multiple of 8 and each warp block has an even number of complex values),
  // then LPW x 3 work buffers of LD
  const size_t per_warp = zns_per_warp(LD, Kzp, LPW);
  C* base = sm + (size_t)warp * per_warp;
  C* stg = base + (size_t)sub * 6 * Kzp;
  C* buf = base + (size_t)LPW * 6 * Kzp + (size_t)sub * 3 * LD;
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const long long fs = a.nlines * Kzp;
  const C* in = reinterpret_cast<const C*>(a.in);
  C* out = reinterpret_cast<C*>(a.out);
  const long long wstride = (long long)gridDim.x * (blockDim.x >> 5) * LPW;
  const long long wfirst = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * LPW;
  long long line = wfirst + sub;
  constexpr int VB = 16 / (int)sizeof(C);  // complex values per 16-byte copy
  auto stage = [&](long long ln) {
    if (ln < a.nlines) {
      const int nchunk = 6 * Kzp / VB;
      for (int q = g; q < nchunk; q += G) {
        const int f = (q * VB) / Kzp, k = q * VB - f * Kzp;
        cp_async16(stg + f * Kzp + k, in + f * fs + ln * Kzp + k);
      }
    }
    cp_commit();
  };
  stage(line);
  double rmax = 0.0;
  // all lanes of a warp iterate together (the loop bound is the warp's first line)
  for (long long wl = wfirst; wl < a.nlines; wl += wstride, line += wstride) {
    const bool valid = line < a.nlines;
    cp_wait_all();
    __syncwarp();
    // pack 3 pairs from staging into the work buffers
    for (int p = 0; p < 3; ++p)
      pack_pair(buf + p * LD, stg + (2 * p) * Kzp, stg + (2 * p + 1) * Kzp, a.Kz, N, g, G, valid);
    __syncwarp();
    stage(line + wstride);
    for (int p = 0; p < 3; ++p) line_fft<E, +1>(buf + p * LD, g, N, tw);
#pragma unroll 4
    for (int m = 0; m < E; ++m) {
      const int n = padp(g + G * m);
      const C c0 = buf[n], c1 = buf[LD + n], c2 = buf[2 * LD + n];
      const Real u0 = c0.x, u1 = c0.y, u2 = c1.x, w0 = c1.y, w1 = c2.x, w2 = c2.y;
      if (a.cfl_rate && valid)
        rmax = fmax(rmax, fabs((double)u0) * a.inv_dx[0] + fabs((double)u1) * a.inv_dx[1] +
                              fabs((double)u2) * a.inv_dx[2]);
      buf[n] = mk<C>(u1 * w2 - u2 * w1, u2 * w0 - u0 * w2);
      buf[LD + n] = mk<C>(u0 * w1 - u1 * w0, (Real)0);
    }
    __syncwarp();
    line_fft<E, -1>(buf, g, N, tw);
    line_fft<E, -1>(buf + LD, g, N, tw);
    if (valid) {
      const long long lo = line * Kzp;
      for (int kz = g; kz < Kzp; kz += G) {
        C oa = czero<C>(), ob = czero<C>(), oc = czero<C>();
        if (kz < a.Kz) {
          unpack_pair<C, Real>(buf, kz, N, oa, ob);
          oc = buf[LD + padp(kz)];
        }
        out[lo + kz] = oa;
        out[fs + lo + kz] = ob;
        out[2 * fs + lo + kz] = oc;
      }
    }
    __syncwarp();
  }
  cp_wait_all();
  if (a.cfl_rate) {
    for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    if (lane == 0 && rmax > 0.0)
      atomicMax(reinterpret_cast<unsigned long long*>(a.cfl_rate), (unsigned long long)__double_as_longlong(rmax));
  }
}

// FP32 z sweep of 1024-point lines: the structure of k_zline_ns (persistent
// warps, one line per warp, the next line's six rows staged with cp.async while
// the current one is transformed) with the two-pass radix-32 transforms of the
// strided sweeps (compile-time strides; the inverse transforms skip the zero
// middle of the line in their first pass).
// With PF false there is no staging area: the rows are read from global memory
// as the pairs are packed, and the smaller footprint fits twice the warps per SM.
__host__ __device__ inline size_t zr32_per_warp(int LD, int Kzp, bool pf) {
  const size_t n = (pf ? (size_t)6 * Kzp : 0) + (size_t)3 * LD;
  return (n + 1) & ~(size_t)1;
}

template <int N, bool PR, bool PF>
__global__ void __launch_bounds__(64) k_zline_ns_r32(ZArgs a) {
  using C = float2;
  constexpr int E = 32, G = N / E;
  static_assert(G == 32, "one 1024-point line per warp");
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int LD = line_ld(N);
  const int warp = threadIdx.x >> 5, g = threadIdx.x & 31;
  const int Kzp = a.Kzp, Kz = a.Kz;
  C* base = sm + (size_t)warp * zr32_per_warp(LD, Kzp, PF);
  C* stg = base;
  C* buf = base + (PF ? (size_t)6 * Kzp : 0);
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const long long fs = a.nlines * Kzp;
  const C* in = reinterpret_cast<const C*>(a.in);
  C* out = reinterpret_cast<C*>(a.out);
  const long long wstride = (long long)gridDim.x * (blockDim.x >> 5);
  const long long wfirst = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
  auto stage = [&](long long ln) {
    if (!PF) return;
    if (ln < a.nlines) {
      const C* src = in + ln * Kzp;
#pragma unroll
      for (int f = 0; f < 6; ++f)
        for (int k = g * 2; k < Kzp; k += 64) cp_async16(stg + f * Kzp + k, src + f * fs + k);
    }
    cp_commit();
  };
  stage(wfirst);
  float rmax = 0.f;
  const float idx0 = (float)a.inv_dx[0], idx1 = (float)a.inv_dx[1], idx2 = (float)a.inv_dx[2];
  for (long long line = wfirst; line < a.nlines; line += wstride) {
    if (PF) cp_wait_all();
    __syncwarp();
    const C* rows = PF ? stg : in + line * Kzp;
    const long long rs = PF ? Kzp : fs;
#pragma unroll 1
    for (int p = 0; p < 3; ++p)
      pack_pair(buf + p * LD, rows + (2 * p) * rs, rows + (2 * p + 1) * rs, Kz, N, g, G, true);
    __syncwarp();
    stage(line + wstride);
#pragma unroll 1
    for (int p = 0; p < 3; ++p) line_fft_r32<N, 1, PR>(buf + p * LD, g, tw);
#pragma unroll 4
    for (int m = 0; m < E; ++m) {
      const int n = padp(g + G * m);
      const C c0 = buf[n], c1 = buf[LD + n], c2 = buf[2 * LD + n];
      const float u0 = c0.x, u1 = c0.y, u2 = c1.x, w0 = c1.y, w1 = c2.x, w2 = c2.y;
      if (a.cfl_rate) rmax = fmaxf(rmax, fabsf(u0) * idx0 + fabsf(u1) * idx1 + fabsf(u2) * idx2);
      buf[n] = make_float2(u1 * w2 - u2 * w1, u2 * w0 - u0 * w2);
      buf[LD + n] = make_float2(u0 * w1 - u1 * w0, 0.f);
    }
    __syncwarp();
    line_fft_r32<N, -1, false>(buf, g, tw);
    line_fft_r32<N, -1, false>(buf + LD, g, tw);
    const long long lo = line * Kzp;
    for (int kz = g; kz < Kzp; kz += G) {
      C oa = make_float2(0.f, 0.f), ob = oa, oc = oa;
      if (kz < Kz) {
        unpack_pair<C, float>(buf, kz, N, oa, ob);
        oc = buf[LD + padp(kz)];
      }
      out[lo + kz] = oa;
      out[fs + lo + kz] = ob;
      out[2 * fs + lo + kz] = oc;
    }
    __syncwarp();
  }
  if (PF) cp_wait_all();
  if (a.cfl_rate) {
    for (int o = 16; o > 0; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    const double rm = (double)rmax;
    if (g == 0 && rm > 0.0)
      atomicMax(reinterpret_cast<unsigned long long*>(a.cfl_rate), (unsigned long long)__double_as_longlong(rm));
  }
}

// complex values of shared memory per warp of k_zline_ns_t: LPW staging
// areas of 6 rows and LPW x 3 line buffers (kept even: 16-byte alignment)
__host__ __device__ inline size_t znsr_per_warp(int LD, int Kzp, int LPW) {
  const size_t n = (size_t)LPW * ((size_t)6 * Kzp + (size_t)3 * LD);
  return (n + 1) & ~(size_t)1;
}

// Same sweep with the line length fixed at compile time.  The three inverse
// transforms of a line run together (conj(fwd(conj(.))), one batched body
// of three interleaved chains sharing the twiddle loads), then u x w, then
// the two forward transforms together; the pack is folded into the first
// pass and the unpack done with warp shuffles.
template <typename Real, int N, bool PR>
__global__ void __launch_bounds__(64, 4) k_zline_ns_t(ZArgs a) {
  constexpr int E = 16, G = N / E, LPW = 32 / G;
  using C = typename cplx_of<Real>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int LD = line_ld(N);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G, g = lane % G;
  const int Kzp = a.Kzp, Kz = a.Kz;
  C* base = sm + (size_t)warp * znsr_per_warp(LD, Kzp, LPW);
  C* stg = base + (size_t)sub * 6 * Kzp;
  C* buf = base + (size_t)LPW * 6 * Kzp + (size_t)sub * 3 * LD;
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const long long fs = a.nlines * Kzp;
  const C* in = reinterpret_cast<const C*>(a.in);
  C* out = reinterpret_cast<C*>(a.out);
  const long long wstride = (long long)gridDim.x * (blockDim.x >> 5) * LPW;
  const long long wfirst = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * LPW;
  long long line = wfirst + sub;
  constexpr int VB = 16 / (int)sizeof(C);
  auto stage = [&](long long ln) {
    if (ln < a.nlines) {
      const C* src = in + ln * Kzp;
#pragma unroll
      for (int f = 0; f < 6; ++f)
        for (int k = g * VB; k < Kzp; k += G * VB) cp_async16(stg + f * Kzp + k, src + f * fs + k);
    }
    cp_commit();
  };
  stage(line);
  Real rmax = 0;  // CFL rate in the working precision (FP32: no FP64 arithmetic per point)
  const Real idx0 = (Real)a.inv_dx[0], idx1 = (Real)a.inv_dx[1], idx2 = (Real)a.inv_dx[2];
  const int src_lane = sub * G + ((G - g) & (G - 1));
  for (long long wl = wfirst; wl < a.nlines; wl += wstride, line += wstride) {
    const bool valid = line < a.nlines;
    cp_wait_all();
    __syncwarp();
    C U[3][E];
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      const C* ra = stg + (2 * p) * Kzp;
      const C* rb = stg + (2 * p + 1) * Kzp;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int P = g + G * m;
        C v = czero<C>();
        if (PR && pruned_r(m)) {  // kc < P < N - kc for every lane: zero (the first pass folds it away)
          U[p][m] = v;
          continue;
        }
        if (valid) {
          if (P < Kz) {
            C A = ra[P], B = rb[P];
            if (P == 0) { A.y = 0; B.y = 0; }
            v = mk<C>(A.x - B.y, A.y + B.x);
          } else if (N - P < Kz) {
            const C A = ra[N - P], B = rb[N - P];
            v = mk<C>(A.x + B.y, B.x - A.y);
          }
        }
        U[p][m] = cconj(v);  // inverse = conj(fwd(conj(.)))
      }
    }
    fwd_lines_regs<N, 3>(buf, LD, g, tw, U);
    __syncwarp();
    stage(line + wstride);
    // u x w in registers; conj(U0) = (ux, uy), conj(U1) = (uz, wx), conj(U2) = (wy, wz)
    C X[2][E];
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const Real u0 = U[0][m].x, u1 = -U[0][m].y, u2 = U[1][m].x, w0 = -U[1][m].y, w1 = U[2][m].x,
                 w2 = -U[2][m].y;
      if (a.cfl_rate && valid) rmax = fmax(rmax, fabs(u0) * idx0 + fabs(u1) * idx1 + fabs(u2) * idx2);
      X[0][m] = mk<C>(u1 * w2 - u2 * w1, u2 * w0 - u0 * w2);
      X[1][m] = mk<C>(u0 * w1 - u1 * w0, (Real)0);
    }
    fwd_lines_regs<N, 2>(buf, LD, g, tw, X);
    const long long lo = line * Kzp;
#pragma unroll
    for (int m = 0; m < E; ++m) {
      if (G * m >= Kzp) break;  // no lane stores from here on (warp-uniform)
      const C snd = (g == 0) ? X[0][(E - m) & (E - 1)] : X[0][E - 1 - m];
      C mir;
      mir.x = __shfl_sync(0xffffffffu, snd.x, src_lane);
      mir.y = __shfl_sync(0xffffffffu, snd.y, src_lane);
      const int kz = g + G * m;
      if (valid && kz < Kzp) {
        C oa = czero<C>(), ob = czero<C>(), oc = czero<C>();
        if (kz < Kz) {
          const C Xm = X[0][m];
          oa = mk<C>((Real)0.5 * (Xm.x + mir.x), (Real)0.5 * (Xm.y - mir.y));
          ob = mk<C>((Real)0.5 * (Xm.y + mir.y), (Real)0.5 * (mir.x - Xm.x));
          oc = X[1][m];
        }
        out[lo + kz] = oa;
        out[fs + lo + kz] = ob;
        out[2 * fs + lo + kz] = oc;
      }
    }
  }
  cp_wait_all();
  if (a.cfl_rate) {
    for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    const double rm = (double)rmax;
    if (lane == 0 && rm > 0.0)
      atomicMax(reinterpret_cast<unsigned long long*>(a.cfl_rate), (unsigned long long)__double_as_longlong(rm));
  }
}

// C2R-only (MODE 1) and R2C-only (MODE 2) z sweeps of the unpruned
// diagnostic transforms (not on the RK4 path).
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
  C* buf = sm + (size_t)((warp * LPW + sub) * 2) * LD;
  const C* tw = reinterpret_cast<const C*>(a.tw);
  const long long fs = a.nlines * a.Kzp;
  const long long lo = line * a.Kzp;
  const int npair = (a.nf + 1) / 2;
  const long long pfs = a.nlines * (long long)N;
  if (MODE == 1) {
    const C* in = reinterpret_cast<const C*>(a.in);
    for (int p = 0; p < npair; ++p) {
      const int fb = 2 * p + 1;
      pack_pair(buf + p * LD, in + (2 * p) * fs + lo, fb < a.nf ? in + fb * fs + lo : (const C*)nullptr, a.Kz, N, g,
                G, valid);
    }
    __syncwarp();
    for (int p = 0; p < npair; ++p) line_fft<E, +1>(buf + p * LD, g, N, tw);
    Real* ph = reinterpret_cast<Real*>(a.phys);
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
  const Real* ph = reinterpret_cast<const Real*>(a.phys);
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
  __syncwarp();
  for (int p = 0; p < npair; ++p) line_fft<E, -1>(buf + p * LD, g, N, tw);
  if (!valid) return;
  C* out = reinterpret_cast<C*>(a.out);
  for (int kz = g; kz < a.Kzp; kz += G) {
    for (int p = 0; p < npair; ++p) {
      const bool two = (2 * p + 1 < a.nf);
      C oa = czero<C>(), ob = czero<C>();
      if (kz < a.Kz) {
        if (two) unpack_pair<C, Real>(buf + p * LD, kz, N, oa, ob);
        else oa = buf[p * LD + padp(kz)];
      }
      out[(2 * p) * fs + lo + kz] = oa;
      if (two) out[(2 * p + 1) * fs + lo + kz] = ob;
    }
  }
}

// ---------------------------------------------------------------------------
// final x sweep + projection + diffusion + source + RK4 stage update.
// Single solver: right-hand side in FP32, S and A float-float (compensated);
// double solver: FP64 throughout.
// ---------------------------------------------------------------------------
template <typename Real, int E>
__global__ void __launch_bounds__(256, 2) k_axis_rk(RKArgs a) {
  using C = typename cplx_of<Real>::type;
  using AT = typename Acc<Real>::T;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int N = a.m0.n, G = N / E, W = blockDim.x / G, LD = line_ld(N);
  const int wsh = __ffs(W) - 1;
  C* sm = reinterpret_cast<C*>(smraw);
  int* ck1 = reinterpret_cast<int*>(sm + (size_t)3 * W * LD);
  int* ckz = ck1 + W;
  __shared__ double red[2][8];
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
  for (int i = tid; i < 3 * N * W; i += nth) {
    const int w = i & (W - 1), fr = i >> wsh, f = fr / N, r = fr - f * N;
    const long long l = l0 + w;
    if (l < nl) cp_async<sizeof(C)>(&sm[(f * W + w) * LD + padp(r)], in + ((long long)f * N + r) * nl + l);
  }
  cp_commit();
  cp_wait_all();
  __syncthreads();
  {
    const int lane = tid & 31, warp = tid >> 5;
    const int w = warp * (32 / G) + lane / G;
    const C* tw = reinterpret_cast<const C*>(a.tw);
    for (int f = 0; f < 3; ++f) {
      C* line = sm + (f * W + w) * LD;
      auto ld = [&](int p) -> C { return line[padp(p)]; };
      line_fft_ld<E, -1>(line, lane % G, N, tw, ld);
    }
  }
  __syncthreads();

  const int K0 = a.m0.rows();
  const long long cs = (long long)K0 * nl;  // component stride of the compact layout
  const double dt = *a.dt;
  const double alpha = a.force_alpha ? *a.force_alpha : 0.0;
  C* Y = reinterpret_cast<C*>(a.Y);
  AT* Sg = reinterpret_cast<AT*>(a.S);
  AT* Ag = reinterpret_cast<AT*>(a.A);
  const AT* src = reinterpret_cast<const AT*>(a.source);
  const Real sc = (Real)a.scale;
  const Real ks0 = (Real)a.kscale[0], ks1 = (Real)a.kscale[1], ks2 = (Real)a.kscale[2];
  const Real nu = (Real)a.nu;
  const Real bdt = (Real)(a.b * dt), adt = (Real)(a.a * dt), alph = (Real)alpha;
  const Real kf2 = (Real)a.kf2;
  double e_sum = 0.0, z_sum = 0.0;
  for (int i = tid; i < K0 * W; i += nth) {
    const int r = i >> wsh, w = i & (W - 1);
    const int k1row = ck1[w], kz = ckz[w];
    if (k1row < 0) continue;
    const long long o = (long long)r * nl + l0 + w;
    if (kz >= a.Kz) {  // padding of the R2C axis stays zero
      AT z0;
      memset(&z0, 0, sizeof(z0));
      for (int c = 0; c < 3; ++c) {
        if (a.stage == 4) {
          reinterpret_cast<C*>(a.rhs_out)[c * cs + o] = czero<C>();
        } else {
          Y[c * cs + o] = czero<C>();
          if (a.stage == 3) Sg[c * cs + o] = z0; else Ag[c * cs + o] = z0;
        }
      }
      if (a.p_out) reinterpret_cast<C*>(a.p_out)[o] = czero<C>();
      continue;
    }
    const int p = a.m0.pos(r);
    const Real k[3] = {ks0 * (Real)a.m0.wave(r), ks1 * (Real)a.m1.wave(k1row), ks2 * (Real)kz};
    const Real K2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    const Real iK2 = K2 > (Real)0 ? (Real)1 / K2 : (Real)0;
    C nlv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C v = sm[(c * W + w) * LD + padp(p)];
      nlv[c] = mk<C>(v.x * sc, v.y * sc);
    }
    const C P = mk<C>((nlv[0].x * k[0] + nlv[1].x * k[1] + nlv[2].x * k[2]) * iK2,
                      (nlv[0].y * k[0] + nlv[1].y * k[1] + nlv[2].y * k[2]) * iK2);
    if (a.p_out) reinterpret_cast<C*>(a.p_out)[o] = P;
    const bool forced = a.force_alpha && K2 > (Real)0 && K2 <= kf2;
    const Real nuK2 = nu * K2;
    Real snx[3] = {0, 0, 0}, sny[3] = {0, 0, 0};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long oc = c * cs + o;
      AT s, acc;
      memset(&s, 0, sizeof(s));
      C u;
      const bool need_s = a.stage == 0 || a.stage == 1 || a.stage == 2 || forced;
      if (need_s) s = Sg[oc];
      if (a.stage == 0) u = mk<C>((Real)s.x, (Real)s.y);
      else u = Y[oc];
      C rhs = mk<C>(nlv[c].x - P.x * k[c] - nuK2 * u.x, nlv[c].y - P.y * k[c] - nuK2 * u.y);
      if (src) { const AT q = src[oc]; rhs.x += (Real)q.x; rhs.y += (Real)q.y; }
      if (forced) { rhs.x += alph * (Real)s.x; rhs.y += alph * (Real)s.y; }
      if (a.stage == 4) {
        reinterpret_cast<C*>(a.rhs_out)[oc] = rhs;
        continue;
      }
      if constexpr (sizeof(Real) == 4) {
        // compensated FP32: Y' = S + b dt rhs ; A' = (S or A) + a dt rhs
        if (a.stage < 3) {
          float yx = s.x, ylx = s.z, yy = s.y, yly = s.w;
          ff_add(yx, ylx, bdt * rhs.x);
          ff_add(yy, yly, bdt * rhs.y);
          Y[oc] = mk<C>(yx, yy);
          if (a.stage == 0) acc = s; else acc = Ag[oc];
          ff_add(acc.x, acc.z, adt * rhs.x);
          ff_add(acc.y, acc.w, adt * rhs.y);
          Ag[oc] = acc;
        } else {
          acc = Ag[oc];
          ff_add(acc.x, acc.z, adt * rhs.x);
          ff_add(acc.y, acc.w, adt * rhs.y);
          Sg[oc] = acc;
          Y[oc] = mk<C>(acc.x, acc.y);
          snx[c] = acc.x;
          sny[c] = acc.y;
        }
      } else {
        const double bd = a.b * dt, ad = a.a * dt;
        if (a.stage < 3) {
          Y[oc] = mk<C>(s.x + bd * rhs.x, s.y + bd * rhs.y);
          if (a.stage == 0) acc = s; else acc = Ag[oc];
          acc.x += ad * rhs.x;
          acc.y += ad * rhs.y;
          Ag[oc] = acc;
        } else {
          acc = Ag[oc];
          acc.x += ad * rhs.x;
          acc.y += ad * rhs.y;
          Sg[oc] = acc;
          Y[oc] = mk<C>(acc.x, acc.y);
          snx[c] = (Real)acc.x;
          sny[c] = (Real)acc.y;
        }
      }
    }
    if (a.stage == 3) {
      const Real wz = (kz == 0) ? (Real)0.5 : (Real)1;  // 1/2 * Hermitian weight
      const Real e = snx[0] * snx[0] + sny[0] * sny[0] + snx[1] * snx[1] + sny[1] * sny[1] + snx[2] * snx[2] +
                     sny[2] * sny[2];
      const Real cxr = k[1] * snx[2] - k[2] * snx[1], cxi = k[1] * sny[2] - k[2] * sny[1];
      const Real cyr = k[2] * snx[0] - k[0] * snx[2], cyi = k[2] * sny[0] - k[0] * sny[2];
      const Real czr = k[0] * snx[1] - k[1] * snx[0], czi = k[0] * sny[1] - k[1] * sny[0];
      const Real z = cxr * cxr + cxi * cxi + cyr * cyr + cyi * cyi + czr * czr + czi * czi;
      e_sum += (double)(wz * e);
      z_sum += (double)(wz * z);
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
// Pointwise end of a stage after the x forward sweep (which wrote the scaled,
// masked nonlinear term in the compact layout to a.in): pressure projection,
// diffusion, source, forcing and the RK4 stage update, one thread per mode.
// Grid: x over b = k1row*Kzp + kz (blockDim.x modes per block), y over the
// compact rows of axis 0.  Stage 3 also writes per-block energy and
// enstrophy partial sums of the new state (block id y*gridDim.x + x).
// ---------------------------------------------------------------------------
// error-free sum of two float-float numbers (hi, lo) += (h2, l2)
__device__ __forceinline__ void ff_add2(float& hi, float& lo, float h2, float l2) {
  const float s = __fadd_rn(hi, h2);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
  const float t = __fadd_rn(__fadd_rn(e, lo), l2);
  hi = __fadd_rn(s, t);
  lo = __fsub_rn(t, __fsub_rn(hi, s));
}

// block sum of per-thread values; FP32 values are summed as float-float
// (compensated), FP64 values directly.  Valid in thread 0.
__device__ __forceinline__ double block_sum2(float x, float y, double* red, double& ys) {
  float xh = x, xl = 0.f, yh = y, yl = 0.f;
  for (int q = 16; q > 0; q >>= 1) {
    const float a0 = __shfl_xor_sync(0xffffffffu, xh, q), a1 = __shfl_xor_sync(0xffffffffu, xl, q);
    const float b0 = __shfl_xor_sync(0xffffffffu, yh, q), b1 = __shfl_xor_sync(0xffffffffu, yl, q);
    ff_add2(xh, xl, a0, a1);
    ff_add2(yh, yl, b0, b1);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[2 * warp] = (double)xh + (double)xl;
    red[2 * warp + 1] = (double)yh + (double)yl;
  }
  __syncthreads();
  double xs = 0;
  ys = 0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x + 31) / 32; ++q) { xs += red[2 * q]; ys += red[2 * q + 1]; }
  return xs;
}
__device__ __forceinline__ double block_sum2(double x, double y, double* red, double& ys) {
  for (int q = 16; q > 0; q >>= 1) {
    x += __shfl_xor_sync(0xffffffffu, x, q);
    y += __shfl_xor_sync(0xffffffffu, y, q);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { red[2 * warp] = x; red[2 * warp + 1] = y; }
  __syncthreads();
  double xs = 0;
  ys = 0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x + 31) / 32; ++q) { xs += red[2 * q]; ys += red[2 * q + 1]; }
  return xs;
}

template <typename Real, bool VV = false>
__global__ void __launch_bounds__(256) k_rk_update(RKArgs a) {
  using C = typename cplx_of<Real>::type;
  using AT = typename Acc<Real>::T;
  __shared__ double red[16];
  __shared__ Real coef[3];  // b dt, a dt, forcing alpha of this stage
  const int tid = threadIdx.x;
  if (tid == 0) {
    const double dt = *a.dt;
    coef[0] = (Real)(a.b * dt);
    coef[1] = (Real)(a.a * dt);
    coef[2] = (Real)(a.force_alpha ? *a.force_alpha : 0.0);
  }
  __syncthreads();
  const long long nl = a.nlines;
  const int r = blockIdx.y;
  const long long bi = (long long)blockIdx.x * blockDim.x + tid;
  const int K0 = a.m0.rows();
  const long long cs = (long long)K0 * nl;  // component stride of the compact layout
  const int stage = a.stage;
  Real e_sum = 0, z_sum = 0;
  if (bi < nl) {
    const int k1row = (int)((unsigned)bi / (unsigned)a.Kzp), kz = (int)bi - k1row * a.Kzp;
    const long long o = (long long)r * nl + bi;
    C* Y = reinterpret_cast<C*>(a.Y);
    AT* Sg = reinterpret_cast<AT*>(a.S);
    AT* Ag = reinterpret_cast<AT*>(a.A);
    const C* nlp = reinterpret_cast<const C*>(a.in);
    if (kz >= a.Kz) {  // padding of the R2C axis stays zero
      AT z0;
      memset(&z0, 0, sizeof(z0));
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (stage == 4) {
          reinterpret_cast<C*>(a.rhs_out)[c * cs + o] = czero<C>();
        } else {
          Y[c * cs + o] = czero<C>();
          if (stage == 3) Sg[c * cs + o] = z0; else Ag[c * cs + o] = z0;
        }
      }
      if (a.p_out) reinterpret_cast<C*>(a.p_out)[o] = czero<C>();
    } else {
      const Real bdt = coef[0], adt = coef[1], alph = coef[2];
      const Real k[3] = {(Real)a.kscale[0] * (Real)a.m0.wave(r), (Real)a.kscale[1] * (Real)a.m1.wave(k1row),
                         (Real)a.kscale[2] * (Real)kz};
      const Real K2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
      const bool forced = a.force_alpha && K2 > (Real)0 && K2 <= (Real)a.kf2;
      const bool need_s = stage <= 2 || forced;
      const bool need_a = stage >= 1 && stage <= 3;
      const AT* src = reinterpret_cast<const AT*>(a.source);
      // every load of this mode is issued before the first store
      C nlv[3], uv[3];
      AT sv[3], av[3], qv[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const long long oc = c * cs + o;
        nlv[c] = nlp[oc];
        memset(&sv[c], 0, sizeof(AT));
        memset(&av[c], 0, sizeof(AT));
        memset(&qv[c], 0, sizeof(AT));
        if (need_s) sv[c] = Sg[oc];
        if (need_a) av[c] = Ag[oc];
        if (stage != 0) uv[c] = Y[oc];
        if (src) qv[c] = src[oc];
      }
      const Real iK2 = K2 > (Real)0 ? (Real)1 / K2 : (Real)0;
      // convective term: NS projects the nonlinear term (NS.py:203-212), VV
      // takes its curl i K x nl (VV.py:103), component by component below
      C P = czero<C>();
      if constexpr (!VV) {
        P = mk<C>((nlv[0].x * k[0] + nlv[1].x * k[1] + nlv[2].x * k[2]) * iK2,
                  (nlv[0].y * k[0] + nlv[1].y * k[1] + nlv[2].y * k[2]) * iK2);
        if (a.p_out) reinterpret_cast<C*>(a.p_out)[o] = P;
      }
      const Real nuK2 = (Real)a.nu * K2;
      Real snx[3] = {0, 0, 0}, sny[3] = {0, 0, 0};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const long long oc = c * cs + o;
        const AT s = sv[c];
        AT acc = av[c];
        const C u = stage == 0 ? mk<C>((Real)s.x, (Real)s.y) : uv[c];
        C rhs;
        if constexpr (VV) {
          const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
          rhs = mk<C>(-(k[c1] * nlv[c2].y - k[c2] * nlv[c1].y) - nuK2 * u.x,
                      (k[c1] * nlv[c2].x - k[c2] * nlv[c1].x) - nuK2 * u.y);
        } else {
          rhs = mk<C>(nlv[c].x - P.x * k[c] - nuK2 * u.x, nlv[c].y - P.y * k[c] - nuK2 * u.y);
        }
        if (src) { rhs.x += (Real)qv[c].x; rhs.y += (Real)qv[c].y; }
        if (forced) { rhs.x += alph * (Real)s.x; rhs.y += alph * (Real)s.y; }
        if (stage == 4) {
          reinterpret_cast<C*>(a.rhs_out)[oc] = rhs;
          continue;
        }
        if (stage == 0) acc = s;
        if constexpr (sizeof(Real) == 4) {
          // compensated FP32: Y' = S + b dt rhs ; A' = (S or A) + a dt rhs
          if (stage < 3) {
            float yx = s.x, ylx = s.z, yy = s.y, yly = s.w;
            ff_add(yx, ylx, bdt * rhs.x);
            ff_add(yy, yly, bdt * rhs.y);
            Y[oc] = mk<C>(yx, yy);
            ff_add(acc.x, acc.z, adt * rhs.x);
            ff_add(acc.y, acc.w, adt * rhs.y);
            Ag[oc] = acc;
          } else {
            ff_add(acc.x, acc.z, adt * rhs.x);
            ff_add(acc.y, acc.w, adt * rhs.y);
            Sg[oc] = acc;
            Y[oc] = mk<C>(acc.x, acc.y);
            snx[c] = acc.x;
            sny[c] = acc.y;
          }
        } else {
          if (stage < 3) {
            Y[oc] = mk<C>(s.x + bdt * rhs.x, s.y + bdt * rhs.y);
            acc.x += adt * rhs.x;
            acc.y += adt * rhs.y;
            Ag[oc] = acc;
          } else {
            acc.x += adt * rhs.x;
            acc.y += adt * rhs.y;
            Sg[oc] = acc;
            Y[oc] = mk<C>(acc.x, acc.y);
            snx[c] = (Real)acc.x;
            sny[c] = (Real)acc.y;
          }
        }
      }
      if (stage == 3) {
        const Real wz = (kz == 0) ? (Real)0.5 : (Real)1;  // 1/2 * Hermitian weight
        const Real e = snx[0] * snx[0] + sny[0] * sny[0] + snx[1] * snx[1] + sny[1] * sny[1] + snx[2] * snx[2] +
                       sny[2] * sny[2];
        const Real cxr = k[1] * snx[2] - k[2] * snx[1], cxi = k[1] * sny[2] - k[2] * sny[1];
        const Real cyr = k[2] * snx[0] - k[0] * snx[2], cyi = k[2] * sny[0] - k[0] * sny[2];
        const Real czr = k[0] * snx[1] - k[1] * snx[0], czi = k[0] * sny[1] - k[1] * sny[0];
        const Real z = cxr * cxr + cxi * cxi + cyr * cyr + cyi * cyi + czr * czr + czi * czi;
        if constexpr (VV) {  // state w_hat: energy of i K x w_hat / K^2, enstrophy of w_hat
          e_sum = wz * z * iK2 * iK2;
          z_sum = wz * e;
        } else {
          e_sum = wz * e;
          z_sum = wz * z;
        }
      }
    }
  }
  if (stage == 3 && a.partials) {
    double zs;
    const double es = block_sum2(e_sum, z_sum, red, zs);
    if (tid == 0) {
      const long long blk = (long long)blockIdx.y * gridDim.x + blockIdx.x;
      a.partials[2 * blk] = es;
      a.partials[2 * blk + 1] = zs;
    }
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
inline int elems_for(int n) { return n >= 1024 ? 32 : 16; }

inline size_t smem_limit() {
  int dev = 0, mx = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return (size_t)mx - 1024;  // static shared memory of the kernels stays below 1 KB
}

template <typename Real, int N, int S>
static int launch_axis_p(const AxisArgs& a, cudaStream_t s) {
  using C = typename cplx_of<Real>::type;
  constexpr bool R32 = axis_r32<Real, N>::value;
  constexpr int G = N / (R32 ? 32 : axis_e<N>::value);
  const size_t lim = smem_limit();
  // 256 threads.  Radix-32 sweeps: 16-line tiles (128-byte rows at FP32 N = 512), one tile
  // buffer, two blocks per SM (measured faster than 8-line tiles double buffered, and than
  // 16-line tiles double buffered at one block per SM).  Others: double buffered.
  int W = 256 / G;
  const int nbuf = R32 ? 1 : 2;
  while (W > 2 && (size_t)nbuf * W * axis_ld(N, W, (int)sizeof(C)) * sizeof(C) > lim) W >>= 1;
  const size_t sm = (size_t)nbuf * W * axis_ld(N, W, (int)sizeof(C)) * sizeof(C);
  AxisArgs args = a;
  args.nbuf = nbuf;
  auto kern = k_axis_p<Real, N, S>;
  int dev = 0, nsm = 148, occ = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, W * G, sm);
  if (occ < 1) occ = 1;
  const long long ntask = (a.nlines + W - 1) / W * a.nfield;
  if (a.nlines * a.nfield >= (1LL << 31) || a.B < 1) return (int)cudaErrorInvalidValue;
  long long nb = (long long)occ * nsm;
  if (nb > ntask) nb = ntask;
  if (nb < 1) return 0;
  kern<<<(unsigned)nb, W * G, sm, s>>>(args);
  return (int)cudaGetLastError();
}

template <typename Real, int S>
static int axis_p_n(const AxisArgs& a, cudaStream_t s) {
  switch (a.min.n) {
    case 16: return launch_axis_p<Real, 16, S>(a, s);
    case 32: return launch_axis_p<Real, 32, S>(a, s);
    case 64: return launch_axis_p<Real, 64, S>(a, s);
    case 128: return launch_axis_p<Real, 128, S>(a, s);
    case 256: return launch_axis_p<Real, 256, S>(a, s);
    case 512: return launch_axis_p<Real, 512, S>(a, s);
    case 1024: return launch_axis_p<Real, 1024, S>(a, s);
    default: return (int)cudaErrorInvalidValue;
  }
}

template <typename Real>
int Kernels<Real>::axis_plain(const AxisArgs& a, int sign, cudaStream_t s) {
  return sign < 0 ? axis_p_n<Real, -1>(a, s) : axis_p_n<Real, 1>(a, s);
}

template <typename Real, int N>
static int launch_curl6(const AxisArgs& a, cudaStream_t s, bool vv) {
  using C = typename cplx_of<Real>::type;
  // the x sweep reads lines l at in + c*in_fs + l (one run of lines per field)
  if (a.B != a.nlines || a.in_ss != 0 || a.out_ss != 0 || a.nfield != 6 || (a.out_rs & 1)) return (int)cudaErrorInvalidValue;
  constexpr int G = N / axis_e<N>::value;
  const int cs = (int)sizeof(C), rin = a.min.rows();
  auto bytes = [&](int w) {
    return (size_t)w * ((size_t)3 * staged_rows(rin, w, cs) + axis_ld(N, w, cs)) * sizeof(C);
  };
  const size_t lim = smem_limit();
  int W = 512 / G;  // 16-line tiles at N = 512 (128-byte rows), halved while they do not fit
  while (W > 2 && bytes(W) > lim) W >>= 1;
  const size_t sm = bytes(W);
  if (vv) k_axis_curl6<Real, N, true><<<(unsigned)((a.nlines + W - 1) / W), W * G, sm, s>>>(a);
  else k_axis_curl6<Real, N, false><<<(unsigned)((a.nlines + W - 1) / W), W * G, sm, s>>>(a);
  return (int)cudaGetLastError();
}

template <typename Real>
int Kernels<Real>::axis_curl_inv(const AxisArgs& a, cudaStream_t s, bool vv) {
  switch (a.min.n) {
    case 16: return launch_curl6<Real, 16>(a, s, vv);
    case 32: return launch_curl6<Real, 32>(a, s, vv);
    case 64: return launch_curl6<Real, 64>(a, s, vv);
    case 128: return launch_curl6<Real, 128>(a, s, vv);
    case 256: return launch_curl6<Real, 256>(a, s, vv);
    case 512: return launch_curl6<Real, 512>(a, s, vv);
    case 1024: return launch_curl6<Real, 1024>(a, s, vv);
    default: return (int)cudaErrorInvalidValue;
  }
}

template <typename Real>
int Kernels<Real>::rk_update(const RKArgs& a, cudaStream_t s) {
  const dim3 grid((unsigned)((a.nlines + 255) / 256), (unsigned)a.m0.rows());
  if (a.vv) k_rk_update<Real, true><<<grid, 256, 0, s>>>(a);
  else k_rk_update<Real, false><<<grid, 256, 0, s>>>(a);
  return (int)cudaGetLastError();
}

template <typename Real, int E>
static int launch_zns(const ZArgs& a, cudaStream_t s) {
  using C = typename cplx_of<Real>::type;
  const int G = a.n / E, LPW = 32 / G;
  const int warps = 2;
  if (a.Kzp % 8 != 0) return (int)cudaErrorInvalidValue;  // 16-byte staging copies need Kzp % 8 == 0
  const size_t sm = (size_t)warps * zns_per_warp(line_ld(a.n), a.Kzp, LPW) * sizeof(C);
  auto kern = k_zline_ns<Real, E>;
  int dev = 0, nsm = 148, occ = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, warps * 32, sm);
  if (occ < 1) occ = 1;
  const long long per_block = (long long)warps * LPW;
  long long nb = (a.nlines + per_block - 1) / per_block;
  if (nb > (long long)occ * nsm) nb = (long long)occ * nsm;
  kern<<<(unsigned)nb, warps * 32, sm, s>>>(a);
  return (int)cudaGetLastError();
}

// The 1024-point z sweep reads its rows directly (PF false): 8 warps per SM
// instead of 4 with the staging area, 20.1 instead of 22.6 ms per 1024^3 launch.
constexpr bool kZr32Prefetch = false;

template <int N, bool PR>
static int launch_zns_r32(const ZArgs& a, cudaStream_t s) {
  constexpr int warps = 2;
  constexpr bool PF = kZr32Prefetch;
  if (a.n != N || a.Kzp % 8 != 0 || a.nf != 6) return (int)cudaErrorInvalidValue;
  const size_t sm = (size_t)warps * zr32_per_warp(line_ld(N), a.Kzp, PF) * sizeof(float2);
  auto kern = k_zline_ns_r32<N, PR, PF>;
  int dev = 0, nsm = 148, occ = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, warps * 32, sm);
  if (occ < 1) occ = 1;
  long long nb = (a.nlines + warps - 1) / warps;
  if (nb > (long long)occ * nsm) nb = (long long)occ * nsm;
  kern<<<(unsigned)nb, warps * 32, sm, s>>>(a);
  return (int)cudaGetLastError();
}

template <typename Real, int E, int MODE>
static int launch_z(const ZArgs& a, cudaStream_t s) {
  using C = typename cplx_of<Real>::type;
  const int G = a.n / E, LPW = 32 / G;
  const int warps = 4;
  const size_t sm = (size_t)warps * LPW * 2 * line_ld(a.n) * sizeof(C);
  auto kern = k_zline<Real, E, MODE>;
  const long long per_block = (long long)warps * LPW;
  dim3 grid((unsigned)((a.nlines + per_block - 1) / per_block));
  kern<<<grid, warps * 32, sm, s>>>(a);
  return (int)cudaGetLastError();
}

template <typename Real, int N, bool PR>
static int launch_zns_t(const ZArgs& a, cudaStream_t s) {
  using C = typename cplx_of<Real>::type;
  constexpr int G = N / 16, LPW = 32 / G;
  const int warps = 2;
  if (a.Kzp % 8 != 0 || a.n != N) return (int)cudaErrorInvalidValue;
  const size_t sm = (size_t)warps * znsr_per_warp(line_ld(N), a.Kzp, LPW) * sizeof(C);
  auto kern = k_zline_ns_t<Real, N, PR>;
  int dev = 0, nsm = 148, occ = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, warps * 32, sm);
  if (occ < 1) occ = 1;
  const long long per_block = (long long)warps * LPW;
  long long nb = (a.nlines + per_block - 1) / per_block;
  if (nb > (long long)occ * nsm) nb = (long long)occ * nsm;
  kern<<<(unsigned)nb, warps * 32, sm, s>>>(a);
  return (int)cudaGetLastError();
}

template <typename Real, bool PR>
static int zns_n(const ZArgs& a, cudaStream_t s) {
  switch (a.n) {
    case 16: return launch_zns_t<Real, 16, PR>(a, s);
    case 32: return launch_zns_t<Real, 32, PR>(a, s);
    case 64: return launch_zns_t<Real, 64, PR>(a, s);
    case 128: return launch_zns_t<Real, 128, PR>(a, s);
    case 256: return launch_zns_t<Real, 256, PR>(a, s);
    case 512: return launch_zns_t<Real, 512, PR>(a, s);
    case 1024:
      if constexpr (sizeof(Real) == 4) return launch_zns_r32<1024, PR>(a, s);
      else return launch_zns<Real, 32>(a, s);
    default: return launch_zns<Real, 32>(a, s);
  }
}
template <typename Real>
int Kernels<Real>::zline_ns(const ZArgs& a, cudaStream_t s) {
  return prunable(a.n, a.Kz - 1) ? zns_n<Real, true>(a, s) : zns_n<Real, false>(a, s);
}
template <typename Real>
int Kernels<Real>::zline_c2r(const ZArgs& a, cudaStream_t s) {
  return elems_for(a.n) == 16 ? launch_z<Real, 16, 1>(a, s) : launch_z<Real, 32, 1>(a, s);
}
template <typename Real>
int Kernels<Real>::zline_r2c(const ZArgs& a, cudaStream_t s) {
  return elems_for(a.n) == 16 ? launch_z<Real, 16, 2>(a, s) : launch_z<Real, 32, 2>(a, s);
}

// tile width (lines) of the RK sweep for an axis of n0 points
inline int rk_width(int n0, size_t csz) {
  const int E = elems_for(n0), G = n0 / E;
  int W = 256 / G;
  while (W > 1 && (size_t)3 * W * line_ld(n0) * csz + 2 * W * sizeof(int) + 16 > 200 * 1024) W /= 2;
  return W;
}

template <typename Real, int E>
static int launch_rk(const RKArgs& a, cudaStream_t s, int* nblocks) {
  using C = typename cplx_of<Real>::type;
  const int G = a.m0.n / E;
  const int W = rk_width(a.m0.n, sizeof(C));
  const size_t sm = (size_t)3 * W * line_ld(a.m0.n) * sizeof(C) + 2 * W * sizeof(int) + 16;
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

template <typename K> static cudaError_t optin_one(K kern, int optin) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

// Allow the large dynamic shared-memory tiles once per device (outside any
// stream capture).
template <typename Real>
int Kernels<Real>::smem_optin(int dev) {
  int mx = 0;
  cudaError_t e = cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
#define SDNS_OPT(k) if (e == cudaSuccess) e = optin_one(k, mx)
#define SDNS_OPT_N(n) SDNS_OPT((k_axis_p<Real, n, -1>)); SDNS_OPT((k_axis_p<Real, n, 1>)); \
  SDNS_OPT((k_axis_curl6<Real, n, false>)); SDNS_OPT((k_axis_curl6<Real, n, true>))
  SDNS_OPT_N(16); SDNS_OPT_N(32); SDNS_OPT_N(64); SDNS_OPT_N(128); SDNS_OPT_N(256); SDNS_OPT_N(512); SDNS_OPT_N(1024);
#undef SDNS_OPT_N
  SDNS_OPT((k_zline_ns<Real, 16>)); SDNS_OPT((k_zline_ns<Real, 32>));
  if constexpr (sizeof(Real) == 4) {
    SDNS_OPT((k_zline_ns_r32<1024, true, kZr32Prefetch>));
    SDNS_OPT((k_zline_ns_r32<1024, false, kZr32Prefetch>));
  }
#define SDNS_OPT_Z(n) SDNS_OPT((k_zline_ns_t<Real, n, true>)); SDNS_OPT((k_zline_ns_t<Real, n, false>))
  SDNS_OPT_Z(16); SDNS_OPT_Z(32); SDNS_OPT_Z(64); SDNS_OPT_Z(128); SDNS_OPT_Z(256); SDNS_OPT_Z(512);
#undef SDNS_OPT_Z
  SDNS_OPT((k_zline<Real, 16, 1>)); SDNS_OPT((k_zline<Real, 16, 2>));
  SDNS_OPT((k_zline<Real, 32, 1>)); SDNS_OPT((k_zline<Real, 32, 2>));
  SDNS_OPT((k_axis_rk<Real, 16>)); SDNS_OPT((k_axis_rk<Real, 32>));
#undef SDNS_OPT
  return (int)e;
}

}  // namespace sdns
