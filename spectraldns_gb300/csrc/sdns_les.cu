// Learned subgrid-stress closure for a coarse-grid LES (GB300, sm_103a).
//
// Not part of the reference solver: the closure of the benchmark's LES case.
// Pieces, all on device pointers and a caller stream:
//   * box filter of a fine velocity field (ratio r) -> coarse velocity and the
//     subgrid stress tau_ij = bar(u_i u_j) - bar(u_i) bar(u_j);
//   * spectral velocity gradients i k_j u_hat_i and the projected SGS force
//     -P(i k_j tau_hat_ij) (added to the LES right-hand side as a Source);
//   * a periodic 3x3x3 convolution layer on channels-last BF16 activations
//     with FP32 accumulation: forward (+bias, optional ReLU), backward data,
//     backward weights/bias;
//   * MSE loss gradient and an Adam step that refreshes the BF16 weights.
// The convolution works on 8x8x8 bricks of the periodic grid: the brick and
// its one-point halo are staged in shared memory, the 27 x CO x CI weights as
// well, and every thread accumulates two points x CO outputs in registers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/sdns_gb300.h"
#include "sdns_internal.h"

namespace {

typedef __nv_bfloat16 bf16;

inline unsigned nb(long long n, int bs = 256) {
  long long b = (n + bs - 1) / bs;
  if (b > 152LL * 32) b = 152LL * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// ---------------------------------------------------------------------------
// box filter: fine [3][N0][N1][N2] -> coarse ubar [3][n0][n1][n2] and tau
// channels-last [p][6] (xx, yy, zz, xy, xz, yz)
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_box_filter(const R* u, int N0, int N1, int N2, int r, float* ubar, float* tau) {
  const int n0 = N0 / r, n1 = N1 / r, n2 = N2 / r;
  const long long nc = (long long)n0 * n1 * n2;
  const long long fs = (long long)N0 * N1 * N2;
  const double inv = 1.0 / ((double)r * r * r);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nc; p += (long long)gridDim.x * blockDim.x) {
    const int i2 = (int)(p % n2), i1 = (int)((p / n2) % n1), i0 = (int)(p / ((long long)n2 * n1));
    double s[3] = {0, 0, 0}, q[6] = {0, 0, 0, 0, 0, 0};
    for (int a = 0; a < r; ++a)
      for (int b = 0; b < r; ++b) {
        const long long base = ((long long)(i0 * r + a) * N1 + (i1 * r + b)) * N2 + (long long)i2 * r;
        for (int c = 0; c < r; ++c) {
          const double x = (double)u[base + c], y = (double)u[fs + base + c], z = (double)u[2 * fs + base + c];
          s[0] += x; s[1] += y; s[2] += z;
          q[0] += x * x; q[1] += y * y; q[2] += z * z; q[3] += x * y; q[4] += x * z; q[5] += y * z;
        }
      }
    for (int i = 0; i < 3; ++i) s[i] *= inv;
    for (int i = 0; i < 6; ++i) q[i] *= inv;
    ubar[p] = (float)s[0];
    ubar[nc + p] = (float)s[1];
    ubar[2 * nc + p] = (float)s[2];
    tau[6 * p + 0] = (float)(q[0] - s[0] * s[0]);
    tau[6 * p + 1] = (float)(q[1] - s[1] * s[1]);
    tau[6 * p + 2] = (float)(q[2] - s[2] * s[2]);
    tau[6 * p + 3] = (float)(q[3] - s[0] * s[1]);
    tau[6 * p + 4] = (float)(q[4] - s[0] * s[2]);
    tau[6 * p + 5] = (float)(q[5] - s[1] * s[2]);
  }
}

// wave number of index p on an axis of n points (FFT order), R2C axis: kz = p
__device__ __forceinline__ double wnum(int p, int n) { return (double)(p < (n + 1) / 2 ? p : p - n); }

// spectral gradients: uhat [3][n0][n1][n2h] -> ghat [9][...] with ghat[3 i + j] = i k_j uhat_i
template <typename C>
__global__ void k_grad_hat(const C* uh, C* gh, int n0, int n1, int n2, double s0, double s1, double s2) {
  const int n2h = n2 / 2 + 1;
  const long long m = (long long)n0 * n1 * n2h;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < m; q += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(q % n2h), p1 = (int)((q / n2h) % n1), p0 = (int)(q / ((long long)n2h * n1));
    const double k[3] = {s0 * wnum(p0, n0), s1 * wnum(p1, n1), s2 * kz};
    for (int i = 0; i < 3; ++i) {
      const C u = uh[i * m + q];
      for (int j = 0; j < 3; ++j) {
        C o;
        o.x = (decltype(o.x))(-k[j] * u.y);
        o.y = (decltype(o.x))(k[j] * u.x);
        gh[(3 * i + j) * m + q] = o;
      }
    }
  }
}

// SGS force S_i = -i k_j tau_hat_ij, projected on k.S = 0; tau_hat [6][...] (xx yy zz xy xz yz)
template <typename C>
__global__ void k_sgs_force(const C* th, C* S, int n0, int n1, int n2, double s0, double s1, double s2, double scale) {
  const int n2h = n2 / 2 + 1;
  const long long m = (long long)n0 * n1 * n2h;
  const int idx[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < m; q += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(q % n2h), p1 = (int)((q / n2h) % n1), p0 = (int)(q / ((long long)n2h * n1));
    const double k[3] = {s0 * wnum(p0, n0), s1 * wnum(p1, n1), s2 * kz};
    double fr[3], fi[3];
    for (int i = 0; i < 3; ++i) {
      double ar = 0, ai = 0;
      for (int j = 0; j < 3; ++j) {
        const C t = th[idx[i][j] * m + q];
        ar += k[j] * t.x;
        ai += k[j] * t.y;
      }
      fr[i] = ai * scale;   // -i (ar + i ai) = ai - i ar
      fi[i] = -ar * scale;
    }
    const double K2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    if (K2 > 0) {
      const double pr = (fr[0] * k[0] + fr[1] * k[1] + fr[2] * k[2]) / K2;
      const double pi = (fi[0] * k[0] + fi[1] * k[1] + fi[2] * k[2]) / K2;
      for (int i = 0; i < 3; ++i) { fr[i] -= pr * k[i]; fi[i] -= pi * k[i]; }
    } else {
      for (int i = 0; i < 3; ++i) { fr[i] = 0; fi[i] = 0; }
    }
    for (int i = 0; i < 3; ++i) {
      C o;
      o.x = (decltype(o.x))fr[i];
      o.y = (decltype(o.x))fi[i];
      S[i * m + q] = o;
    }
  }
}

// planar f32 [nch][P] -> channels-last bf16 [P][cpad] with per-channel affine (x - mu) * isd
__global__ void k_pack_cl(const float* x, int nch, long long P, int cpad, const float* mu, const float* isd, bf16* y) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x)
    for (int c = 0; c < cpad; ++c)
      y[p * cpad + c] = __float2bfloat16_rn(c < nch ? (x[c * P + p] - mu[c]) * isd[c] : 0.f);
}

// channels-last f32 [P][cpad] (first nch) -> planar f32 [nch][P] with x * sd + mu
__global__ void k_unpack_cl(const float* y, int cpad, int nch, long long P, const float* mu, const float* sd, float* x) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x)
    for (int c = 0; c < nch; ++c) x[c * P + p] = y[p * cpad + c] * sd[c] + mu[c];
}

// ---------------------------------------------------------------------------
// periodic 3x3x3 convolution on channels-last activations, 8^3 bricks
// MODE 0 (forward):   y[p][o] = b[o] + sum_t sum_i W[t][o][i] x[p + d(t)][i]
// MODE 1 (bwd data):  y[p][o] = sum_t sum_i W[t][i][o] x[p - d(t)][i]   (x = upstream grad, o = input channel)
// d(t) = (t/9 - 1, (t/3)%3 - 1, t%3 - 1).  TIN: bf16 or float inputs; output f32 (+ optional bf16 ReLU copy)
// ---------------------------------------------------------------------------
constexpr int BR = 8;              // brick edge
constexpr int HB = BR + 2;         // with halo
constexpr int BP = BR * BR * BR;   // points per brick

template <typename TIN> __device__ __forceinline__ float tof(TIN v);
template <> __device__ __forceinline__ float tof<bf16>(bf16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ float tof<float>(float v) { return v; }

template <int CI, int CO, int MODE> struct ConvSmem {
  // staged inputs: BF16 activations (forward) or FP32 gradients (backward data);
  // weights in FP32 when everything fits in 200 KB, else BF16
  using SX = typename std::conditional<MODE == 1, float, bf16>::type;
  static constexpr size_t xbytes = (size_t)HB * HB * HB * CI * sizeof(SX);
  static constexpr bool wf32 = xbytes + (size_t)27 * CI * CO * 4 <= 200 * 1024;
  using SW = typename std::conditional<wf32, float, bf16>::type;
  static constexpr size_t bytes = xbytes + (size_t)27 * CI * CO * sizeof(SW);
};

__device__ __forceinline__ float ld(const float* p) { return *p; }
__device__ __forceinline__ float ld(const bf16* p) { return __bfloat162float(*p); }
template <typename T> __device__ __forceinline__ T st(float v);
template <> __device__ __forceinline__ float st<float>(float v) { return v; }
template <> __device__ __forceinline__ bf16 st<bf16>(float v) { return __float2bfloat16_rn(v); }

template <typename TIN, int CI, int CO, int MODE>
__global__ void __launch_bounds__(256) k_conv3(const TIN* __restrict__ x, const bf16* __restrict__ W,
                                               const float* __restrict__ bias, float* __restrict__ y,
                                               bf16* __restrict__ yact, int n0, int n1, int n2, int relu) {
  using SM = ConvSmem<CI, CO, MODE>;
  using SX = typename SM::SX;
  using SW = typename SM::SW;
  extern __shared__ __align__(16) unsigned char smraw[];
  SX* sx = reinterpret_cast<SX*>(smraw);                           // [HB^3][CI]
  SW* sw = reinterpret_cast<SW*>(smraw + SM::xbytes);              // [27][CI][CO]
  const int nbx = n2 / BR, nby = n1 / BR;
  const int bz = blockIdx.x % nbx, by = (blockIdx.x / nbx) % nby, bxx = blockIdx.x / (nbx * nby);
  const int o0 = bxx * BR, o1 = by * BR, o2 = bz * BR;
  for (int e = threadIdx.x; e < 27 * CI * CO; e += blockDim.x) {
    const int t = e / (CI * CO), rem = e % (CI * CO), i = rem / CO, o = rem % CO;
    float w;
    if (MODE == 0) w = __bfloat162float(W[(t * CO + o) * CI + i]);
    else w = __bfloat162float(W[(t * CI + i) * CO + o]);  // forward layer: CO_f = CI here, CI_f = CO here
    sw[e] = st<SW>(w);
  }
  for (int e = threadIdx.x; e < HB * HB * HB * CI; e += blockDim.x) {
    const int c = e % CI, hp = e / CI;
    const int h2 = hp % HB, h1 = (hp / HB) % HB, h0 = hp / (HB * HB);
    const int g0 = wrap(o0 + h0 - 1, n0), g1 = wrap(o1 + h1 - 1, n1), g2 = wrap(o2 + h2 - 1, n2);
    sx[e] = st<SX>(tof<TIN>(x[(((long long)g0 * n1 + g1) * n2 + g2) * CI + c]));
  }
  __syncthreads();
  for (int pp = threadIdx.x; pp < BP / 2; pp += blockDim.x) {
    const int pa = pp, pb = pp + BP / 2;
    const int a2 = pa % BR, a1 = (pa / BR) % BR, a0 = pa / (BR * BR);
    const int b2 = pb % BR, b1 = (pb / BR) % BR, b0 = pb / (BR * BR);
    float acc0[CO], acc1[CO];
#pragma unroll
    for (int o = 0; o < CO; ++o) {
      const float bo = (MODE == 0 && bias) ? bias[o] : 0.f;
      acc0[o] = bo;
      acc1[o] = bo;
    }
    for (int t = 0; t < 27; ++t) {
      int d0 = t / 9 - 1, d1 = (t / 3) % 3 - 1, d2 = t % 3 - 1;
      if (MODE == 1) { d0 = -d0; d1 = -d1; d2 = -d2; }
      const SX* xa = sx + (((a0 + 1 + d0) * HB + (a1 + 1 + d1)) * HB + (a2 + 1 + d2)) * CI;
      const SX* xb = sx + (((b0 + 1 + d0) * HB + (b1 + 1 + d1)) * HB + (b2 + 1 + d2)) * CI;
      const SW* wt = sw + t * CI * CO;
#pragma unroll 4
      for (int i = 0; i < CI; ++i) {
        const float va = ld(xa + i), vb = ld(xb + i);
        const SW* wi = wt + i * CO;
#pragma unroll
        for (int o = 0; o < CO; ++o) {
          const float w = ld(wi + o);
          acc0[o] = fmaf(w, va, acc0[o]);
          acc1[o] = fmaf(w, vb, acc1[o]);
        }
      }
    }
    const long long ga = (((long long)(o0 + a0) * n1 + (o1 + a1)) * n2 + (o2 + a2));
    const long long gb = (((long long)(o0 + b0) * n1 + (o1 + b1)) * n2 + (o2 + b2));
#pragma unroll
    for (int o = 0; o < CO; ++o) {
      y[ga * CO + o] = acc0[o];
      y[gb * CO + o] = acc1[o];
      if (yact) {
        yact[ga * CO + o] = __float2bfloat16_rn(relu ? fmaxf(acc0[o], 0.f) : acc0[o]);
        yact[gb * CO + o] = __float2bfloat16_rn(relu ? fmaxf(acc1[o], 0.f) : acc1[o]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Forward convolution on the tensor cores: an implicit GEMM per 8^3 brick,
// D[point][o] = b[o] + sum_t sum_i X[point + d(t)][i] W[t][o][i], with BF16
// mma.sync m16n8k16 and FP32 accumulation.  The brick's 10^3 halo (channels
// last) and all 27 x CO rows of CI weights are staged in shared memory with
// the 16-byte chunks of every row XOR-swizzled, so that the fragment loads of
// 8 consecutive rows hit distinct banks.  Each warp owns 4 M-tiles of 16
// points (two z-lines of 8) and all CO/8 N-tiles.
// ---------------------------------------------------------------------------
template <int CI> __device__ __forceinline__ int swz(int row) { return CI == 16 ? ((row >> 2) & 1) : ((row >> 1) & 3); }
// byte offset of element k (even) of row `row` in a swizzled [rows][CI] BF16 array
template <int CI> __device__ __forceinline__ int soff(int row, int k) {
  return row * (CI * 2) + (((k >> 3) ^ swz<CI>(row)) << 4) + ((k & 7) << 1);
}
__device__ __forceinline__ uint32_t lds32(const unsigned char* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
template <int CI, int CO> struct MmaSmem {
  static constexpr size_t xbytes = (size_t)HB * HB * HB * CI * 2;
  static constexpr size_t bytes = xbytes + (size_t)27 * CO * CI * 2;
};

template <int CI, int CO>
__global__ void __launch_bounds__(256) k_conv3_mma(const bf16* __restrict__ x, const bf16* __restrict__ W,
                                                   const float* __restrict__ bias, float* __restrict__ y,
                                                   bf16* __restrict__ yact, int n0, int n1, int n2, int relu) {
  static_assert(CI == 16 || CI == 32, "16 or 32 input channels");
  static_assert(CO % 8 == 0, "output channels in multiples of 8");
  constexpr int NCH = CI / 8, NT = CO / 8;
  extern __shared__ __align__(16) unsigned char smraw[];
  unsigned char* sx = smraw;                              // [HB^3][CI] swizzled
  unsigned char* sw = smraw + MmaSmem<CI, CO>::xbytes;    // [27*CO][CI] swizzled
  const int nbx = n2 / BR, nby = n1 / BR;
  const int bz = blockIdx.x % nbx, by = (blockIdx.x / nbx) % nby, bxx = blockIdx.x / (nbx * nby);
  const int o0 = bxx * BR, o1 = by * BR, o2 = bz * BR;
  for (int e = threadIdx.x; e < 27 * CO * NCH; e += blockDim.x) {
    const int R = e / NCH, c = e % NCH;
    *reinterpret_cast<uint4*>(sw + R * (CI * 2) + ((c ^ swz<CI>(R)) << 4)) = reinterpret_cast<const uint4*>(W)[e];
  }
  for (int e = threadIdx.x; e < HB * HB * HB * NCH; e += blockDim.x) {
    const int h = e / NCH, c = e % NCH;
    const int h2 = h % HB, h1 = (h / HB) % HB, h0 = h / (HB * HB);
    const int g0 = wrap(o0 + h0 - 1, n0), g1 = wrap(o1 + h1 - 1, n1), g2 = wrap(o2 + h2 - 1, n2);
    const uint4* src = reinterpret_cast<const uint4*>(x + (((long long)g0 * n1 + g1) * n2 + g2) * CI);
    *reinterpret_cast<uint4*>(sx + h * (CI * 2) + ((c ^ swz<CI>(h)) << 4)) = src[c];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gq = lane >> 2, tq = lane & 3;
  float acc[4][NT][4];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[m][nt][q] = 0.f;
#pragma unroll 1
  for (int t = 0; t < 27; ++t) {
    const int d0 = t / 9 - 1, d1 = (t / 3) % 3 - 1, d2 = t % 3 - 1;
#pragma unroll
    for (int kc = 0; kc < CI / 16; ++kc) {
      uint32_t bfr[NT][2];
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int R = t * CO + nt * 8 + gq;
        bfr[nt][0] = lds32(sw + soff<CI>(R, kc * 16 + 2 * tq));
        bfr[nt][1] = lds32(sw + soff<CI>(R, kc * 16 + 8 + 2 * tq));
      }
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int mt = warp * 4 + m;
        const int px = mt >> 2, py = 2 * (mt & 3);
        const int h = ((px + 1 + d0) * HB + (py + 1 + d1)) * HB + (gq + 1 + d2);  // point (px, py, gq)
        const int h8 = h + HB;                                                      // point (px, py + 1, gq)
        uint32_t a[4];
        a[0] = lds32(sx + soff<CI>(h, kc * 16 + 2 * tq));
        a[1] = lds32(sx + soff<CI>(h8, kc * 16 + 2 * tq));
        a[2] = lds32(sx + soff<CI>(h, kc * 16 + 8 + 2 * tq));
        a[3] = lds32(sx + soff<CI>(h8, kc * 16 + 8 + 2 * tq));
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) mma_bf16(acc[m][nt], a, bfr[nt]);
      }
    }
  }
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int mt = warp * 4 + m;
    const int px = mt >> 2, py = 2 * (mt & 3);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const long long p = ((long long)(o0 + px) * n1 + (o1 + py + half)) * n2 + (o2 + gq);
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int col = nt * 8 + 2 * tq;
        const float v0 = acc[m][nt][2 * half] + (bias ? bias[col] : 0.f);
        const float v1 = acc[m][nt][2 * half + 1] + (bias ? bias[col + 1] : 0.f);
        *reinterpret_cast<float2*>(y + p * CO + col) = make_float2(v0, v1);
        if (yact)
          *reinterpret_cast<__nv_bfloat162*>(yact + p * CO + col) =
              __floats2bfloat162_rn(relu ? fmaxf(v0, 0.f) : v0, relu ? fmaxf(v1, 0.f) : v1);
      }
    }
  }
}

// grad of the pre-activation: g_pre = g_post * (pre > 0) (relu) or g_post
__global__ void k_relu_bwd(const float* gpost, const float* pre, float* gpre, long long n, int relu) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    gpre[i] = (relu && pre[i] <= 0.f) ? 0.f : gpost[i];
}

// dW[t][o][i] += sum_p g[p][o] x[p + d(t)][i]; db[o] += sum_p g[p][o]   (one brick per block)
template <int CI, int CO>
__global__ void __launch_bounds__(256) k_conv3_wgrad(const bf16* __restrict__ x, const float* __restrict__ g,
                                                     float* __restrict__ dW, float* __restrict__ db, int n0, int n1,
                                                     int n2) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* sx = reinterpret_cast<float*>(smraw);   // [HB^3][CI]
  float* sg = sx + HB * HB * HB * CI;            // [BP][CO]
  const int nbx = n2 / BR, nby = n1 / BR;
  const int bz = blockIdx.x % nbx, by = (blockIdx.x / nbx) % nby, bxx = blockIdx.x / (nbx * nby);
  const int o0 = bxx * BR, o1 = by * BR, o2 = bz * BR;
  for (int e = threadIdx.x; e < HB * HB * HB * CI; e += blockDim.x) {
    const int c = e % CI, hp = e / CI;
    const int h2 = hp % HB, h1 = (hp / HB) % HB, h0 = hp / (HB * HB);
    const int g0 = wrap(o0 + h0 - 1, n0), g1 = wrap(o1 + h1 - 1, n1), g2 = wrap(o2 + h2 - 1, n2);
    sx[e] = __bfloat162float(x[(((long long)g0 * n1 + g1) * n2 + g2) * CI + c]);
  }
  for (int e = threadIdx.x; e < BP * CO; e += blockDim.x) {
    const int o = e % CO, p = e / CO;
    const int p2 = p % BR, p1 = (p / BR) % BR, p0 = p / (BR * BR);
    sg[e] = g[(((long long)(o0 + p0) * n1 + (o1 + p1)) * n2 + (o2 + p2)) * CO + o];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 27 * CO * CI; e += blockDim.x) {
    const int t = e / (CO * CI), o = (e / CI) % CO, i = e % CI;
    const int d0 = t / 9 - 1, d1 = (t / 3) % 3 - 1, d2 = t % 3 - 1;
    float acc = 0.f;
    for (int p = 0; p < BP; ++p) {
      const int p2 = p % BR, p1 = (p / BR) % BR, p0 = p / (BR * BR);
      acc = fmaf(sg[p * CO + o], sx[(((p0 + 1 + d0) * HB + (p1 + 1 + d1)) * HB + (p2 + 1 + d2)) * CI + i], acc);
    }
    atomicAdd(&dW[e], acc);
  }
  if (db) {
    for (int o = threadIdx.x; o < CO; o += blockDim.x) {
      float acc = 0.f;
      for (int p = 0; p < BP; ++p) acc += sg[p * CO + o];
      atomicAdd(&db[o], acc);
    }
  }
}

// mean-square loss over the first nch of cpad channels: grad = 2 (y - t) / (P nch), loss partials in FP64
__global__ void k_mse(const float* y, int cpad, int nch, const float* t, long long P, float* grad, double* loss) {
  __shared__ double red[32];
  double s = 0.0;
  const double inv = 1.0 / ((double)P * nch);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x)
    for (int c = 0; c < cpad; ++c) {
      float gv = 0.f;
      if (c < nch) {
        const float d = y[p * cpad + c] - t[p * nch + c];
        s += (double)d * d;
        gv = (float)(2.0 * d * inv);
      }
      grad[p * cpad + c] = gv;
    }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) a += red[w];
    atomicAdd(loss, a * inv);
  }
}

// Adam (Kingma & Ba): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2; w -= lr mhat / (sqrt(vhat) + eps)
__global__ void k_adam(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2, bf16* wb) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void k_to_bf16(const float* a, bf16* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16_rn(a[i]);
}

template <typename TIN, int CI, int CO, int MODE>
int launch_conv(const void* x, const void* W, const float* b, float* y, void* yact, const int n[3], int relu,
                cudaStream_t st) {
  const size_t sm = ConvSmem<CI, CO, MODE>::bytes;
  auto kern = k_conv3<TIN, CI, CO, MODE>;
  static bool opted = false;
  if (!opted) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    opted = true;
  }
  const int nblk = (n[0] / BR) * (n[1] / BR) * (n[2] / BR);
  kern<<<nblk, 256, sm, st>>>((const TIN*)x, (const bf16*)W, b, y, (bf16*)yact, n[0], n[1], n[2], relu);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

template <int CI, int CO>
int launch_conv_mma(const void* x, const void* W, const float* b, float* y, void* yact, const int n[3], int relu,
                    cudaStream_t st) {
  const size_t sm = MmaSmem<CI, CO>::bytes;
  auto kern = k_conv3_mma<CI, CO>;
  static bool opted = false;
  if (!opted) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    opted = true;
  }
  // 16-byte rows of the staged arrays: 16-byte aligned activations and weights
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(W)) & 15) return SDNS_EINVAL;
  const int nblk = (n[0] / BR) * (n[1] / BR) * (n[2] / BR);
  kern<<<nblk, 256, sm, st>>>((const bf16*)x, (const bf16*)W, b, y, (bf16*)yact, n[0], n[1], n[2], relu);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

template <int CI, int CO>
int launch_wgrad(const void* x, const float* g, float* dW, float* db, const int n[3], cudaStream_t st) {
  const size_t sm = (size_t)(HB * HB * HB * CI + BP * CO) * sizeof(float);
  auto kern = k_conv3_wgrad<CI, CO>;
  static bool opted = false;
  if (!opted) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    opted = true;
  }
  const int nblk = (n[0] / BR) * (n[1] / BR) * (n[2] / BR);
  kern<<<nblk, 256, sm, st>>>((const bf16*)x, g, dW, db, n[0], n[1], n[2]);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

bool grid_ok(const int n[3]) {
  for (int i = 0; i < 3; ++i)
    if (n[i] < BR || n[i] % BR != 0) return false;
  return true;
}

}  // namespace

extern "C" {

int sdns_les_box_filter(const void* u, int32_t precision, const int32_t* N, int32_t ratio, float* ubar, float* tau,
                        void* stream) {
  if (!u || !N || !ubar || !tau || ratio < 1) return SDNS_EINVAL;
  for (int i = 0; i < 3; ++i)
    if (N[i] % ratio != 0) return SDNS_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const long long nc = (long long)(N[0] / ratio) * (N[1] / ratio) * (N[2] / ratio);
  if (precision == SDNS_DOUBLE)
    k_box_filter<double><<<nb(nc), 256, 0, st>>>((const double*)u, N[0], N[1], N[2], ratio, ubar, tau);
  else
    k_box_filter<float><<<nb(nc), 256, 0, st>>>((const float*)u, N[0], N[1], N[2], ratio, ubar, tau);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

int sdns_les_grad_hat(const void* uhat, void* ghat, int32_t precision, const int32_t* n, const double* L,
                      void* stream) {
  if (!uhat || !ghat || !n || !L) return SDNS_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const long long m = (long long)n[0] * n[1] * (n[2] / 2 + 1);
  const double s0 = 2 * M_PI / L[0], s1 = 2 * M_PI / L[1], s2 = 2 * M_PI / L[2];
  if (precision == SDNS_DOUBLE)
    k_grad_hat<double2><<<nb(m), 256, 0, st>>>((const double2*)uhat, (double2*)ghat, n[0], n[1], n[2], s0, s1, s2);
  else
    k_grad_hat<float2><<<nb(m), 256, 0, st>>>((const float2*)uhat, (float2*)ghat, n[0], n[1], n[2], s0, s1, s2);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

int sdns_les_sgs_force(const void* tauhat, void* force, int32_t precision, const int32_t* n, const double* L,
                       double scale, void* stream) {
  if (!tauhat || !force || !n || !L) return SDNS_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const long long m = (long long)n[0] * n[1] * (n[2] / 2 + 1);
  const double s0 = 2 * M_PI / L[0], s1 = 2 * M_PI / L[1], s2 = 2 * M_PI / L[2];
  if (precision == SDNS_DOUBLE)
    k_sgs_force<double2><<<nb(m), 256, 0, st>>>((const double2*)tauhat, (double2*)force, n[0], n[1], n[2], s0, s1, s2,
                                               scale);
  else
    k_sgs_force<float2><<<nb(m), 256, 0, st>>>((const float2*)tauhat, (float2*)force, n[0], n[1], n[2], s0, s1, s2,
                                              scale);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

int sdns_les_pack(const float* x, int32_t nch, int64_t P, int32_t cpad, const float* mu, const float* isd, void* y,
                  void* stream) {
  if (!x || !y || !mu || !isd || nch > cpad) return SDNS_EINVAL;
  k_pack_cl<<<nb(P), 256, 0, (cudaStream_t)stream>>>(x, nch, P, cpad, mu, isd, (bf16*)y);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

int sdns_les_unpack(const float* y, int32_t cpad, int32_t nch, int64_t P, const float* mu, const float* sd, float* x,
                    void* stream) {
  if (!x || !y || !mu || !sd || nch > cpad) return SDNS_EINVAL;
  k_unpack_cl<<<nb(P), 256, 0, (cudaStream_t)stream>>>(y, cpad, nch, P, mu, sd, x);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

// layer shapes supported: (ci, co) in {(16,32), (32,32), (32,8)}
int sdns_conv3d_fwd(const void* x, const void* W, const float* b, float* y, void* yact, const int32_t* n, int32_t ci,
                    int32_t co, int32_t relu, void* stream) {
  if (!x || !W || !y || !n || !grid_ok(n)) return SDNS_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  if (ci == 16 && co == 32) return launch_conv_mma<16, 32>(x, W, b, y, yact, n, relu, st);
  if (ci == 32 && co == 32) return launch_conv_mma<32, 32>(x, W, b, y, yact, n, relu, st);
  if (ci == 32 && co == 8) return launch_conv_mma<32, 8>(x, W, b, y, yact, n, relu, st);
  return SDNS_EINVAL;
}

// gradient w.r.t. the layer input: g_in[p][ci] = sum_t sum_co W[t][co][ci] g_pre[p - d(t)][co]
int sdns_conv3d_bwd_data(const float* gpre, const void* W, float* gin, const int32_t* n, int32_t ci, int32_t co,
                         void* stream) {
  if (!gpre || !W || !gin || !n || !grid_ok(n)) return SDNS_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  if (ci == 32 && co == 32) return launch_conv<float, 32, 32, 1>(gpre, W, nullptr, gin, nullptr, n, 0, st);
  if (ci == 32 && co == 8) return launch_conv<float, 8, 32, 1>(gpre, W, nullptr, gin, nullptr, n, 0, st);
  if (ci == 16 && co == 32) return launch_conv<float, 32, 16, 1>(gpre, W, nullptr, gin, nullptr, n, 0, st);
  return SDNS_EINVAL;
}

int sdns_conv3d_bwd_weight(const void* x, const float* gpre, float* dW, float* db, const int32_t* n, int32_t ci,
                           int32_t co, void* stream) {
  if (!x || !gpre || !dW || !n || !grid_ok(n)) return SDNS_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  if (ci == 16 && co == 32) return launch_wgrad<16, 32>(x, gpre, dW, db, n, st);
  if (ci == 32 && co == 32) return launch_wgrad<32, 32>(x, gpre, dW, db, n, st);
  if (ci == 32 && co == 8) return launch_wgrad<32, 8>(x, gpre, dW, db, n, st);
  return SDNS_EINVAL;
}

int sdns_relu_bwd(const float* gpost, const float* pre, float* gpre, int64_t count, int32_t relu, void* stream) {
  if (!gpost || !pre || !gpre) return SDNS_EINVAL;
  k_relu_bwd<<<nb(count), 256, 0, (cudaStream_t)stream>>>(gpost, pre, gpre, count, relu);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

int sdns_mse_grad(const float* y, int32_t cpad, int32_t nch, const float* target, int64_t P, float* grad, double* loss,
                  void* stream) {
  if (!y || !target || !grad || !loss) return SDNS_EINVAL;
  k_mse<<<nb(P), 256, 0, (cudaStream_t)stream>>>(y, cpad, nch, target, P, grad, loss);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

int sdns_adam_step(float* w, const float* g, float* m, float* v, int64_t count, float lr, float b1, float b2,
                   float eps, int32_t step, void* wbf16, void* stream) {
  if (!w || !g || !m || !v || step < 1) return SDNS_EINVAL;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<nb(count), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, count, lr, b1, b2, eps, c1, c2, (bf16*)wbf16);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

int sdns_to_bf16(const float* a, void* b, int64_t count, void* stream) {
  if (!a || !b) return SDNS_EINVAL;
  k_to_bf16<<<nb(count), 256, 0, (cudaStream_t)stream>>>(a, (bf16*)b, count);
  return cudaGetLastError() == cudaSuccess ? SDNS_OK : SDNS_ECUDA;
}

}  // extern "C"
