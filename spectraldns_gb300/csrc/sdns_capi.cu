// C ABI of the GB300 Navier-Stokes backend: context management, boundary
// layout conversion, RK4 orchestration (CUDA graph per step) and float64
// diagnostics.  See include/sdns_gb300.h for the reference interfaces each
// entry point replaces.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/sdns_gb300.h"
#include "sdns_fft.cuh"
#include "sdns_internal.h"

using namespace sdns;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? SDNS_ENOMEM : SDNS_ECUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                    \
  } while (0)

#define CKL(expr)                                                                         \
  do {                                                                                    \
    int e_ = (expr);                                                                      \
    if (e_ != 0)                                                                          \
      return fail(SDNS_ECUDA, "kernel launch failed: %s (%s:%d)",                         \
                  cudaGetErrorString((cudaError_t)e_), __FILE__, __LINE__);               \
  } while (0)

inline long long rup(long long a, long long b) { return (a + b - 1) / b * b; }
inline bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

int cutoff(int n, int rule) {
  if (rule == SDNS_DEALIAS_NONE) return n / 2 - 1;
  const double kmax = 2.0 / 3.0 * (n / 2 + 1);
  int kc = (int)ceil(kmax) - 1;
  while (kc + 1 < kmax) ++kc;
  while (kc >= kmax) --kc;
  return kc;
}

enum { SC_DT = 0, SC_RATE = 1, SC_ALPHA = 2, SC_TIME = 3, SC_LASTRATE = 4, SC_ENERGY = 5, SC_ENSTROPHY = 6,
       SC_FLAG = 7, SC_COUNT = 16 };

}  // namespace

void sdns::set_last_error(const char* msg) { g_err = msg ? msg : ""; }

struct sdns_ctx {
  sdns_config cfg;
  int dev = 0;
  bool dbl = false;
  bool vv = false;           // velocity-vorticity formulation (state W_hat)
  size_t rsz = 4, csz = 8;  // real / complex element sizes of the working precision
  cudaStream_t st = nullptr;
  int N0, N1, N2, N2h;
  RowMap m0, m1, f0, f1;     // compact and full row maps of axes 0, 1
  int Kz, Kzp, Kzpf;         // compact kz count / pitch, full padded pitch
  long long K0, K1;
  long long ncomp1;          // one compact component: K0*K1*Kzp
  long long nfull1;          // one caller-layout spectral component: N0*N1*N2h
  long long npadf1;          // one padded full component: N0*N1*Kzpf
  long long nphys1;          // one physical component
  double kscale[3];
  // device buffers
  void* Y = nullptr;         // Real complex compact
  void* S = nullptr;         // compact step-start state, Acc<Real>::T (16 B per mode)
  void* A = nullptr;         // compact RK4 accumulator, Acc<Real>::T
  void* T1 = nullptr;        // [6][N0][K1][Kzp]
  void* T2 = nullptr;        // [6][N0][N1][Kzp]
  void* Pc = nullptr;        // compact P_hat
  void* Yx = nullptr;        // compact input of compute_rhs
  void* src = nullptr;       // compact source, Acc<Real>::T
  void* src_full = nullptr;  // caller-layout source (compute_rhs outside modes)
  void* H = nullptr;         // caller-layout modes outside the dealiased set
  bool high = false;
  void* F1 = nullptr;        // padded full [3][N0][N1][Kzpf]
  void* F2 = nullptr;
  void* PH = nullptr;        // physical [3][N0][N1][N2]
  void* stage = nullptr;     // caller-layout spectral staging [3][N0][N1][N2h]
  void* tw = nullptr;
  long long twoff[3] = {0, 0, 0};
  double* sc = nullptr;      // device scalars
  double* partials = nullptr;
  long long nblk_rk = 0;
  int* flag = nullptr;
  double* red = nullptr;     // per-block partial sums of sdns_error_norm
  // 3/2-rule contexts: caller-layout state and RK4 vectors, padded scratch
  bool pad32 = false;
  int M[3] = {0, 0, 0};
  void* U32 = nullptr;       // state [3][N0][N1][N2h]
  void* U32a = nullptr;      // RK4 u1
  void* U32b = nullptr;      // RK4 u2
  void* R32 = nullptr;       // rhs
  void* P32 = nullptr;       // P_hat of the last rhs (store_pressure)
  void* spec32 = nullptr;    // [6][M0][M1][M2h]
  void* phys32 = nullptr;    // [6][M0][M1][M2]
  void* tw32 = nullptr;      // W_{M_i}^j tables, one per axis
  long long twoff32[3] = {0, 0, 0};
  // host state
  double eps = 0, kf = 0, cfl = 0, last_dt = -1;
  bool has_state = false;
  bool timing = false;
  double tms[8] = {0};
  int tcount[8] = {0};
  std::vector<cudaEvent_t> evpool;  // timing mode: a start/stop pair per launch
  std::vector<int> evclass;
  size_t evused = 0;
  cudaGraphExec_t gexec = nullptr;
  unsigned long long gkey = ~0ull;
  int64_t bytes = 0;
};

namespace {

template <typename T> int dalloc(sdns_ctx* c, T** p, long long bytes) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, (size_t)bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SDNS_ENOMEM, "cudaMalloc(%lld bytes) failed: %s", bytes, cudaGetErrorString(e));
  }
  c->bytes += bytes;
  *p = reinterpret_cast<T*>(q);
  return SDNS_OK;
}

// ---------------------------------------------------------------------------
// boundary and reduction kernels
// ---------------------------------------------------------------------------
struct Geo {
  RowMap m0, m1;
  int N0, N1, N2h, Kz, Kzp, Kzpf;
  double ks[3];
  __device__ bool inside(int p0, int p1, int kz) const {
    auto in = [](const RowMap& m, int p) { return m.kc < 0 || p <= m.kc || p >= m.n - m.kc; };
    return in(m0, p0) && in(m1, p1) && kz < Kz;
  }
  __device__ int row(const RowMap& m, int p) const { return (m.kc < 0 || p <= m.kc) ? p : p - m.n + 2 * m.kc + 1; }
  __device__ double wave(int p, int n) const { return (double)(p < (n + 1) / 2 ? p : p - n); }
};

// caller layout [3][N0][N1][N2h] -> compact Y (Real) and S (FP64)
template <typename C>
__global__ void k_gather(const C* full, C* Y, void* Sv, Geo g, long long ncomp1) {
  using AC = Acc<decltype(C::x)>;
  typename AC::T* S = reinterpret_cast<typename AC::T*>(Sv);
  const long long n = 3 * ncomp1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long c = i / ncomp1;
    long long rem = i - c * ncomp1;
    const int kz = (int)(rem % g.Kzp);
    rem /= g.Kzp;
    const int r1 = (int)(rem % g.m1.rows());
    const int r0 = (int)(rem / g.m1.rows());
    C v;
    v.x = 0; v.y = 0;
    if (kz < g.Kz) {
      const long long fi = ((c * g.N0 + g.m0.pos(r0)) * g.N1 + g.m1.pos(r1)) * g.N2h + kz;
      v = full[fi];
    }
    if (Y) Y[i] = v;
    if (S) AC::put(S, i, (double)v.x, (double)v.y);
  }
}

// flag modes outside the dealiased set that are nonzero
template <typename C>
__global__ void k_outside(const C* full, Geo g, int* flag) {
  const long long n1 = (long long)g.N0 * g.N1 * g.N2h, n = 3 * n1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long rem = i % n1;
    const int kz = (int)(rem % g.N2h);
    rem /= g.N2h;
    const int p1 = (int)(rem % g.N1), p0 = (int)(rem / g.N1);
    if (!g.inside(p0, p1, kz)) {
      const C v = full[i];
      if (v.x != 0 || v.y != 0) atomicOr(flag, 1);
    }
  }
}

// compact (FP64 or Real) -> full layout with pitch `pitch` (N2h for the caller
// layout, Kzpf for the padded transform layout).  Outside modes: from
// `outside` (same layout as the caller array) or zero.  mult = 0: x1, 1: x(-i)
// comp_is_acc: the compact source is the accumulator format (S), else Real complex
template <typename C>
__global__ void k_scatter(const void* comp, int comp_is_acc, C* full, const C* outside, Geo g, int nf, int pitch,
                          long long ncomp1, int mult) {
  using AC = Acc<decltype(C::x)>;
  const long long n1 = (long long)g.N0 * g.N1 * pitch, n = nf * n1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long c = i / n1;
    long long rem = i - c * n1;
    const int kz = (int)(rem % pitch);
    rem /= pitch;
    const int p1 = (int)(rem % g.N1), p0 = (int)(rem / g.N1);
    C v;
    v.x = 0; v.y = 0;
    if (kz < g.N2h) {
      if (g.inside(p0, p1, kz)) {
        const long long ci = c * ncomp1 + ((long long)g.row(g.m0, p0) * g.m1.rows() + g.row(g.m1, p1)) * g.Kzp + kz;
        if (comp_is_acc) {
          const double2 s = AC::get(reinterpret_cast<const typename AC::T*>(comp), ci);
          v.x = (decltype(v.x))s.x;
          v.y = (decltype(v.x))s.y;
        } else {
          v = reinterpret_cast<const C*>(comp)[ci];
        }
      } else if (outside) {
        v = outside[((c * g.N0 + p0) * g.N1 + p1) * g.N2h + kz];
      }
      if (mult == 1) { const auto t = v.x; v.x = v.y; v.y = -t; }
    }
    full[i] = v;
  }
}

// ComputeRHS outside the dealiased set: rhs = -nu K^2 u_hat (+ Source)
template <typename C>
__global__ void k_rhs_outside(const C* uh, const C* srcf, C* rhs, Geo g, double nu) {
  const long long n1 = (long long)g.N0 * g.N1 * g.N2h, n = 3 * n1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long rem = i % n1;
    const int kz = (int)(rem % g.N2h);
    rem /= g.N2h;
    const int p1 = (int)(rem % g.N1), p0 = (int)(rem / g.N1);
    if (g.inside(p0, p1, kz)) continue;
    const double k0 = g.ks[0] * g.wave(p0, g.N0), k1 = g.ks[1] * g.wave(p1, g.N1), k2 = g.ks[2] * kz;
    const double z = nu * (k0 * k0 + k1 * k1 + k2 * k2);
    const C u = uh[i];
    C r;
    r.x = (decltype(r.x))(-z * u.x);
    r.y = (decltype(r.x))(-z * u.y);
    if (srcf) { r.x += srcf[i].x; r.y += srcf[i].y; }
    rhs[i] = r;
  }
}

// exact RK4 amplification of the pure-diffusion modes outside the set
template <typename C>
__global__ void k_decay_high(C* H, Geo g, double nu, const double* dt) {
  const long long n1 = (long long)g.N0 * g.N1 * g.N2h, n = 3 * n1;
  const double h = *dt;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long rem = i % n1;
    const int kz = (int)(rem % g.N2h);
    rem /= g.N2h;
    const int p1 = (int)(rem % g.N1), p0 = (int)(rem / g.N1);
    if (g.inside(p0, p1, kz)) continue;
    const double k0 = g.ks[0] * g.wave(p0, g.N0), k1 = g.ks[1] * g.wave(p1, g.N1), k2 = g.ks[2] * kz;
    const double z = -nu * (k0 * k0 + k1 * k1 + k2 * k2) * h;
    const double R = 1.0 + z * (1.0 + z * (0.5 + z * (1.0 / 6.0 + z * (1.0 / 24.0))));
    C v = H[i];
    v.x = (decltype(v.x))(v.x * R);
    v.y = (decltype(v.x))(v.y * R);
    H[i] = v;
  }
}

// caller layout (pitch N2h) <-> padded layout (pitch Kzpf)
template <typename C>
__global__ void k_repitch(const C* in, C* out, long long rows, int pin, int pout, int ncopy) {
  const long long n = rows * pout;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / pout;
    const int k = (int)(i - r * pout);
    C v;
    v.x = 0; v.y = 0;
    if (k < ncopy) v = in[r * pin + k];
    out[i] = v;
  }
}

// i K x u (mode 0, curl), i K . u (mode 1, divergence) or i K x u / K^2
// (mode 2, the velocity of the vorticity u, spectralDNS/solvers/VV.py:52-67;
// 0 at K = 0) on the padded full layout
template <typename C>
__global__ void k_curl_div(const C* u, C* out, Geo g, int div) {
  const long long n1 = (long long)g.N0 * g.N1 * g.Kzpf;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n1; i += (long long)gridDim.x * blockDim.x) {
    long long rem = i;
    const int kz = (int)(rem % g.Kzpf);
    rem /= g.Kzpf;
    const int p1 = (int)(rem % g.N1), p0 = (int)(rem / g.N1);
    const double k0 = g.ks[0] * g.wave(p0, g.N0), k1 = g.ks[1] * g.wave(p1, g.N1), k2 = g.ks[2] * kz;
    const C a = u[i], b = u[n1 + i], c = u[2 * n1 + i];
    typedef decltype(a.x) R;
    if (div == 1) {
      const double tr = k0 * a.x + k1 * b.x + k2 * c.x, ti = k0 * a.y + k1 * b.y + k2 * c.y;
      C o; o.x = (R)(-ti); o.y = (R)tr;
      out[i] = o;
    } else {
      double tr, ti;
      C o;
      const double K2 = k0 * k0 + k1 * k1 + k2 * k2;
      const double s = div == 2 ? (K2 > 0.0 ? 1.0 / K2 : 0.0) : 1.0;
      tr = s * (k1 * c.x - k2 * b.x); ti = s * (k1 * c.y - k2 * b.y); o.x = (R)(-ti); o.y = (R)tr; out[i] = o;
      tr = s * (k2 * a.x - k0 * c.x); ti = s * (k2 * a.y - k0 * c.y); o.x = (R)(-ti); o.y = (R)tr; out[n1 + i] = o;
      tr = s * (k0 * b.x - k1 * a.x); ti = s * (k0 * b.y - k1 * a.y); o.x = (R)(-ti); o.y = (R)tr; out[2 * n1 + i] = o;
    }
  }
}

// start of an RK4 step: reset the CFL maximum, forcing coefficient from S
template <typename Real>
__global__ void k_step_begin(const void* Sv, Geo g, long long ncomp1, double* sc, double eps, double kf2, int kfi0,
                             int kfi1, int kfi2) {
  const typename Acc<Real>::T* S = reinterpret_cast<const typename Acc<Real>::T*>(Sv);
  __shared__ double red[32];
  double e = 0.0;
  if (eps > 0.0) {
    const int n0 = 2 * kfi0 + 1, n1 = 2 * kfi1 + 1, n2 = kfi2 + 1;
    for (int i = threadIdx.x; i < n0 * n1 * n2; i += blockDim.x) {
      const int kz = i % n2, j1 = (i / n2) % n1 - kfi1, j0 = i / (n2 * n1) - kfi0;
      if (kz >= g.Kz || j0 < -g.m0.kc || j0 > g.m0.kc || j1 < -g.m1.kc || j1 > g.m1.kc) continue;
      const double k0 = g.ks[0] * j0, k1 = g.ks[1] * j1, k2 = g.ks[2] * kz;
      const double K2 = k0 * k0 + k1 * k1 + k2 * k2;
      if (K2 <= 0.0 || K2 > kf2) continue;
      const int r0 = j0 >= 0 ? j0 : j0 + 2 * g.m0.kc + 1, r1 = j1 >= 0 ? j1 : j1 + 2 * g.m1.kc + 1;
      const long long o = ((long long)r0 * g.m1.rows() + r1) * g.Kzp + kz;
      const double w = kz == 0 ? 0.5 : 1.0;
      for (int c = 0; c < 3; ++c) {
        const double2 v = Acc<Real>::get(S, c * ncomp1 + o);
        e += w * (v.x * v.x + v.y * v.y);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double Ef = 0.0;
    for (int q = 0; q < (int)(blockDim.x + 31) / 32; ++q) Ef += red[q];
    sc[SC_ALPHA] = (eps > 0.0 && Ef > 0.0) ? eps / (2.0 * Ef) : 0.0;
    sc[SC_RATE] = 0.0;
  }
}

__global__ void k_cfl_dt(double* sc, double cfl) {
  const double r = sc[SC_RATE];
  sc[SC_LASTRATE] = r;
  sc[SC_DT] = r > 0.0 ? cfl / r : 0.0;
}

// end of an RK4 step: deterministic sum of the per-CTA energy partials
__global__ void k_step_end(const double* partials, long long nb, double* sc) {
  __shared__ double red[2][32];
  double e = 0.0, z = 0.0;
  for (long long i = threadIdx.x; i < nb; i += blockDim.x) { e += partials[2 * i]; z += partials[2 * i + 1]; }
  for (int o = 16; o > 0; o >>= 1) { e += __shfl_xor_sync(0xffffffffu, e, o); z += __shfl_xor_sync(0xffffffffu, z, o); }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = e; red[1][threadIdx.x >> 5] = z; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double E = 0, Z = 0;
    for (int q = 0; q < (int)(blockDim.x + 31) / 32; ++q) { E += red[0][q]; Z += red[1][q]; }
    sc[SC_ENERGY] = E;
    sc[SC_ENSTROPHY] = Z;
    sc[SC_TIME] += sc[SC_DT];
    if (!(E == E) || E > 1e300) sc[SC_FLAG] = 1.0;
  }
}

// float64 sums over the compact state (+ outside modes in H): 1/2 sum |u|^2,
// 1/2 sum |K x u|^2, 1/2 sum |K.u|^2.  vv: the state is the vorticity w and the
// sums are 1/2 sum |u|^2, 1/2 sum |w|^2, 1/2 sum |K.u|^2 of u = i K x w / K^2.
__device__ inline void diag_mode(double k0, double k1, double k2, double2 a, double2 b, double2 c, double w, bool vv,
                                 double* s) {
  const double xr = k1 * c.x - k2 * b.x, xi = k1 * c.y - k2 * b.y;
  const double yr = k2 * a.x - k0 * c.x, yi = k2 * a.y - k0 * c.y;
  const double zr = k0 * b.x - k1 * a.x, zi = k0 * b.y - k1 * a.y;
  const double aa = a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y;
  const double xx = xr * xr + xi * xi + yr * yr + yi * yi + zr * zr + zi * zi;
  if (vv) {
    const double K2 = k0 * k0 + k1 * k1 + k2 * k2;
    const double iK2 = K2 > 0.0 ? 1.0 / K2 : 0.0;
    s[0] += w * xx * iK2 * iK2;
    s[1] += w * aa;
    // u = i (K x w) / K^2: K . u = 0 up to rounding
    const double dr = (k0 * xr + k1 * yr + k2 * zr) * iK2, di = (k0 * xi + k1 * yi + k2 * zi) * iK2;
    s[2] += w * (dr * dr + di * di);
  } else {
    s[0] += w * aa;
    s[1] += w * xx;
    const double dr = k0 * a.x + k1 * b.x + k2 * c.x, di = k0 * a.y + k1 * b.y + k2 * c.y;
    s[2] += w * (dr * dr + di * di);
  }
}

template <typename C>
__global__ void k_diag(const void* Sv, const C* H, Geo g, long long ncomp1, double* part, int vv) {
  using AC = Acc<decltype(C::x)>;
  const typename AC::T* S = reinterpret_cast<const typename AC::T*>(Sv);
  __shared__ double red[3][32];
  double s[3] = {0, 0, 0};
  const long long n1 = (long long)g.m0.rows() * g.m1.rows() * g.Kzp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n1; i += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(i % g.Kzp);
    if (kz >= g.Kz) continue;
    const int r1 = (int)((i / g.Kzp) % g.m1.rows()), r0 = (int)(i / ((long long)g.Kzp * g.m1.rows()));
    const double k0 = g.ks[0] * g.m0.wave(r0), k1 = g.ks[1] * g.m1.wave(r1), k2 = g.ks[2] * kz;
    const double2 a = AC::get(S, i), b = AC::get(S, ncomp1 + i), c = AC::get(S, 2 * ncomp1 + i);
    const double w = (kz == 0 || 2 * kz == 2 * (g.N2h - 1)) ? 0.5 : 1.0;
    diag_mode(k0, k1, k2, a, b, c, w, vv != 0, s);
  }
  if (H) {
    const long long f1 = (long long)g.N0 * g.N1 * g.N2h;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < f1; i += (long long)gridDim.x * blockDim.x) {
      const int kz = (int)(i % g.N2h);
      const int p1 = (int)((i / g.N2h) % g.N1), p0 = (int)(i / ((long long)g.N2h * g.N1));
      if (g.inside(p0, p1, kz)) continue;
      const double k0 = g.ks[0] * g.wave(p0, g.N0), k1 = g.ks[1] * g.wave(p1, g.N1), k2 = g.ks[2] * kz;
      const C a = H[i], b = H[f1 + i], c = H[2 * f1 + i];
      const double w = (kz == 0 || kz == g.N2h - 1) ? 0.5 : 1.0;
      diag_mode(k0, k1, k2, make_double2(a.x, a.y), make_double2(b.x, b.y), make_double2(c.x, c.y), w, vv != 0, s);
    }
  }
  for (int q = 0; q < 3; ++q)
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
  if ((threadIdx.x & 31) == 0)
    for (int q = 0; q < 3; ++q) red[q][threadIdx.x >> 5] = s[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < 3; ++q) {
      double t = 0;
      for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) t += red[q][w];
      part[3 * blockIdx.x + q] = t;
    }
  }
}

// |u|^2 of one mode: the state itself, or (vv) the velocity i K x w / K^2 of the vorticity state
__device__ inline double mode_u2(double k0, double k1, double k2, double2 a, double2 b, double2 c, int vv) {
  if (!vv) return a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y;
  const double xr = k1 * c.x - k2 * b.x, xi = k1 * c.y - k2 * b.y;
  const double yr = k2 * a.x - k0 * c.x, yi = k2 * a.y - k0 * c.y;
  const double zr = k0 * b.x - k1 * a.x, zi = k0 * b.y - k1 * a.y;
  const double K2 = k0 * k0 + k1 * k1 + k2 * k2;
  return K2 > 0.0 ? (xr * xr + xi * xi + yr * yr + yi * yi + zr * zr + zi * zi) / (K2 * K2) : 0.0;
}

// shell spectrum of demo/Isotropic.py:88-114: bin i collects i+0.5 < |K| <= i+1.5
template <typename C>
__global__ void k_spectrum(const void* Sv, const C* H, Geo g, long long ncomp1, double* sums, double* counts,
                           int nb, int vv) {
  using AC = Acc<decltype(C::x)>;
  const typename AC::T* S = reinterpret_cast<const typename AC::T*>(Sv);
  const long long n1 = (long long)g.m0.rows() * g.m1.rows() * g.Kzp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n1; i += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(i % g.Kzp);
    if (kz >= g.Kz) continue;
    const int r1 = (int)((i / g.Kzp) % g.m1.rows()), r0 = (int)(i / ((long long)g.Kzp * g.m1.rows()));
    const double k0 = g.ks[0] * g.m0.wave(r0), k1 = g.ks[1] * g.m1.wave(r1), k2 = g.ks[2] * kz;
    const double km = sqrt(k0 * k0 + k1 * k1 + k2 * k2);
    const int b = (int)ceil(km - 0.5) - 1;
    if (b < 0 || b > nb - 2) continue;
    const double2 a = AC::get(S, i), bb = AC::get(S, ncomp1 + i), c = AC::get(S, 2 * ncomp1 + i);
    const double w = (kz == 0) ? 1.0 : 2.0;
    atomicAdd(&sums[b], w * mode_u2(k0, k1, k2, a, bb, c, vv));
  }
  // the reference averages over every mode of the (N0, N1, N2/2+1) array in the shell
  const long long f1c = (long long)g.N0 * g.N1 * g.N2h;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < f1c; i += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(i % g.N2h);
    const int p1 = (int)((i / g.N2h) % g.N1), p0 = (int)(i / ((long long)g.N2h * g.N1));
    const double k0 = g.ks[0] * g.wave(p0, g.N0), k1 = g.ks[1] * g.wave(p1, g.N1), k2 = g.ks[2] * kz;
    const int b = (int)ceil(sqrt(k0 * k0 + k1 * k1 + k2 * k2) - 0.5) - 1;
    if (b >= 0 && b <= nb - 2) atomicAdd(&counts[b], 1.0);
  }
  if (H) {
    const long long f1 = (long long)g.N0 * g.N1 * g.N2h;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < f1; i += (long long)gridDim.x * blockDim.x) {
      const int kz = (int)(i % g.N2h);
      const int p1 = (int)((i / g.N2h) % g.N1), p0 = (int)(i / ((long long)g.N2h * g.N1));
      const double k0 = g.ks[0] * g.wave(p0, g.N0), k1 = g.ks[1] * g.wave(p1, g.N1), k2 = g.ks[2] * kz;
      const double km = sqrt(k0 * k0 + k1 * k1 + k2 * k2);
      const int b = (int)ceil(km - 0.5) - 1;
      if (b < 0 || b > nb - 2) continue;
      const bool in = g.inside(p0, p1, kz);
      const C a = H[i], bb = H[f1 + i], c = H[2 * f1 + i];
      const double w = (kz == 0 || kz == g.N2h - 1) ? 1.0 : 2.0;
      if (!in)
        atomicAdd(&sums[b], w * mode_u2(k0, k1, k2, make_double2(a.x, a.y), make_double2(bb.x, bb.y),
                                        make_double2(c.x, c.y), vv));
    }
  }
}

// ---------------------------------------------------------------------------
// integrator kernels: the linear combinations and the error estimate of the
// ForwardEuler, AB2 and embedded Runge-Kutta (BS5) steps of
// spectralDNS/maths/integrators.py:15-147, 161-175 on caller-layout vectors
// ---------------------------------------------------------------------------
struct LinTerms {
  const void* t[SDNS_LINCOMB_MAX];
  double c[SDNS_LINCOMB_MAX];
  int n;
};

// out = base + sum_k c_k t_k, accumulated term by term in the working
// precision (the order of the reference's `u += c*t` updates)
template <typename C>
__global__ void k_lincomb(C* out, const C* base, LinTerms lt, long long count) {
  using Real = decltype(C::x);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    Real x = 0, y = 0;
    if (base) {
      const C b = base[i];
      x = b.x;
      y = b.y;
    }
#pragma unroll
    for (int k = 0; k < SDNS_LINCOMB_MAX; ++k) {
      if (k < lt.n) {
        const C v = reinterpret_cast<const C*>(lt.t[k])[i];
        const Real ck = (Real)lt.c[k];
        x += ck * v.x;
        y += ck * v.y;
      }
    }
    out[i] = mk<C>(x, y);
  }
}

// per-block float64 sums over each of the 3 components of |err / sc|^2 with
// sc = atol + max(|u0|, |u1|) rtol (integrators.py:87-92)
template <typename C>
__global__ void __launch_bounds__(256) k_err_norm(const C* err, const C* u0, const C* u1, double atol, double rtol,
                                                  long long n1, double* part) {
  __shared__ double red[3][256];
  double s[3] = {0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 3 * n1; i += (long long)gridDim.x * blockDim.x) {
    const C e = err[i], a = u0[i], b = u1[i];
    const double ma = hypot((double)a.x, (double)a.y), mb = hypot((double)b.x, (double)b.y);
    const double sc = atol + fmax(ma, mb) * rtol;
    const double v = ((double)e.x * e.x + (double)e.y * e.y) / (sc * sc);
    const int q = (int)(i / n1);
    s[0] += q == 0 ? v : 0.0;
    s[1] += q == 1 ? v : 0.0;
    s[2] += q == 2 ? v : 0.0;
  }
  for (int q = 0; q < 3; ++q) red[q][threadIdx.x] = s[q];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) part[3 * blockIdx.x + q] = red[q][0];
}

// ---------------------------------------------------------------------------
// helpers on the context
// ---------------------------------------------------------------------------
Geo geo(const sdns_ctx* c) {
  Geo g;
  g.m0 = c->m0; g.m1 = c->m1;
  g.N0 = c->N0; g.N1 = c->N1; g.N2h = c->N2h;
  g.Kz = c->Kz; g.Kzp = c->Kzp; g.Kzpf = c->Kzpf;
  for (int i = 0; i < 3; ++i) g.ks[i] = c->kscale[i];
  return g;
}

// geometry and caller-layout array of the float64 reductions: the compact
// state plus the modes outside it (H), or, for a 3/2-rule context, the whole
// caller-layout state as "outside" modes of an empty compact set
Geo diag_geo(const sdns_ctx* c) {
  Geo g = geo(c);
  if (c->pad32) { g.Kz = 0; g.Kzp = 0; }
  return g;
}
const void* diag_full(const sdns_ctx* c) { return c->pad32 ? c->U32 : (c->high ? c->H : nullptr); }

inline unsigned nblocks(long long n, int bs = 256) {
  long long b = (n + bs - 1) / bs;
  if (b > 152LL * 32) b = 152LL * 32;
  if (b < 1) b = 1;
  return (unsigned)b;
}

const void* twp(const sdns_ctx* c, int axis) {
  return (const char*)c->tw + c->twoff[axis] * c->csz;
}

int ensure_full_bufs(sdns_ctx* c) {
  if (c->F1) return SDNS_OK;
  int e;
  if ((e = dalloc(c, &c->F1, 3 * c->npadf1 * (long long)c->csz))) return e;
  if ((e = dalloc(c, &c->F2, 3 * c->npadf1 * (long long)c->csz))) return e;
  if ((e = dalloc(c, &c->PH, 3 * c->nphys1 * (long long)c->rsz))) return e;
  return SDNS_OK;
}

int ensure_stage(sdns_ctx* c) {
  if (c->stage) return SDNS_OK;
  return dalloc(c, &c->stage, 3 * c->nfull1 * (long long)c->csz);
}

int copy_in(sdns_ctx* c, void* dst, const void* src, long long bytes, int where) {
  CK(cudaMemcpyAsync(dst, src, (size_t)bytes, where == SDNS_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                     c->st));
  return SDNS_OK;
}
int copy_out(sdns_ctx* c, void* dst, const void* src, long long bytes, int where) {
  CK(cudaMemcpyAsync(dst, src, (size_t)bytes, where == SDNS_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                     c->st));
  if (where == SDNS_HOST) CK(cudaStreamSynchronize(c->st));
  return SDNS_OK;
}

template <typename Real> int dispatch_axis(const AxisArgs& a, int sign, cudaStream_t s) {
  return Kernels<Real>::axis_plain(a, sign, s);
}

int axis_plain(sdns_ctx* c, const AxisArgs& a, int sign) {
  return c->dbl ? Kernels<double>::axis_plain(a, sign, c->st) : Kernels<float>::axis_plain(a, sign, c->st);
}

// ---- full (unpruned) 3D transforms on the padded layout -------------------
// inverse: F (padded full, nf fields) -> PH ; uses F1/F2 as ping-pong, input in `src`
int full_backward(sdns_ctx* c, void* src, void* tmp, int nf) {
  const long long Kp = c->Kzpf;
  AxisArgs a = {};
  // x: lines (N1*Kp), rows N0 stride N1*Kp
  a.in = src; a.out = tmp;
  a.min = c->f0; a.mout = c->f0;
  a.in_fs = a.out_fs = c->npadf1;
  a.in_ss = a.out_ss = 0;
  a.in_rs = a.out_rs = (long long)c->N1 * Kp;
  a.nlines = (long long)c->N1 * Kp; a.B = a.nlines; a.nfield = nf; a.scale = 1.0; a.tw = twp(c, 0);
  CKL(axis_plain(c, a, +1));
  // y: lines (N0*Kp), rows N1 stride Kp, slab x0 stride N1*Kp
  a.in = tmp; a.out = src;
  a.min = c->f1; a.mout = c->f1;
  a.in_rs = a.out_rs = Kp;
  a.in_ss = a.out_ss = (long long)c->N1 * Kp;
  a.nlines = (long long)c->N0 * Kp; a.B = Kp; a.tw = twp(c, 1);
  CKL(axis_plain(c, a, +1));
  ZArgs z = {};
  z.in = src; z.phys = c->PH; z.nlines = (long long)c->N0 * c->N1; z.n = c->N2; z.Kz = c->N2h; z.Kzp = c->Kzpf;
  z.nf = nf; z.tw = twp(c, 2);
  CKL(c->dbl ? Kernels<double>::zline_c2r(z, c->st) : Kernels<float>::zline_c2r(z, c->st));
  return SDNS_OK;
}

// forward: PH -> dst (padded full, scaled by 1/(N0 N1 N2)), tmp as scratch
int full_forward(sdns_ctx* c, void* dst, void* tmp, int nf) {
  const long long Kp = c->Kzpf;
  ZArgs z = {};
  z.out = dst; z.phys = c->PH; z.nlines = (long long)c->N0 * c->N1; z.n = c->N2; z.Kz = c->N2h; z.Kzp = Kp;
  z.nf = nf; z.tw = twp(c, 2);
  CKL(c->dbl ? Kernels<double>::zline_r2c(z, c->st) : Kernels<float>::zline_r2c(z, c->st));
  AxisArgs a = {};
  a.in = dst; a.out = tmp;
  a.min = c->f1; a.mout = c->f1;
  a.in_fs = a.out_fs = c->npadf1;
  a.in_rs = a.out_rs = Kp;
  a.in_ss = a.out_ss = (long long)c->N1 * Kp;
  a.nlines = (long long)c->N0 * Kp; a.B = Kp; a.nfield = nf; a.scale = 1.0; a.tw = twp(c, 1);
  CKL(axis_plain(c, a, -1));
  a.in = tmp; a.out = dst;
  a.min = c->f0; a.mout = c->f0;
  a.in_ss = a.out_ss = 0;
  a.in_rs = a.out_rs = (long long)c->N1 * Kp;
  a.nlines = (long long)c->N1 * Kp; a.B = a.nlines; a.tw = twp(c, 0);
  a.scale = 1.0 / ((double)c->N0 * c->N1 * c->N2);
  CKL(axis_plain(c, a, -1));
  return SDNS_OK;
}

template <typename C> int repitch(sdns_ctx* c, const void* in, void* out, int nf, int pin, int pout, int ncopy) {
  const long long rows = (long long)nf * c->N0 * c->N1;
  k_repitch<C><<<nblocks(rows * pout), 256, 0, c->st>>>((const C*)in, (C*)out, rows, pin, pout, ncopy);
  CK(cudaGetLastError());
  return SDNS_OK;
}
int repitch(sdns_ctx* c, const void* in, void* out, int nf, int pin, int pout, int ncopy) {
  return c->dbl ? repitch<double2>(c, in, out, nf, pin, pout, ncopy) : repitch<float2>(c, in, out, nf, pin, pout, ncopy);
}

// compact FP64 state (+H) -> padded full F (3 fields); a 3/2-rule context's
// state is already in the caller layout
int state_to_padded(sdns_ctx* c, void* F) {
  if (c->pad32) return repitch(c, c->U32, F, 3, c->N2h, c->Kzpf, c->N2h);
  Geo g = geo(c);
  if (c->dbl)
    k_scatter<double2><<<nblocks(3 * c->npadf1), 256, 0, c->st>>>(
        c->S, 1, (double2*)F, c->high ? (const double2*)c->H : nullptr, g, 3, c->Kzpf, c->ncomp1, 0);
  else
    k_scatter<float2><<<nblocks(3 * c->npadf1), 256, 0, c->st>>>(
        c->S, 1, (float2*)F, c->high ? (const float2*)c->H : nullptr, g, 3, c->Kzpf, c->ncomp1, 0);
  CK(cudaGetLastError());
  return SDNS_OK;
}

// ---- 3/2-rule contexts -------------------------------------------------------
Pad32 pad32_of(const sdns_ctx* c) {
  Pad32 p;
  for (int i = 0; i < 3; ++i) {
    p.N[i] = c->cfg.n[i];
    p.M[i] = c->M[i];
    p.ks[i] = c->kscale[i];
    p.tw[i] = (const char*)c->tw32 + c->twoff32[i] * c->csz;
  }
  p.nu = c->cfg.nu;
  p.dbl = c->dbl;
  p.vv = c->vv;
  p.spec = c->spec32;
  p.phys = c->phys32;
  return p;
}

int rhs32(sdns_ctx* c, const void* u, void* rhs, bool store_p) {
  CKL(pad32_rhs(pad32_of(c), u, c->src_full, rhs, store_p ? c->P32 : nullptr, c->st));
  return SDNS_OK;
}

__global__ void k_time_step(double* sc) { sc[SC_TIME] += sc[SC_DT]; }

// out = base + sum c_k t_k on caller-layout vectors (the lincomb kernel)
int lincomb_full(sdns_ctx* c, void* out, const void* base, int n, const double* coef, void* const* terms) {
  LinTerms lt = {};
  lt.n = n;
  for (int k = 0; k < n; ++k) { lt.t[k] = terms[k]; lt.c[k] = coef[k]; }
  const long long cnt = 3 * c->nfull1;
  if (c->dbl) k_lincomb<double2><<<nblocks(cnt), 256, 0, c->st>>>((double2*)out, (const double2*)base, lt, cnt);
  else k_lincomb<float2><<<nblocks(cnt), 256, 0, c->st>>>((float2*)out, (const float2*)base, lt, cnt);
  CK(cudaGetLastError());
  return SDNS_OK;
}

// classic RK4 (spectralDNS/maths/integrators.py:149-159) on the caller-layout
// state of a 3/2-rule context: u2 = u1 = u0; four stages; u0 = u2
int rk4_step32(sdns_ctx* c, double dt) {
  static const double ca[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
  static const double cb[3] = {0.5, 0.5, 1.0};
  const size_t fb = 3 * c->nfull1 * c->csz;
  CK(cudaMemcpyAsync(c->U32a, c->U32, fb, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(c->U32b, c->U32, fb, cudaMemcpyDeviceToDevice, c->st));
  int e;
  for (int rk = 0; rk < 4; ++rk) {
    if ((e = rhs32(c, c->U32, c->R32, rk == 3 && c->P32))) return e;
    void* t[1] = {c->R32};
    if (rk < 3) {
      const double cf = cb[rk] * dt;
      if ((e = lincomb_full(c, c->U32, c->U32a, 1, &cf, t))) return e;
    }
    const double cf2 = ca[rk] * dt;
    if ((e = lincomb_full(c, c->U32b, c->U32b, 1, &cf2, t))) return e;
  }
  CK(cudaMemcpyAsync(c->U32, c->U32b, fb, cudaMemcpyDeviceToDevice, c->st));
  k_time_step<<<1, 1, 0, c->st>>>(c->sc);
  CK(cudaGetLastError());
  return SDNS_OK;
}

// ---- one RK4 step ----------------------------------------------------------
int launch_stage_sweeps(sdns_ctx* c, const void* yin, int stage, bool cfl_rate, void* rhs_out, void* p_out) {
  const long long Kzp = c->Kzp, K1 = c->K1;
  cudaStream_t s = c->st;
  auto tstart = [&](int k) {
    if (!c->timing) return;
    if (c->evused + 2 > c->evpool.size()) {
      for (int q = 0; q < 64; ++q) { cudaEvent_t e; cudaEventCreate(&e); c->evpool.push_back(e); }
      c->evclass.resize(c->evpool.size() / 2);
    }
    c->evclass[c->evused / 2] = k;
    cudaEventRecord(c->evpool[c->evused], s);
  };
  auto tstop = [&](int) {
    if (!c->timing) return;
    cudaEventRecord(c->evpool[c->evused + 1], s);
    c->evused += 2;
  };
  // x^-1 with curl: Y [3][K0][K1][Kzp] -> T1 [6][N0][K1][Kzp]
  AxisArgs a = {};
  a.in = yin; a.out = c->T1;
  a.min = c->m0; a.mout = c->f0;
  a.in_fs = c->ncomp1; a.in_ss = 0; a.in_rs = K1 * Kzp;
  a.out_fs = (long long)c->N0 * K1 * Kzp; a.out_ss = 0; a.out_rs = K1 * Kzp;
  a.nlines = K1 * Kzp; a.B = a.nlines; a.nfield = 6; a.scale = 1.0; a.tw = twp(c, 0);
  for (int i = 0; i < 3; ++i) a.kscale[i] = c->kscale[i];
  a.m1 = c->m1; a.Kzp = (int)Kzp;
  tstart(0);
  CKL(c->dbl ? Kernels<double>::axis_curl_inv(a, s, c->vv) : Kernels<float>::axis_curl_inv(a, s, c->vv));
  tstop(0);
  // y^-1: T1 -> T2 [6][N0][N1][Kzp]
  AxisArgs b = {};
  b.in = c->T1; b.out = c->T2;
  b.min = c->m1; b.mout = c->f1;
  b.in_fs = (long long)c->N0 * K1 * Kzp; b.in_ss = K1 * Kzp; b.in_rs = Kzp;
  b.out_fs = (long long)c->N0 * c->N1 * Kzp; b.out_ss = (long long)c->N1 * Kzp; b.out_rs = Kzp;
  b.nlines = (long long)c->N0 * Kzp; b.B = Kzp; b.nfield = 6; b.scale = 1.0; b.tw = twp(c, 1);
  tstart(1);
  CKL(axis_plain(c, b, +1));
  tstop(1);
  // z: C2R x6, u x w, R2C x3 (in place into T2 fields 0..2)
  ZArgs z = {};
  z.in = c->T2; z.out = c->T2; z.nlines = (long long)c->N0 * c->N1; z.n = c->N2; z.Kz = c->Kz; z.Kzp = c->Kzp;
  z.nf = 6; z.tw = twp(c, 2);
  for (int i = 0; i < 3; ++i) z.inv_dx[i] = (double)c->cfg.n[i] / c->cfg.L[i];
  z.cfl_rate = cfl_rate ? c->sc + SC_RATE : nullptr;
  tstart(2);
  CKL(c->dbl ? Kernels<double>::zline_ns(z, s) : Kernels<float>::zline_ns(z, s));
  tstop(2);
  if (cfl_rate) {
    k_cfl_dt<<<1, 1, 0, s>>>(c->sc, c->cfl);
    CK(cudaGetLastError());
  }
  // y forward: T2 [3][N0][N1][Kzp] -> T1 [3][N0][K1][Kzp]
  AxisArgs d = {};
  d.in = c->T2; d.out = c->T1;
  d.min = c->f1; d.mout = c->m1;
  d.in_fs = (long long)c->N0 * c->N1 * Kzp; d.in_ss = (long long)c->N1 * Kzp; d.in_rs = Kzp;
  d.out_fs = (long long)c->N0 * K1 * Kzp; d.out_ss = K1 * Kzp; d.out_rs = Kzp;
  d.nlines = (long long)c->N0 * Kzp; d.B = Kzp; d.nfield = 3; d.scale = 1.0; d.tw = twp(c, 1);
  tstart(3);
  CKL(axis_plain(c, d, -1));
  tstop(3);
  // x forward: T1 [3][N0][K1][Kzp] -> scaled, masked nonlinear term in the
  // compact layout [3][K0][K1][Kzp], written into T2 (free after the y sweep)
  AxisArgs x = {};
  x.in = c->T1; x.out = c->T2;
  x.min = c->f0; x.mout = c->m0;
  x.in_fs = (long long)c->N0 * K1 * Kzp; x.in_ss = 0; x.in_rs = K1 * Kzp;
  x.out_fs = c->ncomp1; x.out_ss = 0; x.out_rs = K1 * Kzp;
  x.nlines = K1 * Kzp; x.B = x.nlines; x.nfield = 3; x.scale = 1.0 / ((double)c->N0 * c->N1 * c->N2);
  x.tw = twp(c, 0);
  tstart(4);
  CKL(axis_plain(c, x, -1));
  tstop(4);
  // projection + diffusion + source + forcing + RK4 stage update
  RKArgs r = {};
  r.in = c->T2; r.m0 = c->m0; r.m1 = c->m1; r.Kz = c->Kz; r.Kzp = c->Kzp; r.nlines = K1 * Kzp;
  r.scale = 1.0 / ((double)c->N0 * c->N1 * c->N2); r.tw = twp(c, 0);
  for (int i = 0; i < 3; ++i) r.kscale[i] = c->kscale[i];
  r.nu = c->cfg.nu; r.stage = stage;
  static const double ca[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
  static const double cb[4] = {0.5, 0.5, 1.0, 0.0};
  r.a = stage < 4 ? ca[stage] : 0.0; r.b = stage < 4 ? cb[stage] : 0.0;
  r.dt = c->sc + SC_DT;
  r.Y = stage < 4 ? c->Y : nullptr;
  r.S = c->S; r.A = c->A;
  r.rhs_out = rhs_out; r.p_out = p_out;
  if (stage == 4) r.Y = const_cast<void*>(yin);
  r.source = c->src;
  r.force_alpha = (c->eps > 0 && stage < 4) ? c->sc + SC_ALPHA : nullptr;
  r.kf2 = c->kf * c->kf;
  r.partials = c->partials;
  r.vv = c->vv ? 1 : 0;
  if (c->vv) r.p_out = nullptr;
  tstart(5);
  CKL(c->dbl ? Kernels<double>::rk_update(r, s) : Kernels<float>::rk_update(r, s));
  tstop(5);
  return SDNS_OK;
}

int launch_step(sdns_ctx* c) {
  Geo g = geo(c);
  const double L0 = c->cfg.L[0], L1 = c->cfg.L[1], L2 = c->cfg.L[2];
  const int kfi0 = (int)floor(c->kf * L0 / (2 * M_PI)) + 1, kfi1 = (int)floor(c->kf * L1 / (2 * M_PI)) + 1,
            kfi2 = (int)floor(c->kf * L2 / (2 * M_PI)) + 1;
  if (c->dbl)
    k_step_begin<double><<<1, 256, 0, c->st>>>(c->S, g, c->ncomp1, c->sc, c->eps, c->kf * c->kf, kfi0, kfi1, kfi2);
  else
    k_step_begin<float><<<1, 256, 0, c->st>>>(c->S, g, c->ncomp1, c->sc, c->eps, c->kf * c->kf, kfi0, kfi1, kfi2);
  CK(cudaGetLastError());
  for (int rk = 0; rk < 4; ++rk) {
    int e = launch_stage_sweeps(c, c->Y, rk, rk == 0 && c->cfl > 0, nullptr,
                                (rk == 3 && c->cfg.store_pressure) ? c->Pc : nullptr);
    if (e) return e;
  }
  k_step_end<<<1, 256, 0, c->st>>>(c->partials, c->nblk_rk, c->sc);
  CK(cudaGetLastError());
  if (c->high) {
    if (c->dbl)
      k_decay_high<double2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>((double2*)c->H, g, c->cfg.nu, c->sc + SC_DT);
    else
      k_decay_high<float2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>((float2*)c->H, g, c->cfg.nu, c->sc + SC_DT);
    CK(cudaGetLastError());
  }
  return SDNS_OK;
}

int check_ctx(sdns_ctx* c) {
  if (!c) return fail(SDNS_EINVAL, "null context");
  CK(cudaSetDevice(c->dev));
  return SDNS_OK;
}

}  // namespace

// ===========================================================================
// public entry points
// ===========================================================================
extern "C" {

int sdns_abi_version(void) { return SDNS_ABI_VERSION; }
const char* sdns_last_error(void) { return g_err.c_str(); }

int sdns_create(const sdns_config* cfg, sdns_ctx** out) {
  if (!cfg || !out) return fail(SDNS_EINVAL, "null argument");
  *out = nullptr;
  for (int i = 0; i < 3; ++i) {
    if (!pow2(cfg->n[i]) || cfg->n[i] < 16 || cfg->n[i] > 1024)
      return fail(SDNS_EINVAL, "n[%d]=%d: grid sizes must be powers of two in [16, 1024]", i, cfg->n[i]);
    if (!(cfg->L[i] > 0)) return fail(SDNS_EINVAL, "L[%d] must be positive", i);
  }
  if (cfg->precision != SDNS_SINGLE && cfg->precision != SDNS_DOUBLE)
    return fail(SDNS_EINVAL, "precision must be SDNS_SINGLE or SDNS_DOUBLE");
  if (cfg->dealias != SDNS_DEALIAS_23 && cfg->dealias != SDNS_DEALIAS_NONE && cfg->dealias != SDNS_DEALIAS_32)
    return fail(SDNS_EINVAL, "dealias must be SDNS_DEALIAS_23, SDNS_DEALIAS_NONE or SDNS_DEALIAS_32");
  if (cfg->formulation != SDNS_NS && cfg->formulation != SDNS_VV)
    return fail(SDNS_EINVAL, "formulation must be SDNS_NS or SDNS_VV");
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(SDNS_ECUDA, "no CUDA device available (%s)", cudaGetErrorString(ce));
  }
  if (cfg->device < 0 || cfg->device >= ndev) return fail(SDNS_EINVAL, "device %d out of range", cfg->device);
  sdns_ctx* c = new sdns_ctx();
  c->cfg = *cfg;
  c->dev = cfg->device;
  c->dbl = cfg->precision == SDNS_DOUBLE;
  c->vv = cfg->formulation == SDNS_VV;
  c->pad32 = cfg->dealias == SDNS_DEALIAS_32;
  c->rsz = c->dbl ? 8 : 4;
  c->csz = 2 * c->rsz;
  c->N0 = cfg->n[0]; c->N1 = cfg->n[1]; c->N2 = cfg->n[2]; c->N2h = c->N2 / 2 + 1;
  c->m0 = {c->N0, cutoff(c->N0, cfg->dealias)};
  c->m1 = {c->N1, cutoff(c->N1, cfg->dealias)};
  c->f0 = {c->N0, -1};
  c->f1 = {c->N1, -1};
  c->Kz = cutoff(c->N2, cfg->dealias) + 1;
  c->Kzp = (int)rup(c->Kz, 8);
  c->Kzpf = (int)rup(c->N2h, 8);
  c->K0 = c->m0.rows(); c->K1 = c->m1.rows();
  c->ncomp1 = c->K0 * c->K1 * c->Kzp;
  c->nfull1 = (long long)c->N0 * c->N1 * c->N2h;
  c->npadf1 = (long long)c->N0 * c->N1 * c->Kzpf;
  c->nphys1 = (long long)c->N0 * c->N1 * c->N2;
  for (int i = 0; i < 3; ++i) c->kscale[i] = 2.0 * M_PI / cfg->L[i];
  int e = SDNS_OK;
  auto bail = [&](int code) { sdns_destroy(c); return code; };
  if (cudaSetDevice(c->dev) != cudaSuccess) { cudaGetLastError(); return bail(fail(SDNS_ECUDA, "cudaSetDevice failed")); }
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(SDNS_ECUDA, "cudaStreamCreate failed"));
  {
    const int oe = c->dbl ? Kernels<double>::smem_optin(c->dev) : Kernels<float>::smem_optin(c->dev);
    if (oe != 0) return bail(fail(SDNS_ECUDA, "shared-memory opt-in failed: %s", cudaGetErrorString((cudaError_t)oe)));
  }
  const long long cb = (long long)c->csz;
  if (c->pad32) {
    // 3/2 rule: caller-layout state and RK4 vectors, padded scratch of M = 3N/2 per axis
    for (int i = 0; i < 3; ++i) c->M[i] = 3 * cfg->n[i] / 2;
    const long long f3 = 3 * c->nfull1 * cb;
    const long long nm = (long long)c->M[0] * c->M[1] * (c->M[2] / 2 + 1);
    const long long np = (long long)c->M[0] * c->M[1] * c->M[2];
    if ((e = dalloc(c, &c->U32, f3))) return bail(e);
    if ((e = dalloc(c, &c->U32a, f3))) return bail(e);
    if ((e = dalloc(c, &c->U32b, f3))) return bail(e);
    if ((e = dalloc(c, &c->R32, f3))) return bail(e);
    if ((e = dalloc(c, &c->spec32, 6 * nm * cb))) return bail(e);
    if ((e = dalloc(c, &c->phys32, 6 * np * (long long)c->rsz))) return bail(e);
    if (cfg->store_pressure && !c->vv && (e = dalloc(c, &c->P32, c->nfull1 * cb))) return bail(e);
    const int oe = pad32_smem_optin(c->dev, c->dbl);
    if (oe != 0) return bail(fail(SDNS_ECUDA, "shared-memory opt-in failed: %s", cudaGetErrorString((cudaError_t)oe)));
    long long tot = 0;
    for (int i = 0; i < 3; ++i) { c->twoff32[i] = tot; tot += c->M[i]; }
    std::vector<double> h(2 * tot);
    for (int i = 0; i < 3; ++i)
      for (int q = 0; q < c->M[i]; ++q) {
        const double ang = -2.0 * M_PI * (double)q / (double)c->M[i];
        h[2 * (c->twoff32[i] + q)] = cos(ang);
        h[2 * (c->twoff32[i] + q) + 1] = sin(ang);
      }
    if ((e = dalloc(c, &c->tw32, tot * cb))) return bail(e);
    std::vector<float> hf(2 * tot);
    for (long long q = 0; q < 2 * tot; ++q) hf[q] = (float)h[q];
    if (cudaMemcpy(c->tw32, c->dbl ? (const void*)h.data() : (const void*)hf.data(), tot * cb, cudaMemcpyHostToDevice) !=
        cudaSuccess)
      return bail(fail(SDNS_ECUDA, "twiddle upload failed"));
    if (cudaMemset(c->U32, 0, f3) != cudaSuccess) return bail(fail(SDNS_ECUDA, "memset failed"));
  } else {
    if ((e = dalloc(c, &c->Y, 3 * c->ncomp1 * cb))) return bail(e);
    if ((e = dalloc(c, &c->S, 3 * c->ncomp1 * 16))) return bail(e);
    if ((e = dalloc(c, &c->A, 3 * c->ncomp1 * 16))) return bail(e);
    if ((e = dalloc(c, &c->T1, 6LL * c->N0 * c->K1 * c->Kzp * cb))) return bail(e);
    if ((e = dalloc(c, &c->T2, 6LL * c->N0 * c->N1 * c->Kzp * cb))) return bail(e);
    if (cfg->store_pressure && !c->vv && (e = dalloc(c, &c->Pc, c->ncomp1 * cb))) return bail(e);
    // blocks of the pointwise RK update (one energy/enstrophy partial pair each)
    c->nblk_rk = (c->K1 * c->Kzp + 255) / 256 * c->K0;
    if ((e = dalloc(c, &c->partials, 2 * c->nblk_rk * 8))) return bail(e);
  }
  if ((e = dalloc(c, &c->sc, SC_COUNT * 8))) return bail(e);
  if ((e = dalloc(c, &c->flag, 16))) return bail(e);
  // twiddle tables: per axis, pass tables [r][k] of W_{Ns R}^{r k} (forward)
  {
    long long tot = 0;
    for (int i = 0; i < 3; ++i) { c->twoff[i] = tot; tot += tw_total(cfg->n[i]); }
    std::vector<double> h(2 * tot);
    for (int i = 0; i < 3; ++i) {
      const int n = cfg->n[i];
      long long off = c->twoff[i];
      int ns = 1;
      while (ns < n) {
        const int r = (n / ns) >= 16 ? 16 : n / ns;
        const long long m = (long long)ns * r;
        for (int q = 0; q < r; ++q)
          for (int k = 0; k < ns; ++k) {
            const long long e2 = ((long long)q * k) % m;
            const double ang = -2.0 * M_PI * (double)e2 / (double)m;
            h[2 * (off + (long long)q * ns + k)] = cos(ang);
            h[2 * (off + (long long)q * ns + k) + 1] = sin(ang);
          }
        off += m;
        ns *= r;
      }
      for (int q = 0; q < n; ++q) {  // full table W_n^q
        const double ang = -2.0 * M_PI * (double)q / (double)n;
        h[2 * (off + q)] = cos(ang);
        h[2 * (off + q) + 1] = sin(ang);
      }
    }
    if ((e = dalloc(c, &c->tw, tot * cb))) return bail(e);
    if (c->dbl) {
      if (cudaMemcpy(c->tw, h.data(), tot * 16, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(SDNS_ECUDA, "twiddle upload failed"));
    } else {
      std::vector<float> hf(2 * tot);
      for (long long q = 0; q < 2 * tot; ++q) hf[q] = (float)h[q];
      if (cudaMemcpy(c->tw, hf.data(), tot * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(SDNS_ECUDA, "twiddle upload failed"));
    }
  }
  if (cudaMemset(c->sc, 0, SC_COUNT * 8) != cudaSuccess) return bail(fail(SDNS_ECUDA, "memset failed"));
  if (c->S && cudaMemset(c->S, 0, 3 * c->ncomp1 * 16) != cudaSuccess) return bail(fail(SDNS_ECUDA, "memset failed"));
  if (c->Y && cudaMemset(c->Y, 0, 3 * c->ncomp1 * cb) != cudaSuccess) return bail(fail(SDNS_ECUDA, "memset failed"));
  *out = c;
  return SDNS_OK;
}

int sdns_destroy(sdns_ctx* c) {
  if (!c) return SDNS_OK;
  cudaSetDevice(c->dev);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  void* bufs[] = {c->Y, c->S, c->A, c->T1, c->T2, c->Pc, c->Yx, c->src, c->src_full, c->H,
                  c->F1, c->F2, c->PH, c->stage, c->tw, c->sc, c->partials, c->flag, c->red,
                  c->U32, c->U32a, c->U32b, c->R32, c->P32, c->spec32, c->phys32, c->tw32};
  for (void* p : bufs)
    if (p) cudaFree(p);
  for (auto& e : c->evpool)
    if (e) cudaEventDestroy(e);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return SDNS_OK;
}

int sdns_synchronize(sdns_ctx* c) {
  int e = check_ctx(c);
  if (e) return e;
  CK(cudaStreamSynchronize(c->st));
  return SDNS_OK;
}

int sdns_get_stream(sdns_ctx* c, void** stream) {
  if (!c || !stream) return fail(SDNS_EINVAL, "null argument");
  *stream = (void*)c->st;
  return SDNS_OK;
}

int sdns_memory_bytes(sdns_ctx* c, int64_t* bytes) {
  if (!c || !bytes) return fail(SDNS_EINVAL, "null argument");
  *bytes = c->bytes;
  return SDNS_OK;
}

int sdns_set_state(sdns_ctx* c, const void* u_hat, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if (!u_hat) return fail(SDNS_EINVAL, "null u_hat");
  if (c->pad32) {
    if ((e = copy_in(c, c->U32, u_hat, 3 * c->nfull1 * (long long)c->csz, where))) return e;
    CK(cudaMemsetAsync(c->sc + SC_FLAG, 0, 8, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->has_state = true;
    return SDNS_OK;
  }
  if ((e = ensure_stage(c))) return e;
  if ((e = copy_in(c, c->stage, u_hat, 3 * c->nfull1 * (long long)c->csz, where))) return e;
  Geo g = geo(c);
  CK(cudaMemsetAsync(c->flag, 0, 4, c->st));
  CK(cudaMemsetAsync(c->sc + SC_FLAG, 0, 8, c->st));  // a new state clears an earlier non-finite report
  if (c->dbl) {
    k_gather<double2><<<nblocks(3 * c->ncomp1), 256, 0, c->st>>>((const double2*)c->stage, (double2*)c->Y, c->S, g, c->ncomp1);
    k_outside<double2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>((const double2*)c->stage, g, c->flag);
  } else {
    k_gather<float2><<<nblocks(3 * c->ncomp1), 256, 0, c->st>>>((const float2*)c->stage, (float2*)c->Y, c->S, g, c->ncomp1);
    k_outside<float2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>((const float2*)c->stage, g, c->flag);
  }
  CK(cudaGetLastError());
  int hflag = 0;
  CK(cudaMemcpyAsync(&hflag, c->flag, 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  const bool was_high = c->high;
  c->high = hflag != 0;
  if (c->high) {
    if (!c->H && (e = dalloc(c, &c->H, 3 * c->nfull1 * (long long)c->csz))) return e;
    CK(cudaMemcpyAsync(c->H, c->stage, 3 * c->nfull1 * c->csz, cudaMemcpyDeviceToDevice, c->st));
  }
  c->has_state = true;
  if (c->high != was_high) c->gkey = ~0ull;  // the step graph depends on `high`
  return SDNS_OK;
}

int sdns_get_state(sdns_ctx* c, void* u_hat, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if (!u_hat) return fail(SDNS_EINVAL, "null u_hat");
  if (c->pad32) return copy_out(c, u_hat, c->U32, 3 * c->nfull1 * (long long)c->csz, where);
  if ((e = ensure_stage(c))) return e;
  Geo g = geo(c);
  if (c->dbl)
    k_scatter<double2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>(
        c->S, 1, (double2*)c->stage, c->high ? (const double2*)c->H : nullptr, g, 3, c->N2h, c->ncomp1, 0);
  else
    k_scatter<float2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>(
        c->S, 1, (float2*)c->stage, c->high ? (const float2*)c->H : nullptr, g, 3, c->N2h, c->ncomp1, 0);
  CK(cudaGetLastError());
  return copy_out(c, u_hat, c->stage, 3 * c->nfull1 * (long long)c->csz, where);
}

int sdns_set_source(sdns_ctx* c, const void* source, int where) {
  int e = check_ctx(c);
  if (e) return e;
  // the RK4 graph depends on whether a source exists, not on its values
  if (!source || !c->src) c->gkey = ~0ull;
  if (!source) {
    if (c->src) { cudaFree(c->src); c->bytes -= 3 * c->ncomp1 * 16; c->src = nullptr; }
    if (c->src_full) { cudaFree(c->src_full); c->bytes -= 3 * c->nfull1 * c->csz; c->src_full = nullptr; }
    return SDNS_OK;
  }
  if (c->pad32) {  // the padded right-hand side reads the caller-layout source
    if (!c->src_full && (e = dalloc(c, &c->src_full, 3 * c->nfull1 * (long long)c->csz))) return e;
    if ((e = copy_in(c, c->src_full, source, 3 * c->nfull1 * (long long)c->csz, where))) return e;
    if (where == SDNS_HOST) CK(cudaStreamSynchronize(c->st));
    return SDNS_OK;
  }
  if (!c->src && (e = dalloc(c, &c->src, 3 * c->ncomp1 * 16))) return e;
  if (!c->src_full && (e = dalloc(c, &c->src_full, 3 * c->nfull1 * (long long)c->csz))) return e;
  if ((e = copy_in(c, c->src_full, source, 3 * c->nfull1 * (long long)c->csz, where))) return e;
  Geo g = geo(c);
  if (c->dbl)
    k_gather<double2><<<nblocks(3 * c->ncomp1), 256, 0, c->st>>>((const double2*)c->src_full, nullptr, c->src, g, c->ncomp1);
  else
    k_gather<float2><<<nblocks(3 * c->ncomp1), 256, 0, c->st>>>((const float2*)c->src_full, nullptr, c->src, g, c->ncomp1);
  CK(cudaGetLastError());
  // a host source may be released on return; a device source is ordered on the stream
  if (where == SDNS_HOST) CK(cudaStreamSynchronize(c->st));
  return SDNS_OK;
}

int sdns_compute_rhs(sdns_ctx* c, const void* u_hat, void* rhs, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if (!u_hat || !rhs) return fail(SDNS_EINVAL, "null argument");
  if ((e = ensure_stage(c))) return e;
  if (c->pad32) {
    const long long fb3 = 3 * c->nfull1 * (long long)c->csz;
    if ((e = copy_in(c, c->stage, u_hat, fb3, where))) return e;
    if ((e = rhs32(c, c->stage, c->R32, c->P32 != nullptr))) return e;
    return copy_out(c, rhs, c->R32, fb3, where);
  }
  if (!c->Yx && (e = dalloc(c, &c->Yx, 3 * c->ncomp1 * (long long)c->csz))) return e;
  const long long fb = 3 * c->nfull1 * (long long)c->csz;
  if ((e = copy_in(c, c->stage, u_hat, fb, where))) return e;
  Geo g = geo(c);
  if (c->dbl)
    k_gather<double2><<<nblocks(3 * c->ncomp1), 256, 0, c->st>>>((const double2*)c->stage, (double2*)c->Yx, nullptr, g, c->ncomp1);
  else
    k_gather<float2><<<nblocks(3 * c->ncomp1), 256, 0, c->st>>>((const float2*)c->stage, (float2*)c->Yx, nullptr, g, c->ncomp1);
  CK(cudaGetLastError());
  // compact rhs lands in T2 (free after the forward y sweep)
  if ((e = launch_stage_sweeps(c, c->Yx, 4, false, c->T2, c->Pc))) return e;
  // scatter: inside -> compact rhs, outside -> -nu K^2 u_hat (+ Source); the
  // result goes to the first half of the padded-full scratch so `stage` (u_hat) survives
  if ((e = ensure_full_bufs(c))) return e;
  void* out = c->F1;
  if (c->dbl) {
    k_scatter<double2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>(
        c->T2, 0, (double2*)out, nullptr, g, 3, c->N2h, c->ncomp1, 0);
    k_rhs_outside<double2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>(
        (const double2*)c->stage, (const double2*)c->src_full, (double2*)out, g, c->cfg.nu);
  } else {
    k_scatter<float2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>(
        c->T2, 0, (float2*)out, nullptr, g, 3, c->N2h, c->ncomp1, 0);
    k_rhs_outside<float2><<<nblocks(3 * c->nfull1), 256, 0, c->st>>>(
        (const float2*)c->stage, (const float2*)c->src_full, (float2*)out, g, c->cfg.nu);
  }
  CK(cudaGetLastError());
  return copy_out(c, rhs, out, fb, where);
}

int sdns_set_forcing(sdns_ctx* c, double eps, double kf) {
  int e = check_ctx(c);
  if (e) return e;
  if (c->vv && eps > 0) return fail(SDNS_EINVAL, "the forcing is defined for the velocity formulation (SDNS_NS) only");
  if (c->pad32 && eps > 0) return fail(SDNS_EINVAL, "the forcing is not available with the 3/2 rule");
  c->eps = eps > 0 ? eps : 0;
  c->kf = kf;
  c->gkey = ~0ull;
  return SDNS_OK;
}

int sdns_set_cfl(sdns_ctx* c, double cfl) {
  int e = check_ctx(c);
  if (e) return e;
  if (c->pad32 && cfl > 0) return fail(SDNS_EINVAL, "the CFL time step is not available with the 3/2 rule");
  c->cfl = cfl > 0 ? cfl : 0;
  c->gkey = ~0ull;
  c->last_dt = -1;
  return SDNS_OK;
}

int sdns_set_time(sdns_ctx* c, double t) {
  int e = check_ctx(c);
  if (e) return e;
  CK(cudaMemcpyAsync(c->sc + SC_TIME, &t, 8, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return SDNS_OK;
}

int sdns_rk4(sdns_ctx* c, double dt, int32_t nsteps) {
  int e = check_ctx(c);
  if (e) return e;
  if (!c->has_state) return fail(SDNS_ESTATE, "sdns_rk4: no state set");
  if (nsteps < 0) return fail(SDNS_EINVAL, "nsteps < 0");
  if (c->cfl <= 0) {
    if (!(dt > 0)) return fail(SDNS_EINVAL, "dt must be positive without CFL");
    if (dt != c->last_dt) {
      CK(cudaMemcpyAsync(c->sc + SC_DT, &dt, 8, cudaMemcpyHostToDevice, c->st));
      CK(cudaStreamSynchronize(c->st));
      c->last_dt = dt;
    }
  }
  if (c->pad32) {
    for (int s = 0; s < nsteps; ++s)
      if ((e = rk4_step32(c, dt))) return e;
    return SDNS_OK;
  }
  if (c->timing) {
    for (int k = 0; k < 8; ++k) { c->tms[k] = 0; c->tcount[k] = 0; }
    c->evused = 0;
    for (int s = 0; s < nsteps; ++s)
      if ((e = launch_step(c))) return e;
    CK(cudaStreamSynchronize(c->st));
    for (size_t q = 0; q < c->evused; q += 2) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, c->evpool[q], c->evpool[q + 1]));
      c->tms[c->evclass[q / 2]] += ms;
      c->tcount[c->evclass[q / 2]] += 1;
    }
    c->evused = 0;
    return SDNS_OK;
  }
  const unsigned long long key = (c->high ? 1 : 0) | (c->cfl > 0 ? 2 : 0) | (c->eps > 0 ? 4 : 0) |
                                 (c->src ? 8 : 0) | (c->cfg.store_pressure ? 16 : 0);
  if (!c->gexec || key != c->gkey) {
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    int le = launch_step(c);
    cudaError_t ce = cudaStreamEndCapture(c->st, &graph);
    if (le) return le;
    if (ce != cudaSuccess) return fail(SDNS_ECUDA, "graph capture failed: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&c->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return fail(SDNS_ECUDA, "graph instantiate failed: %s", cudaGetErrorString(ce));
    c->gkey = key;
  }
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(c->gexec, c->st));
  return SDNS_OK;
}

int sdns_forward(sdns_ctx* c, const void* phys, void* spec, int32_t nf, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if (!phys || !spec || nf < 1 || nf > 3) return fail(SDNS_EINVAL, "bad argument");
  if ((e = ensure_full_bufs(c)) || (e = ensure_stage(c))) return e;
  if ((e = copy_in(c, c->PH, phys, nf * c->nphys1 * (long long)c->rsz, where))) return e;
  if ((e = full_forward(c, c->F1, c->F2, nf))) return e;
  if ((e = repitch(c, c->F1, c->stage, nf, c->Kzpf, c->N2h, c->N2h))) return e;
  return copy_out(c, spec, c->stage, nf * c->nfull1 * (long long)c->csz, where);
}

int sdns_backward(sdns_ctx* c, const void* spec, void* phys, int32_t nf, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if (!phys || !spec || nf < 1 || nf > 3) return fail(SDNS_EINVAL, "bad argument");
  if ((e = ensure_full_bufs(c)) || (e = ensure_stage(c))) return e;
  if ((e = copy_in(c, c->stage, spec, nf * c->nfull1 * (long long)c->csz, where))) return e;
  if ((e = repitch(c, c->stage, c->F1, nf, c->N2h, c->Kzpf, c->N2h))) return e;
  if ((e = full_backward(c, c->F1, c->F2, nf))) return e;
  return copy_out(c, phys, c->PH, nf * c->nphys1 * (long long)c->rsz, where);
}

int sdns_velocity(sdns_ctx* c, void* u, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if (!c->has_state) return fail(SDNS_ESTATE, "no state set");
  if (c->vv) return sdns_velocity_vv(c, nullptr, u, where);
  if ((e = ensure_full_bufs(c))) return e;
  if ((e = state_to_padded(c, c->F1))) return e;
  if ((e = full_backward(c, c->F1, c->F2, 3))) return e;
  return copy_out(c, u, c->PH, 3 * c->nphys1 * (long long)c->rsz, where);
}

// spectral vector (caller layout) or, when u_hat is NULL, the context state -> padded F2
int spectral_to_padded(sdns_ctx* c, const void* u_hat, int where) {
  int e;
  if (!u_hat) {
    if (!c->has_state) return fail(SDNS_ESTATE, "no state set");
    return state_to_padded(c, c->F2);
  }
  if ((e = ensure_stage(c))) return e;
  if ((e = copy_in(c, c->stage, u_hat, 3 * c->nfull1 * (long long)c->csz, where))) return e;
  return repitch(c, c->stage, c->F2, 3, c->N2h, c->Kzpf, c->N2h);
}

// padded F2 (3 fields) -> F1 by k_curl_div in the given mode
int curl_div_f2(sdns_ctx* c, int mode) {
  Geo g = geo(c);
  if (c->dbl) k_curl_div<double2><<<nblocks(c->npadf1), 256, 0, c->st>>>((const double2*)c->F2, (double2*)c->F1, g, mode);
  else k_curl_div<float2><<<nblocks(c->npadf1), 256, 0, c->st>>>((const float2*)c->F2, (float2*)c->F1, g, mode);
  CK(cudaGetLastError());
  return SDNS_OK;
}

int sdns_velocity_vv(sdns_ctx* c, const void* w_hat, void* u, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if (!u) return fail(SDNS_EINVAL, "null output");
  if ((e = ensure_full_bufs(c))) return e;
  if ((e = spectral_to_padded(c, w_hat, where))) return e;
  if ((e = curl_div_f2(c, 2))) return e;
  if ((e = full_backward(c, c->F1, c->F2, 3))) return e;
  return copy_out(c, u, c->PH, 3 * c->nphys1 * (long long)c->rsz, where);
}

int sdns_curl(sdns_ctx* c, const void* u_hat, void* w, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if ((e = ensure_full_bufs(c))) return e;
  if ((e = spectral_to_padded(c, u_hat, where))) return e;
  if ((e = curl_div_f2(c, 0))) return e;
  if ((e = full_backward(c, c->F1, c->F2, 3))) return e;
  return copy_out(c, w, c->PH, 3 * c->nphys1 * (long long)c->rsz, where);
}

int sdns_divergence(sdns_ctx* c, const void* u_hat, void* d, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if ((e = ensure_full_bufs(c))) return e;
  if ((e = spectral_to_padded(c, u_hat, where))) return e;
  if (c->vv && !u_hat) {
    // divergence of the velocity of the state W_hat: F2 -> velocity F1 -> back into F2
    if ((e = curl_div_f2(c, 2))) return e;
    CK(cudaMemcpyAsync(c->F2, c->F1, 3 * c->npadf1 * (long long)c->csz, cudaMemcpyDeviceToDevice, c->st));
  }
  if ((e = curl_div_f2(c, 1))) return e;
  if ((e = full_backward(c, c->F1, c->F2, 1))) return e;
  return copy_out(c, d, c->PH, c->nphys1 * (long long)c->rsz, where);
}

int sdns_pressure(sdns_ctx* c, void* p, int where) {
  int e = check_ctx(c);
  if (e) return e;
  if (c->vv) return fail(SDNS_EINVAL, "the velocity-vorticity formulation has no pressure (VV.py:27)");
  if (c->pad32) {
    if (!c->P32) return fail(SDNS_ESTATE, "pressure is not stored (create the context with store_pressure=1)");
    if ((e = ensure_full_bufs(c))) return e;
    if ((e = repitch(c, c->P32, c->F1, 1, c->N2h, c->Kzpf, c->N2h))) return e;
    if ((e = full_backward(c, c->F1, c->F2, 1))) return e;
    return copy_out(c, p, c->PH, c->nphys1 * (long long)c->rsz, where);
  }
  if (!c->Pc) return fail(SDNS_ESTATE, "pressure is not stored (create the context with store_pressure=1)");
  if ((e = ensure_full_bufs(c))) return e;
  Geo g = geo(c);
  if (c->dbl)
    k_scatter<double2><<<nblocks(c->npadf1), 256, 0, c->st>>>(c->Pc, 0, (double2*)c->F1, nullptr, g, 1, c->Kzpf,
                                                               c->ncomp1, 1);
  else
    k_scatter<float2><<<nblocks(c->npadf1), 256, 0, c->st>>>(c->Pc, 0, (float2*)c->F1, nullptr, g, 1, c->Kzpf,
                                                              c->ncomp1, 1);
  CK(cudaGetLastError());
  if ((e = full_backward(c, c->F1, c->F2, 1))) return e;
  return copy_out(c, p, c->PH, c->nphys1 * (long long)c->rsz, where);
}

int sdns_diagnostics(sdns_ctx* c, double* out) {
  int e = check_ctx(c);
  if (e) return e;
  if (!out) return fail(SDNS_EINVAL, "null out");
  if (!c->has_state) return fail(SDNS_ESTATE, "no state set");
  Geo g = diag_geo(c);
  const unsigned nb = 152 * 4;
  double* part = nullptr;
  if ((e = dalloc(c, &part, 3LL * nb * 8))) return e;
  if (c->dbl)
    k_diag<double2><<<nb, 256, 0, c->st>>>(c->S, (const double2*)diag_full(c), g, c->ncomp1, part, c->vv);
  else
    k_diag<float2><<<nb, 256, 0, c->st>>>(c->S, (const float2*)diag_full(c), g, c->ncomp1, part, c->vv);
  CK(cudaGetLastError());
  std::vector<double> h(3 * nb);
  double scal[SC_COUNT];
  CK(cudaMemcpyAsync(h.data(), part, 3 * nb * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(scal, c->sc, SC_COUNT * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  cudaFree(part);
  c->bytes -= 3LL * nb * 8;
  double s[3] = {0, 0, 0};
  for (unsigned b = 0; b < nb; ++b)
    for (int q = 0; q < 3; ++q) s[q] += h[3 * b + q];
  for (int q = 0; q < SDNS_DIAG_COUNT; ++q) out[q] = 0;
  out[SDNS_DIAG_ENERGY] = s[0];
  out[SDNS_DIAG_ENSTROPHY] = s[1];
  out[SDNS_DIAG_DISSIPATION] = 2.0 * c->cfg.nu * s[1];
  out[SDNS_DIAG_DIVERGENCE] = s[2];
  out[SDNS_DIAG_CFL_RATE] = scal[SC_LASTRATE];
  out[SDNS_DIAG_TIME] = scal[SC_TIME];
  out[SDNS_DIAG_LAST_DT] = scal[SC_DT];
  if (!(s[0] == s[0]) || scal[SC_FLAG] != 0.0) return fail(SDNS_ENONFINITE, "non-finite energy in the solution");
  return SDNS_OK;
}

int sdns_spectrum(sdns_ctx* c, double* Ek, int32_t nbins) {
  int e = check_ctx(c);
  if (e) return e;
  if (!Ek || nbins < 2) return fail(SDNS_EINVAL, "bad argument");
  if (!c->has_state) return fail(SDNS_ESTATE, "no state set");
  double* d = nullptr;
  if ((e = dalloc(c, &d, 2LL * nbins * 8))) return e;
  CK(cudaMemsetAsync(d, 0, 2LL * nbins * 8, c->st));
  Geo g = diag_geo(c);
  if (c->dbl)
    k_spectrum<double2><<<152 * 4, 256, 0, c->st>>>(c->S, (const double2*)diag_full(c), g, c->ncomp1, d, d + nbins,
                                                   nbins, c->vv);
  else
    k_spectrum<float2><<<152 * 4, 256, 0, c->st>>>(c->S, (const float2*)diag_full(c), g, c->ncomp1, d, d + nbins,
                                                  nbins, c->vv);
  CK(cudaGetLastError());
  std::vector<double> h(2 * nbins);
  CK(cudaMemcpyAsync(h.data(), d, 2LL * nbins * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  cudaFree(d);
  c->bytes -= 2LL * nbins * 8;
  for (int i = 0; i < nbins; ++i) {
    const double k0 = i + 0.5, k = i + 1.5;
    Ek[i] = (h[nbins + i] > 0 && i < nbins - 1) ? (4.0 / 3.0 * M_PI) * (k * k * k - k0 * k0 * k0) * h[i] / h[nbins + i] : 0.0;
  }
  return SDNS_OK;
}

int sdns_lincomb(sdns_ctx* c, void* out, const void* base, int32_t nterms, const double* coef,
                 const void* const* terms) {
  int e = check_ctx(c);
  if (e) return e;
  if (!out || nterms < 0 || nterms > SDNS_LINCOMB_MAX || (nterms > 0 && (!coef || !terms)))
    return fail(SDNS_EINVAL, "sdns_lincomb: bad arguments (0 <= nterms <= %d)", SDNS_LINCOMB_MAX);
  LinTerms lt = {};
  lt.n = nterms;
  for (int k = 0; k < nterms; ++k) {
    if (!terms[k]) return fail(SDNS_EINVAL, "sdns_lincomb: null term %d", k);
    lt.t[k] = terms[k];
    lt.c[k] = coef[k];
  }
  const long long n = 3 * c->nfull1;
  if (c->dbl)
    k_lincomb<double2><<<nblocks(n), 256, 0, c->st>>>((double2*)out, (const double2*)base, lt, n);
  else
    k_lincomb<float2><<<nblocks(n), 256, 0, c->st>>>((float2*)out, (const float2*)base, lt, n);
  CK(cudaGetLastError());
  return SDNS_OK;
}

int sdns_error_norm(sdns_ctx* c, const void* err, const void* u0, const void* u1, double atol, double rtol,
                    double* sums) {
  int e = check_ctx(c);
  if (e) return e;
  if (!err || !u0 || !u1 || !sums) return fail(SDNS_EINVAL, "sdns_error_norm: null argument");
  const unsigned nb = 152 * 2;
  if (!c->red && (e = dalloc(c, &c->red, 3LL * nb * 8))) return e;
  if (c->dbl)
    k_err_norm<double2><<<nb, 256, 0, c->st>>>((const double2*)err, (const double2*)u0, (const double2*)u1, atol, rtol,
                                               c->nfull1, c->red);
  else
    k_err_norm<float2><<<nb, 256, 0, c->st>>>((const float2*)err, (const float2*)u0, (const float2*)u1, atol, rtol,
                                              c->nfull1, c->red);
  CK(cudaGetLastError());
  std::vector<double> h(3 * nb);
  CK(cudaMemcpyAsync(h.data(), c->red, 3 * nb * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int q = 0; q < 3; ++q) sums[q] = 0;
  for (unsigned b = 0; b < nb; ++b)
    for (int q = 0; q < 3; ++q) sums[q] += h[3 * b + q];
  return SDNS_OK;
}

int sdns_set_timing(sdns_ctx* c, int32_t on) {
  int e = check_ctx(c);
  if (e) return e;
  c->timing = on != 0;
  return SDNS_OK;
}

int sdns_get_timing(sdns_ctx* c, double* ms, int32_t* launches) {
  if (!c || !ms || !launches) return fail(SDNS_EINVAL, "null argument");
  for (int k = 0; k < 8; ++k) { ms[k] = c->tms[k]; launches[k] = c->tcount[k]; }
  return SDNS_OK;
}

}  // extern "C"
