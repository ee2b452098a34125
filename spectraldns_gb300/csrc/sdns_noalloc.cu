// Allocation-free ComputeRHS (sdns_compute_rhs_noalloc).
//
// Callers that cannot allocate device memory -- code recorded into a CUDA
// graph, a framework whose caching allocator owns the device memory, or a
// real-time loop that forbids allocation -- still need the right-hand side.
// This entry point evaluates it without any cudaMalloc/cudaFree: its scratch
// (twiddle tables, the compact input, the two intermediate fields) lives in
// one file-scope __device__ array of SDNS_NOALLOC_SCRATCH_BYTES, which every
// GPU that loads the library holds until the process exits.
//
// Host code cannot use the array's name as a device address, so the first
// call on a device (with that device current) looks the address up with
// cudaGetSymbolAddress and caches it; that first call should therefore come
// before any stream capture.  All calls share the one array: calls whose
// work overlaps on the GPU (different streams, or different host threads)
// race on it and must be serialised by the caller.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "../../include/sdns_gb300.h"
#include "sdns_fft.cuh"
#include "sdns_internal.h"

using namespace sdns;

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[SDNS_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_mu;

int na_fail(int code, const char* msg) {
  sdns::set_last_error(msg);
  return code;
}

inline long long rup(long long a, long long b) { return (a + b - 1) / b * b; }

int na_cutoff(int n, int rule) {
  if (rule == SDNS_DEALIAS_NONE) return n / 2 - 1;
  const double kmax = 2.0 / 3.0 * (n / 2 + 1);
  int kc = (int)ceil(kmax) - 1;
  while (kc + 1 < kmax) ++kc;
  while (kc >= kmax) --kc;
  return kc;
}

struct NaGeo {
  RowMap m0, m1;
  int N0, N1, N2h, Kz, Kzp;
  double ks[3];
  __device__ bool inside(int p0, int p1, int kz) const {
    auto in = [](const RowMap& m, int p) { return m.kc < 0 || p <= m.kc || p >= m.n - m.kc; };
    return in(m0, p0) && in(m1, p1) && kz < Kz;
  }
  __device__ int row(const RowMap& m, int p) const { return (m.kc < 0 || p <= m.kc) ? p : p - m.n + 2 * m.kc + 1; }
  __device__ double wave(int p, int n) const { return (double)(p < (n + 1) / 2 ? p : p - n); }
};

// twiddle table of an axis of n points (same layout as the context tables),
// generated in FP64 on the device
template <typename C>
__global__ void k_na_twiddles(C* tw, int n) {
  const int len = tw_len(n);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tw_total(n); e += gridDim.x * blockDim.x) {
    if (e >= len) {  // full table W_n^q
      double sn, cs;
      sincospi(-2.0 * (double)(e - len) / (double)n, &sn, &cs);
      C w;
      w.x = (decltype(w.x))cs;
      w.y = (decltype(w.x))sn;
      tw[e] = w;
      continue;
    }
    int ns = 1, off = 0;
    while (true) {
      const int r = (n / ns) >= 16 ? 16 : n / ns;
      if (e < off + r * ns) {
        const int q = (e - off) / ns, k = (e - off) % ns;
        const long long m = (long long)ns * r;
        const long long ex = ((long long)q * k) % m;
        double sn, cs;
        sincospi(-2.0 * (double)ex / (double)m, &sn, &cs);
        C w;
        w.x = (decltype(w.x))cs;
        w.y = (decltype(w.x))sn;
        tw[e] = w;
        break;
      }
      off += r * ns;
      ns *= r;
    }
  }
}

// caller layout [3][N0][N1][N2h] -> compact [3][K0][K1][Kzp] (padding zeroed)
template <typename C>
__global__ void k_na_gather(const C* full, C* comp, NaGeo g, long long ncomp1) {
  const long long n = 3 * ncomp1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long c = i / ncomp1;
    long long rem = i - c * ncomp1;
    const int kz = (int)(rem % g.Kzp);
    rem /= g.Kzp;
    const int r1 = (int)(rem % g.m1.rows());
    const int r0 = (int)(rem / g.m1.rows());
    C v;
    v.x = 0;
    v.y = 0;
    if (kz < g.Kz) v = full[((c * g.N0 + g.m0.pos(r0)) * g.N1 + g.m1.pos(r1)) * g.N2h + kz];
    comp[i] = v;
  }
}

// compact rhs (inside the dealiased set) and -nu K^2 u_hat (outside) -> caller layout
template <typename C>
__global__ void k_na_scatter(const C* comp, const C* uh, C* rhs, NaGeo g, long long ncomp1, double nu) {
  const long long n1 = (long long)g.N0 * g.N1 * g.N2h, n = 3 * n1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long c = i / n1;
    long long rem = i - c * n1;
    const int kz = (int)(rem % g.N2h);
    rem /= g.N2h;
    const int p1 = (int)(rem % g.N1), p0 = (int)(rem / g.N1);
    C v;
    if (g.inside(p0, p1, kz)) {
      v = comp[c * ncomp1 + ((long long)g.row(g.m0, p0) * g.m1.rows() + g.row(g.m1, p1)) * g.Kzp + kz];
    } else {
      const double k0 = g.ks[0] * g.wave(p0, g.N0), k1 = g.ks[1] * g.wave(p1, g.N1), k2 = g.ks[2] * kz;
      const double z = nu * (k0 * k0 + k1 * k1 + k2 * k2);
      const C u = uh[i];
      v.x = (decltype(v.x))(-z * u.x);
      v.y = (decltype(v.x))(-z * u.y);
    }
    rhs[i] = v;
  }
}

inline unsigned na_blocks(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 16) b = 152LL * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

// byte offsets of the scratch regions for one configuration
struct NaLayout {
  size_t tw[3], dt, comp, t1, t2, total;
};

NaLayout na_layout(const int n[3], long long K0, long long K1, long long Kzp, size_t csz) {
  NaLayout L;
  size_t off = 0;
  for (int i = 0; i < 3; ++i) {
    L.tw[i] = off;
    off = (size_t)rup((long long)(off + (size_t)tw_total(n[i]) * csz), 256);
  }
  L.dt = off;
  off += 256;
  L.comp = off;
  off = (size_t)rup((long long)(off + (size_t)3 * K0 * K1 * Kzp * csz), 256);
  L.t1 = off;
  off = (size_t)rup((long long)(off + (size_t)6 * n[0] * K1 * Kzp * csz), 256);
  L.t2 = off;
  off = (size_t)rup((long long)(off + (size_t)6 * n[0] * n[1] * Kzp * csz), 256);
  L.total = off;
  return L;
}

// once per device, with that device current: the device address of the array
int na_setup(int dev, unsigned char** base) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= kMaxDevices) return na_fail(SDNS_EINVAL, "device ordinal out of range");
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return na_fail(SDNS_ECUDA, "cudaGetSymbolAddress of the no-alloc scratch failed");
    }
    int oe = Kernels<float>::smem_optin(dev);
    if (oe == 0) oe = Kernels<double>::smem_optin(dev);
    if (oe != 0) return na_fail(SDNS_ECUDA, "shared-memory opt-in failed");
    g_scratch_ptr[dev] = p;
  }
  *base = reinterpret_cast<unsigned char*>(g_scratch_ptr[dev]);
  return SDNS_OK;
}

template <typename Real>
int na_run(const sdns_config* cfg, const void* u_hat, void* rhs, cudaStream_t st, unsigned char* base) {
  using C = typename cplx_of<Real>::type;
  const size_t csz = sizeof(C);
  const int N0 = cfg->n[0], N1 = cfg->n[1], N2 = cfg->n[2], N2h = N2 / 2 + 1;
  const RowMap m0 = {N0, na_cutoff(N0, cfg->dealias)}, m1 = {N1, na_cutoff(N1, cfg->dealias)};
  const RowMap f0 = {N0, -1}, f1 = {N1, -1};
  const int Kz = na_cutoff(N2, cfg->dealias) + 1;
  const long long Kzp = rup(Kz, 8), K0 = m0.rows(), K1 = m1.rows();
  const long long ncomp1 = K0 * K1 * Kzp;
  const NaLayout L = na_layout(cfg->n, K0, K1, Kzp, csz);
  if (L.total > (size_t)SDNS_NOALLOC_SCRATCH_BYTES) {
    char msg[200];
    snprintf(msg, sizeof msg, "grid %dx%dx%d needs %zu bytes of scratch; the no-alloc entry point has %d",
             N0, N1, N2, L.total, (int)SDNS_NOALLOC_SCRATCH_BYTES);
    return na_fail(SDNS_EINVAL, msg);
  }
  C* tw[3];
  for (int i = 0; i < 3; ++i) {
    tw[i] = reinterpret_cast<C*>(base + L.tw[i]);
    k_na_twiddles<C><<<4, 256, 0, st>>>(tw[i], cfg->n[i]);
  }
  double* dt = reinterpret_cast<double*>(base + L.dt);
  C* comp = reinterpret_cast<C*>(base + L.comp);
  void* T1 = base + L.t1;
  void* T2 = base + L.t2;
  NaGeo g;
  g.m0 = m0; g.m1 = m1; g.N0 = N0; g.N1 = N1; g.N2h = N2h; g.Kz = Kz; g.Kzp = (int)Kzp;
  double ks[3];
  for (int i = 0; i < 3; ++i) { ks[i] = 2.0 * M_PI / cfg->L[i]; g.ks[i] = ks[i]; }
  k_na_gather<C><<<na_blocks(3 * ncomp1), 256, 0, st>>>(reinterpret_cast<const C*>(u_hat), comp, g, ncomp1);
  if (cudaPeekAtLastError() != cudaSuccess) return na_fail(SDNS_ECUDA, "gather launch failed");
  // x^-1 with curl: compact -> T1 [6][N0][K1][Kzp]
  AxisArgs a = {};
  a.in = comp; a.out = T1;
  a.min = m0; a.mout = f0;
  a.in_fs = ncomp1; a.in_ss = 0; a.in_rs = K1 * Kzp;
  a.out_fs = (long long)N0 * K1 * Kzp; a.out_ss = 0; a.out_rs = K1 * Kzp;
  a.nlines = K1 * Kzp; a.B = a.nlines; a.nfield = 6; a.scale = 1.0; a.tw = tw[0];
  for (int i = 0; i < 3; ++i) a.kscale[i] = ks[i];
  a.m1 = m1; a.Kzp = (int)Kzp;
  if (Kernels<Real>::axis_curl_inv(a, st)) return na_fail(SDNS_ECUDA, "x sweep launch failed");
  // y^-1: T1 -> T2 [6][N0][N1][Kzp]
  AxisArgs b = {};
  b.in = T1; b.out = T2;
  b.min = m1; b.mout = f1;
  b.in_fs = (long long)N0 * K1 * Kzp; b.in_ss = K1 * Kzp; b.in_rs = Kzp;
  b.out_fs = (long long)N0 * N1 * Kzp; b.out_ss = (long long)N1 * Kzp; b.out_rs = Kzp;
  b.nlines = (long long)N0 * Kzp; b.B = Kzp; b.nfield = 6; b.scale = 1.0; b.tw = tw[1];
  if (Kernels<Real>::axis_plain(b, +1, st)) return na_fail(SDNS_ECUDA, "y sweep launch failed");
  // z: C2R x6, u x w, R2C x3 (in place into T2 fields 0..2)
  ZArgs z = {};
  z.in = T2; z.out = T2; z.nlines = (long long)N0 * N1; z.n = N2; z.Kz = Kz; z.Kzp = (int)Kzp; z.nf = 6;
  z.tw = tw[2];
  for (int i = 0; i < 3; ++i) z.inv_dx[i] = (double)cfg->n[i] / cfg->L[i];
  if (Kernels<Real>::zline_ns(z, st)) return na_fail(SDNS_ECUDA, "z sweep launch failed");
  // y forward: T2 [3][N0][N1][Kzp] -> T1 [3][N0][K1][Kzp]
  AxisArgs d = {};
  d.in = T2; d.out = T1;
  d.min = f1; d.mout = m1;
  d.in_fs = (long long)N0 * N1 * Kzp; d.in_ss = (long long)N1 * Kzp; d.in_rs = Kzp;
  d.out_fs = (long long)N0 * K1 * Kzp; d.out_ss = K1 * Kzp; d.out_rs = Kzp;
  d.nlines = (long long)N0 * Kzp; d.B = Kzp; d.nfield = 3; d.scale = 1.0; d.tw = tw[1];
  if (Kernels<Real>::axis_plain(d, -1, st)) return na_fail(SDNS_ECUDA, "y forward launch failed");
  // x forward + projection + diffusion -> compact rhs in T2
  RKArgs r = {};
  r.in = T1; r.m0 = m0; r.m1 = m1; r.Kz = Kz; r.Kzp = (int)Kzp; r.nlines = K1 * Kzp;
  r.scale = 1.0 / ((double)N0 * N1 * N2); r.tw = tw[0];
  for (int i = 0; i < 3; ++i) r.kscale[i] = ks[i];
  r.nu = cfg->nu; r.stage = 4; r.dt = dt; r.Y = comp; r.rhs_out = T2;
  if (Kernels<Real>::axis_rk(r, st, nullptr)) return na_fail(SDNS_ECUDA, "x forward launch failed");
  k_na_scatter<C><<<na_blocks(3LL * N0 * N1 * N2h), 256, 0, st>>>(reinterpret_cast<const C*>(T2),
                                                                   reinterpret_cast<const C*>(u_hat),
                                                                   reinterpret_cast<C*>(rhs), g, ncomp1, cfg->nu);
  if (cudaPeekAtLastError() != cudaSuccess) return na_fail(SDNS_ECUDA, "scatter launch failed");
  return SDNS_OK;
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

}  // namespace

extern "C" {

int sdns_compute_rhs_noalloc(const sdns_config* cfg, const void* u_hat, void* rhs, void* stream) {
  if (!cfg || !u_hat || !rhs) return na_fail(SDNS_EINVAL, "null argument");
  for (int i = 0; i < 3; ++i) {
    if (!pow2(cfg->n[i]) || cfg->n[i] < 16 || cfg->n[i] > 1024)
      return na_fail(SDNS_EINVAL, "grid sizes must be powers of two in [16, 1024]");
    if (!(cfg->L[i] > 0)) return na_fail(SDNS_EINVAL, "box lengths must be positive");
  }
  if (cfg->precision != SDNS_SINGLE && cfg->precision != SDNS_DOUBLE)
    return na_fail(SDNS_EINVAL, "precision must be SDNS_SINGLE or SDNS_DOUBLE");
  if (cfg->dealias != SDNS_DEALIAS_23 && cfg->dealias != SDNS_DEALIAS_NONE)
    return na_fail(SDNS_EINVAL, "dealias must be SDNS_DEALIAS_23 or SDNS_DEALIAS_NONE");
  if (cfg->formulation != SDNS_NS)
    return na_fail(SDNS_EINVAL, "the allocation-free right-hand side is the velocity (SDNS_NS) formulation only");
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) { cudaGetLastError(); return na_fail(SDNS_ECUDA, "no CUDA device"); }
  if (cfg->device != prev && cudaSetDevice(cfg->device) != cudaSuccess) {
    cudaGetLastError();
    return na_fail(SDNS_EINVAL, "cannot make the configured device current");
  }
  unsigned char* base = nullptr;
  int e = na_setup(cfg->device, &base);
  if (e == SDNS_OK) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    e = cfg->precision == SDNS_DOUBLE ? na_run<double>(cfg, u_hat, rhs, st, base)
                                      : na_run<float>(cfg, u_hat, rhs, st, base);
  }
  if (cfg->device != prev) cudaSetDevice(prev);
  return e;
}

}  // extern "C"
