// Internal declarations shared by the kernel translation units and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sdns {

// ---------------------------------------------------------------------------
// accumulator storage of the RK4 step-start state S and the accumulator A:
// FP64 complex (double solver) or compensated FP32 "float-float" complex
// {re_hi, im_hi, re_lo, im_lo} (single solver).  Both are 16 bytes.
// ---------------------------------------------------------------------------
template <typename Real> struct Acc;
template <> struct Acc<float> {
  using T = float4;
  __device__ static double2 get(const T* p, long long i) {
    const float4 v = p[i];
    return make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
  }
  __device__ static void put(T* p, long long i, double x, double y) {
    const float hx = (float)x, hy = (float)y;
    p[i] = make_float4(hx, hy, (float)(x - (double)hx), (float)(y - (double)hy));
  }
};
template <> struct Acc<double> {
  using T = double2;
  __device__ static double2 get(const T* p, long long i) { return p[i]; }
  __device__ static void put(T* p, long long i, double x, double y) { p[i] = make_double2(x, y); }
};


// Axis description.  A complex axis of n points stores either all n
// positions (kc < 0) or the 2kc+1 kept wave indices in FFT order
// [0..kc, -kc..-1] ("compact" rows).  The R2C axis stores kz = 0..Kz-1,
// padded to Kzp.
struct RowMap {
  int n;   // transform length
  int kc;  // cutoff, < 0 means all positions stored
  __host__ __device__ int rows() const { return kc < 0 ? n : 2 * kc + 1; }
  __host__ __device__ int pos(int r) const { return (kc < 0 || r <= kc) ? r : n - (2 * kc + 1) + r; }
  // signed integer wave index of a stored row
  __host__ __device__ int wave(int r) const {
    int p = pos(r);
    return p < (n + 1) / 2 ? p : p - n;
  }
};

// Batched transform along one strided axis.  Line l of field f starts at
// f*fs + (l / B)*ss + (l % B); position row r adds r*rs.  Lines l are
// consecutive in memory within runs of B.
struct AxisArgs {
  const void* in;
  void* out;
  RowMap min, mout;          // input rows, output rows (same n)
  long long in_fs, in_ss, in_rs;
  long long out_fs, out_ss, out_rs;
  long long nlines;          // lines per field
  long long B;               // contiguous run length of lines
  int nfield;
  double scale;              // applied to outputs
  const void* tw;            // twiddle table of this axis (forward sign)
  // curl prologue (inverse x sweep): wave-number scales and the compact
  // geometry of the batch index b = k1row*Kzp + kz
  double kscale[3];
  RowMap m1;                 // rows of axis 1 (for k1 of the batch index)
  int Kzp;
  int nbuf;                  // tile buffers of the persistent sweep (set by its launcher: 1 or 2)
};

// Fused z-line sweep: C2R of 6 spectral fields, u x w, R2C of 3 fields.
struct ZArgs {
  const void* in;            // [nf][nlines][Kzp] complex
  void* out;                 // [3][nlines][Kzp] complex (may alias in)
  void* phys;                // [nf][nlines][n] real (C2R-only / R2C-only modes)
  long long nlines;
  int n;                     // z transform length
  int Kz, Kzp;               // stored kz modes and padded pitch
  int nf;                    // number of fields (modes 1, 2)
  const void* tw;
  double inv_dx[3];          // for the CFL rate
  double* cfl_rate;          // nullptr: no CFL reduction
};

// Final x sweep with projection, diffusion, source and the RK4 stage update.
struct RKArgs {
  const void* in;            // [3][N0][K1][Kzp] complex (after forward y)
  RowMap m0, m1;             // rows of axis 0 and 1 of the compact layout
  int Kz, Kzp;
  long long nlines;          // K1*Kzp
  double scale;              // 1/(N0 N1 N2)
  const void* tw;
  double kscale[3];
  double nu;
  int stage;                 // 0..3 RK4 stage, 4 = ComputeRHS only
  double a, b;               // RK4 coefficients of this stage
  const double* dt;          // device scalar
  void* Y;                   // Real complex compact stage input / output
  void* S;                   // compact step-start state (Acc<Real>::T)
  void* A;                   // compact accumulator (Acc<Real>::T)
  void* rhs_out;             // stage 4: Real complex compact rhs
  void* p_out;               // optional Real complex compact P_hat
  const void* source;        // optional compact source (Acc<Real>::T)
  const double* force_alpha; // optional device scalar; forcing on 0 < K2 <= kf2
  double kf2;
  double* partials;          // [gridDim.x][4] energy, enstrophy sums (stage 3)
  int vv;                    // velocity-vorticity form: the state is W_hat and the
                             // convective term is i K x (nonlinear term), no projection
};

// 3/2-rule (padded) right-hand side: grid N, padded grid M = 3N/2 per axis
struct Pad32 {
  int N[3], M[3];
  double ks[3];              // 2 pi / L
  double nu;
  bool dbl, vv;
  void* spec;                // [6][M0][M1][M2/2+1] complex scratch
  void* phys;                // [6][M0][M1][M2] real scratch
  const void* tw[3];         // W_{M_i}^j = exp(-2 pi i j / M_i), j < M_i, per axis
};
// one strided axis of the padded transforms (see k_fft_axis)
struct Pad32Axis {
  int n, W;
  long long nlines, B, fs, ss, rs;
  // lines that can be nonzero: l = a * ld2 + kz with kz < kzmax and (na > 0) a
  // in the N-grid band of an axis of ma points; ld2 = 0: every line
  long long ld2;
  int kzmax, na, ma;
};
// rhs (caller layout) of u_hat (caller layout), + src if not null; phat
// (NS only, may be null) receives the pressure coefficient P_hat
int pad32_rhs(const Pad32& p, const void* u_hat, const void* src, void* rhs, void* phat, cudaStream_t s);
int pad32_smem_optin(int dev, bool dbl);

// message returned by sdns_last_error() (thread-local)
void set_last_error(const char* msg);

template <typename Real> struct Kernels {
  static int axis_plain(const AxisArgs& a, int sign, cudaStream_t s);
  // x^-1 sweep producing the six fields of the z sweep: NS (vv false) u_hat and
  // i K x u_hat; VV (vv true) i K x w_hat / K^2 and w_hat
  static int axis_curl_inv(const AxisArgs& a, cudaStream_t s, bool vv = false);
  static int zline_ns(const ZArgs& a, cudaStream_t s);
  static int zline_c2r(const ZArgs& a, cudaStream_t s);
  static int zline_r2c(const ZArgs& a, cudaStream_t s);
  static int axis_rk(const RKArgs& a, cudaStream_t s, int* nblocks_out);
  static int rk_update(const RKArgs& a, cudaStream_t s);
  static int smem_optin(int dev);
};

}  // namespace sdns
