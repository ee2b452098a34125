/*
 * sdns_gb300.h -- C ABI of the GB300 (sm_103a) backend for the triply
 * periodic pseudo-spectral Navier-Stokes solver of spectralDNS.
 *
 * One context = one grid on one GPU with one CUDA stream.  All entry points
 * return an int status (SDNS_OK == 0); on failure sdns_last_error() gives a
 * message.  Nothing traps or exits.  Buffers passed by the caller are either
 * host memory (where == SDNS_HOST; pinned memory is fastest) or device memory
 * of the context's GPU (where == SDNS_DEVICE); the call is synchronous with
 * respect to the caller's buffers when they are host memory.
 *
 * Array layouts follow the reference's single-rank numpy arrays (C order):
 *   spectral vector  (3, N0, N1, N2/2+1) complex  -- U_hat, dU, Source
 *   physical vector  (3, N0, N1, N2) real         -- U, curl
 * "complex" is complex64 (SDNS_SINGLE) or complex128 (SDNS_DOUBLE), matching
 * spectralDNS/solvers/spectralinit.py:25-29 (datatypes).
 *
 * Reference interfaces replaced (paths inside the spectralDNS tree):
 *   sdns_create/sdns_destroy  spectralDNS/solvers/NS.py:12-72   get_context
 *   sdns_compute_rhs          spectralDNS/solvers/NS.py:219-261 ComputeRHS (Vortex form,
 *                             NS.py:191-198, with add_pressure_diffusion NS.py:203-217)
 *   sdns_rk4                  spectralDNS/maths/integrators.py:149-159 RK4 (closure :188-191)
 *   sdns_forward              shenfun VT.forward as called at NS.py:101-104 (set_velocity)
 *   sdns_backward             shenfun VT.backward as called at NS.py:91-94  (get_velocity)
 *   sdns_curl                 spectralDNS/solvers/NS.py:86-89, 124-129 (get_curl / compute_curl)
 *   sdns_pressure             spectralDNS/solvers/NS.py:96-99  (get_pressure)
 *   sdns_divergence           spectralDNS/solvers/NS.py:106-110 (get_divergence)
 *   sdns_set_state/get_state  the U_hat array of the context (NS.py:52, 58)
 *   sdns_set_source           the Source array added in ComputeRHS (NS.py:63, 259)
 *   sdns_diagnostics          demo/TG.py:97-103 and demo/Isotropic.py:167, 241-249 reductions
 *   sdns_spectrum             demo/Isotropic.py:88-114 (shell spectrum, bins k+0.5)
 *   formulation SDNS_VV       spectralDNS/solvers/VV.py: the velocity-vorticity solver
 *                             (get_context :23-38, Conv :85-103, add_linear :105-110,
 *                             ComputeRHS :112-146); the context state is W_hat
 *   sdns_velocity_vv          spectralDNS/solvers/VV.py:52-72 (compute_velocity / get_velocity)
 */
#ifndef SDNS_GB300_H
#define SDNS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDNS_ABI_VERSION 1

enum sdns_status {
  SDNS_OK = 0,
  SDNS_EINVAL = 1,   /* bad argument or unsupported configuration */
  SDNS_ECUDA = 2,    /* CUDA runtime error */
  SDNS_ENOMEM = 3,   /* device allocation failed */
  SDNS_ESTATE = 4,   /* call out of order (e.g. no state set) */
  SDNS_ENONFINITE = 5 /* a reduction found NaN/Inf in the solution */
};

enum sdns_precision { SDNS_SINGLE = 0, SDNS_DOUBLE = 1 };
enum sdns_dealias { SDNS_DEALIAS_23 = 0, SDNS_DEALIAS_NONE = 1, SDNS_DEALIAS_32 = 2 };
enum sdns_where { SDNS_HOST = 0, SDNS_DEVICE = 1 };
enum sdns_formulation { SDNS_NS = 0, SDNS_VV = 1 };

typedef struct sdns_ctx sdns_ctx;

typedef struct sdns_config {
  int32_t n[3];          /* grid points per axis, powers of two in [16, 1024] */
  double L[3];           /* box lengths (K scaled by 2 pi / L, NS.py:38) */
  double nu;             /* viscosity */
  int32_t precision;     /* SDNS_SINGLE: FP32 transforms, FP64 RK4 accumulators;
                            SDNS_DOUBLE: everything FP64 */
  int32_t dealias;       /* SDNS_DEALIAS_23 (|k_i| < 2/3 (N_i/2+1)),
                            SDNS_DEALIAS_NONE (Nyquist planes masked) or
                            SDNS_DEALIAS_32: the 3/2 rule (NS.py:29-31 with
                            padding_factor 1.5): the nonlinear term is formed
                            on a 3N/2 grid from all modes but the Nyquist ones
                            and truncated back; fixed dt only (no CFL, no
                            forcing), RK4 steps in the working precision */
  int32_t device;        /* CUDA device ordinal */
  int32_t store_pressure;/* keep P_hat of the last RK4 stage for sdns_pressure (NS) */
  int32_t formulation;   /* SDNS_NS (0): the state is the velocity U_hat and ComputeRHS
                            is NS.py's; SDNS_VV: the state is the vorticity W_hat and
                            ComputeRHS is VV.py's (i K x F(u x w) - nu K^2 W_hat + Source,
                            u = F^-1(i K x W_hat / K^2)); no pressure, no forcing */
  int32_t reserved[3];
} sdns_config;

/* diagnostics written by sdns_diagnostics (float64, full-spectrum sums).  For
 * a SDNS_VV context the energy and divergence are those of the velocity
 * i K x W_hat / K^2 and the enstrophy is 1/2 <w.w> of the state W_hat. */
enum sdns_diag {
  SDNS_DIAG_ENERGY = 0,      /* 1/2 <u.u>              (demo/TG.py:98)  */
  SDNS_DIAG_ENSTROPHY = 1,   /* 1/2 <w.w>              (demo/TG.py:97)  */
  SDNS_DIAG_DISSIPATION = 2, /* nu * energy_fourier(i K x u_hat) (demo/Isotropic.py:241-249) */
  SDNS_DIAG_DIVERGENCE = 3,  /* 1/2 <(div u)^2>        (demo/TG.py:102-103) */
  SDNS_DIAG_CFL_RATE = 4,    /* max |u|/dx+|v|/dy+|w|/dz at the last RK4 step start */
  SDNS_DIAG_TIME = 5,        /* simulated time accumulated by sdns_rk4 */
  SDNS_DIAG_LAST_DT = 6,     /* time step of the last RK4 step */
  SDNS_DIAG_COUNT = 8
};

int sdns_abi_version(void);
const char* sdns_last_error(void);

int sdns_create(const sdns_config* cfg, sdns_ctx** out);
int sdns_destroy(sdns_ctx* ctx);
int sdns_synchronize(sdns_ctx* ctx);
/* the context's CUDA stream (cudaStream_t), for callers that time or order
 * their own work against the solver's kernels */
int sdns_get_stream(sdns_ctx* ctx, void** stream);
/* bytes of device memory held by the context */
int sdns_memory_bytes(sdns_ctx* ctx, int64_t* bytes);

int sdns_set_state(sdns_ctx* ctx, const void* u_hat, int where);
int sdns_get_state(sdns_ctx* ctx, void* u_hat, int where);
/* Source term (NULL clears it); spectral vector layout */
int sdns_set_source(sdns_ctx* ctx, const void* source, int where);

int sdns_compute_rhs(sdns_ctx* ctx, const void* u_hat, void* rhs, int where);

/* Constant-power forcing on 0 < |K| <= kf (a Source recomputed from the
 * state at the start of every RK4 step); eps <= 0 switches it off. */
int sdns_set_forcing(sdns_ctx* ctx, double eps, double kf);
/* CFL time step dt = cfl / max(|u|/dx+|v|/dy+|w|/dz), evaluated on the
 * dealiased velocity at the start of each step; cfl <= 0 switches it off. */
int sdns_set_cfl(sdns_ctx* ctx, double cfl);

/* nsteps classic RK4 steps of size dt (ignored when CFL is on).  The
 * simulated time is accumulated on the device (SDNS_DIAG_TIME). */
int sdns_rk4(sdns_ctx* ctx, double dt, int32_t nsteps);
int sdns_set_time(sdns_ctx* ctx, double t);

/* transforms of nfields (1..3) scalar fields stacked on the first axis */
int sdns_forward(sdns_ctx* ctx, const void* phys, void* spec, int32_t nfields, int where);
int sdns_backward(sdns_ctx* ctx, const void* spec, void* phys, int32_t nfields, int where);
/* physical fields: velocity of the context state; curl and divergence of the
 * spectral vector u_hat (NULL: of the context state); pressure of the last
 * right-hand-side evaluation (needs store_pressure) */
int sdns_velocity(sdns_ctx* ctx, void* u, int where);
/* velocity F^-1(i K x w_hat / K^2) of a vorticity spectral vector w_hat (NULL:
 * the context state, which is W_hat for a SDNS_VV context) */
int sdns_velocity_vv(sdns_ctx* ctx, const void* w_hat, void* u, int where);
int sdns_curl(sdns_ctx* ctx, const void* u_hat, void* curl, int where);
int sdns_pressure(sdns_ctx* ctx, void* p, int where);
int sdns_divergence(sdns_ctx* ctx, const void* u_hat, void* div, int where);

int sdns_diagnostics(sdns_ctx* ctx, double* out /* SDNS_DIAG_COUNT */);
int sdns_spectrum(sdns_ctx* ctx, double* Ek, int32_t nbins);

/* ---- integrator building blocks (spectralDNS/maths/integrators.py:15-147
 * adaptiveRK, :161-165 ForwardEuler, :167-175 AB2, driven from the host as
 * getintegrator :177-239 does).  The stage arrays of these
 * integrators stay on the GPU: every pointer is device memory of the context's
 * GPU holding a spectral vector (3, N0, N1, N2/2+1) of the context precision;
 * both run on the context stream. ---- */
#define SDNS_LINCOMB_MAX 8
/* out = base + sum_k coef[k] * terms[k] (k < nterms <= SDNS_LINCOMB_MAX;
 * base NULL: 0), summed term by term in the working precision as the
 * reference's `u0_new += dt*b[j]*fY_hat[j]` updates (integrators.py:66-68,
 * 78-84, 164, 171-174).  out may alias base or a term. */
int sdns_lincomb(sdns_ctx* ctx, void* out, const void* base, int32_t nterms, const double* coef,
                 const void* const* terms);
/* float64 sums[k] = sum over component k of |err/sc|^2 with
 * sc = atol + max(|u0|, |u1|) * rtol (integrators.py:87-92, errnorm "2");
 * synchronous (the adaptive step needs the estimate on the host). */
int sdns_error_norm(sdns_ctx* ctx, const void* err, const void* u0, const void* u1, double atol, double rtol,
                    double* sums /* 3 */);

/* device time (ms) of the kernels of the last sdns_rk4 call, per kernel
 * class, measured with CUDA events on the context stream when timing is on */
int sdns_set_timing(sdns_ctx* ctx, int32_t on);
int sdns_get_timing(sdns_ctx* ctx, double* ms /* 8 */, int32_t* launches /* 8 */);

/* ---- learned subgrid-stress closure for a coarse LES (no counterpart in the
 * reference; the benchmark's LES case).  Device pointers, caller stream. ---- */
/* box filter of ratio r: fine velocity (3, N0, N1, N2) real -> coarse
 * ubar (3, n0, n1, n2) float and tau (n0*n1*n2, 6) float, tau_ij =
 * bar(u_i u_j) - bar(u_i) bar(u_j) in the order xx yy zz xy xz yz */
int sdns_les_box_filter(const void* u, int32_t precision, const int32_t* N, int32_t ratio, float* ubar, float* tau,
                        void* stream);
/* ghat[3 i + j] = i K_j uhat_i for a spectral vector (3, n0, n1, n2/2+1) */
int sdns_les_grad_hat(const void* uhat, void* ghat, int32_t precision, const int32_t* n, const double* L,
                      void* stream);
/* SGS force -P(i K_j tauhat_ij) * scale from tauhat (6, n0, n1, n2/2+1) */
int sdns_les_sgs_force(const void* tauhat, void* force, int32_t precision, const int32_t* n, const double* L,
                       double scale, void* stream);
/* planar float (nch, P) <-> channels-last (P, cpad): pack -> bf16 with (x - mu) * isd,
 * unpack float -> planar with y * sd + mu */
int sdns_les_pack(const float* x, int32_t nch, int64_t P, int32_t cpad, const float* mu, const float* isd, void* y,
                  void* stream);
int sdns_les_unpack(const float* y, int32_t cpad, int32_t nch, int64_t P, const float* mu, const float* sd, float* x,
                    void* stream);
/* periodic 3x3x3 convolution, channels last, bf16 activations and weights
 * W (27, co, ci), FP32 accumulation; (ci, co) in {(16,32), (32,32), (32,8)};
 * forward writes the FP32 pre-activation y and (optional) the bf16
 * activation yact (ReLU when relu != 0); grid sides multiples of 8 */
int sdns_conv3d_fwd(const void* x, const void* W, const float* b, float* y, void* yact, const int32_t* n, int32_t ci,
                    int32_t co, int32_t relu, void* stream);
int sdns_conv3d_bwd_data(const float* gpre, const void* W, float* gin, const int32_t* n, int32_t ci, int32_t co,
                         void* stream);
/* accumulates (+=) into dW (27, co, ci) and db (co) */
int sdns_conv3d_bwd_weight(const void* x, const float* gpre, float* dW, float* db, const int32_t* n, int32_t ci,
                           int32_t co, void* stream);
int sdns_relu_bwd(const float* gpost, const float* pre, float* gpre, int64_t count, int32_t relu, void* stream);
/* grad = 2 (y - t) / (P nch) over the first nch of cpad channels; *loss += mean square */
int sdns_mse_grad(const float* y, int32_t cpad, int32_t nch, const float* target, int64_t P, float* grad, double* loss,
                  void* stream);
/* Adam step (step >= 1) on FP32 weights; refreshes the bf16 copy when wbf16 != NULL */
int sdns_adam_step(float* w, const float* g, float* m, float* v, int64_t count, float lr, float b1, float b2,
                   float eps, int32_t step, void* wbf16, void* stream);
int sdns_to_bf16(const float* a, void* b, int64_t count, void* stream);

/* ComputeRHS that allocates nothing.  This entry point has no counterpart in
 * the reference.  It serves callers that must not call cudaMalloc: work
 * recorded into a CUDA graph, programs whose framework allocator owns the
 * device memory, real-time loops.  It takes the grid description instead of
 * a context, the caller's device arrays u_hat and rhs (spectral vector
 * layout, complex64 or complex128 per cfg->precision, on device cfg->device)
 * and a cudaStream_t (NULL: the legacy default stream), and enqueues the
 * same computation as sdns_compute_rhs with the Source term zero.  Its
 * scratch is one static device array of SDNS_NOALLOC_SCRATCH_BYTES that every
 * GPU loading the library keeps until the process exits; grids that need
 * more (about 64^3 in double, 64x64x128 in single precision is the limit)
 * are rejected with SDNS_EINVAL, and so are the 3/2 rule and the SDNS_VV
 * formulation.  The first call on a device looks up the
 * array's device address, so make that call before any stream capture.  All
 * calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller.  Errors are reported through sdns_last_error. */
#define SDNS_NOALLOC_SCRATCH_BYTES (32 * 1024 * 1024)
int sdns_compute_rhs_noalloc(const sdns_config* cfg, const void* u_hat, void* rhs, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SDNS_GB300_H */
