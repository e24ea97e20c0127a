/*
 * axs.h — C ABI of the GB300 standard-lattice evolution path of Axion-Strings.
 *
 * The reference has no plugin or FFI layer: its hot path is a set of C++
 * calls inside run_standard() (src/standard/s_run.cpp:26-232) that mutate
 * calloc'd host arrays. Each entry point below replaces one of those calls;
 * the comment names the reference function (file:line) it stands in for.
 *
 * Conventions
 *   - Every function returns an int status: AXS_OK (0) or a negative AXS_ERR_*.
 *     axs_last_error() returns the message of the last failure on the calling
 *     thread. No C++ exception crosses this boundary.
 *   - Lattice state lives on the GPU between calls. Host buffers are plain
 *     arrays in the reference's layout: 2D offset2(i,j) = i + N*j, 3D
 *     offset3(i,j,k) = (i*N + j)*N + k (src/common/common.hpp:88-108).
 *     Offsets are 64-bit (the reference's are int).
 *   - The fields are the reference's rescaled field psi = tau*phi ("phi1",
 *     "phi2") and its conformal-time derivative ("phidot1", "phidot2"),
 *     exactly the arrays of struct _all_data (src/standard/s_internal.hpp:6-20).
 *   - One CUDA stream per handle; calls on one handle are not thread-safe,
 *     calls on different handles may come from different threads.
 *     Calls that return host results synchronise that stream.
 */
#ifndef AXS_H
#define AXS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define AXS_OK               0
#define AXS_ERR_ARG         -1   /* invalid argument or unsupported size            */
#define AXS_ERR_CUDA        -2   /* CUDA runtime or cuFFT failure                   */
#define AXS_ERR_NOMEM       -3   /* device or host allocation failed                */
#define AXS_ERR_STATE       -4   /* call not valid in the handle's current state    */
#define AXS_ERR_NONFINITE   -5   /* NaN or Inf found in the fields                  */
#define AXS_ERR_TIMEOUT     -6   /* a device-side wait gave up (kernel returned)    */
#define AXS_ERR_PARSE       -7   /* parameter file error                            */

/* ---- precision of the device state ---------------------------------------- */
#define AXS_F32 32   /* psi, pi stored and stepped in FP32; reductions FP64/Kahan */
#define AXS_F64 64   /* plain FP64 step                                           */

/* ---- field ids ------------------------------------------------------------ */
#define AXS_PHI1     0
#define AXS_PHI2     1
#define AXS_PHIDOT1  2
#define AXS_PHIDOT2  3

/*
 * Lattice parameters. The first ten members are the fields of the reference's
 * `struct parameters` (src/common/common.hpp:30-69) that the hot path reads,
 * with the same names, types and meaning. The rest are additions.
 */
typedef struct axs_params {
    float        lambda;           /* quartic coupling                                  */
    int          enable_PRS;       /* read and ignored by the standard path, as in the reference */
    float        T_initial;        /* T_0: thermal mass term and thermal init           */
    int          NDIMS;            /* 2 or 3                                            */
    int          N;                /* points per side, even, >= 4; at most 4096 (3D) or */
                                   /* 32768 (2D)                                        */
    float        space_step;       /* dx                                                */
    float        time_step;        /* dt                                                */
    int          stencil_setting;  /* 0..3 -> stencil radius 1..4                       */
    unsigned int seed;             /* initial-condition seed                            */
    int          thr;              /* string-finder threshold percent                   */
    /* additions */
    int          precision;        /* AXS_F32 or AXS_F64                                */
    int          prs;              /* potential coefficient lambda / tau^(2*prs):
                                      1 = the reference's standard integrator,
                                      0 = the unrescaled-coupling (physical) equation */
    double       tau_initial;      /* starting conformal time (the reference uses 1)    */
    int          form;             /* equation of motion: 0 = field-rescaled psi = tau phi
                                      (vvsl_field_rescaled, s_integrate.cpp:305-348),
                                      1 = Hamiltonian-like form in phi and pi = tau^2 phi'
                                      (vvsl_hamiltonian_form, s_integrate.cpp:358-395) */
    int          laplacian;        /* 0 = finite-difference stencil (stencil_setting,
                                      build_coefficient_matrix, s_integrate.cpp:5-149),
                                      1 = spectral (compute_laplacian_fft, s_integrate.cpp:179-296,
                                      the reference's compile-time alternative at :327-329) */
} axs_params;

typedef struct axs_lattice axs_lattice;     /* one lattice on the GPU            */
typedef struct axs_ensemble axs_ensemble;   /* independent lattices, batched     */

/* Fill p with the values of the reference's default.param plus
 * precision = AXS_F64, prs = 1, tau_initial = 1, form = 0, laplacian = 0. */
void axs_default_params(axs_params *p);

/* Copy the message of the last failure on this thread into buf. */
int axs_last_error(char *buf, size_t len);

/* ---- lifetime --------------------------------------------------------------- */

/* Allocate the device state of one lattice on the current CUDA device.
 * Replaces the calloc of the 8 field arrays and build_coefficient_matrix
 * (s_run.cpp:35-53, src/standard/s_integrate.cpp:5-149): no matrix is built,
 * the stencil is applied directly. Fields start at zero, tau at tau_initial. */
int axs_create(const axs_params *p, axs_lattice **out);
int axs_destroy(axs_lattice *h);

/* ---- state transfer (host arrays of N^NDIMS values; NULL skips a field) ------ */

/* Set the state from host arrays. Like a freshly initialised reference run,
 * the next step is a pure drift (the reference's ker_curr arrays are zero
 * after calloc: s_run.cpp:44-47, s_integrate.cpp:313-314). tau and the step
 * counter are left as they are. When all four arrays are given, that drift is
 * formed while the momentum is transferred (the next axs_evolve then starts
 * from it); the results are the same bits as drifting in the first step. */
int axs_upload(axs_lattice *h, const double *phi1, const double *phi2,
               const double *phidot1, const double *phidot2);
int axs_upload_f32(axs_lattice *h, const float *phi1, const float *phi2,
                   const float *phidot1, const float *phidot2);
/* Copy the synchronised state (fields and derivatives at the current tau,
 * what the reference's arrays hold between steps) to host arrays. */
int axs_download(axs_lattice *h, double *phi1, double *phi2, double *phidot1, double *phidot2);
int axs_download_f32(axs_lattice *h, float *phi1, float *phi2, float *phidot1, float *phidot2);

/* Current conformal time and number of steps taken (physics.cpp globals). */
int axs_get_time(axs_lattice *h, double *tau, int64_t *steps);
/* Set tau and the step counter (used when resuming). */
int axs_set_time(axs_lattice *h, double tau, int64_t steps);

/* ---- initial conditions ------------------------------------------------------- */

/* gaussian_thermal (src/common/init.cpp:33-200): Bose-Einstein amplitudes at
 * T_initial for phi and phidot, inverse FFT, checkerboard shift, 1/N^d.
 * The deviates are the project's Philox-4x32-10 + Box-Muller stream, not MKL
 * SFMT19937. The 3D k=0 phidot amplitude (never set by init.cpp:163-164,
 * which assign the phi amplitude twice) is 0; the reference as compiled keeps
 * the previous mode's value there, a constant offset of its phidot. Resets
 * tau to tau_initial and the step counter to 0. */
int axs_init_gaussian_thermal(axs_lattice *h, uint64_t seed);
/* Flat spectrum for 0 < |k| < kcut (k = 2 pi n / L), zero elsewhere, scaled
 * to <|phi|^2> = 1 at tau_initial, phidot = 0 (no reference counterpart). */
int axs_init_flat(axs_lattice *h, uint64_t seed, double kcut);

/* ---- evolution ---------------------------------------------------------------- */

/* nsteps calls of vvsl_field_rescaled (src/standard/s_integrate.cpp:305-348),
 * fused into one kernel per step; tau advances by (double)dt per step as at
 * s_integrate.cpp:317. Runs asynchronously on the handle's stream (captured
 * once into a CUDA graph per distinct nsteps). */
int axs_evolve(axs_lattice *h, int nsteps);
/* axs_evolve with the device time of the steps measured by CUDA events on
 * the handle's stream; synchronises. */
int axs_evolve_timed(axs_lattice *h, int nsteps, double *ms);

/* (1/dx^2) A phi for one field, A the matrix of build_coefficient_matrix
 * applied as at s_integrate.cpp:322 (the operator of src/tests/laplacian.cpp
 * and src/tests/fdm_matrix.cpp). out: N^NDIMS doubles. */
int axs_laplacian(axs_lattice *h, int field, double *out);

/* ---- string finding ------------------------------------------------------------ */

/* cores2 / cores3 (src/common/string_finding.cpp:3-86) on
 * theta = atan2(phi1, phi2) (s_run.cpp:94), or on a caller-supplied theta
 * (N^NDIMS doubles) when theta != NULL. The plaquette decision is bit-exact
 * to the reference's double arithmetic on a given theta.
 *   mask           optional, N^NDIMS bytes: 1 where the cell is flagged
 *   n_plaquettes   number of flagged cells (cores2/cores3's return value)
 *   num_cores      2D: n_plaquettes minus neighbouring pairs in ascending
 *                  offset order (s_run.cpp:101-109); 3D: n_plaquettes */
int axs_find_strings(axs_lattice *h, const double *theta, uint8_t *mask,
                     int64_t *n_plaquettes, int64_t *num_cores);
/* Positions of the flagged cells of the last axs_find_strings, in ascending
 * offset order (the order of a serial cores2/cores3 list), NDIMS ints each:
 * 2D (i,j), 3D (i,j,k) as vec2i/vec3i (src/common/common.hpp:71-72).
 * Writes min(cap, n) entries; *n = total. */
int axs_string_positions(axs_lattice *h, int32_t *pos, int64_t cap, int64_t *n);
/* xi exactly as run_standard computes it in float (s_run.cpp:111-114, 123-129). */
int axs_xi(const axs_params *p, int64_t n_plaquettes, int64_t num_cores, double tau, float *xi);

/* ---- spectra ---------------------------------------------------------------------- */

/* output_powerspec(field, NULL) (src/common/pk_estimation.cpp:37-214):
 * forward FFT, bins floor(|n|)-1 for 0 < |n| < N/2, pk /= 2 pi <|n|> (2D) or
 * 4 pi <|n|>^2 (3D), ks = <|n|> 2 pi / L. Arrays of N/2 entries; empty bins
 * hold count 0 (and NaN pk/ks, as the reference computes them). */
int axs_powerspec(axs_lattice *h, int field, double *pk, double *ks, int *count);
/* Axion kinetic-energy spectrum (no reference counterpart): f = |phi| theta'
 * = (psi2 pi1 - psi1 pi2)/(tau |psi|), FFT, nbins log-spaced |k| bins from
 * 2 pi / L to sqrt(NDIMS) pi / dx; pk = L^d / N^(2d) <|F|^2>_bin. FP64 sums. */
int axs_axion_spectrum(axs_lattice *h, int nbins, double *kmean, double *pk, int64_t *count);

/* Allocation-free variant of the spectrum binning in axs_powerspec. No
 * counterpart in the reference: it exists for callers that own all device
 * memory and cannot let this library call cudaMalloc or cudaFree (hosts that
 * budget the device up front, frameworks whose caching allocator must be the
 * only source of device memory, codes that cannot absorb the device-wide
 * synchronisation of a cudaFree).
 *   spectrum   device pointer to the R2C half spectrum of a real N^NDIMS field
 *              as cuFFT writes it (cufftComplex for AXS_F32, cufftDoubleComplex
 *              for AXS_F64; [N][N/2+1] in 2D, [N][N][N/2+1] in 3D)
 *   pk, ks, count   device arrays of N/2 entries, filled as axs_powerspec fills
 *              its host arrays (output_powerspec's bins and normalisation)
 *   stream     cudaStream_t to run on (NULL: the legacy default stream); the
 *              call is asynchronous on it
 * It allocates nothing: its scratch is a static device array of 2 MiB + 8 KiB
 * per GPU, held from library load to process exit, which limits it to N <= 2048
 * (larger N is rejected with AXS_ERR_ARG). The first call on each device does
 * a one-time set-up with that device current (it looks up the array's device
 * address); make that first call before any stream capture. All calls share
 * the array, which keeps the last call's contents (the counts are cleared on
 * every call): calls in order on one stream are independent; calls that
 * overlap on the GPU race and give wrong results. */
int axs_powerspec_noalloc(const void *spectrum, int NDIMS, int N, int precision, float space_step,
                          double *pk, double *ks, int *count, void *stream);

/* ---- reductions -------------------------------------------------------------------- */

/* The six background means of s_run.cpp:135-150: phi1, phi2, phidot1, phidot2,
 * |atan2(phi1,phi2)|, |phi|. Deterministic FP64 (Kahan-compensated FP32 per
 * thread on the FP32 path). The phidot means equal the means of the per-site
 * synchronised momentum to rounding; they are formed from the means of pih
 * and of the local part of the half kick, plus the stencil weights' sum times
 * the mean field (the Laplacian's share on a periodic lattice), so the call
 * streams the state once. */
int axs_background(axs_lattice *h, double out[6]);
/* Mean kinetic, gradient and potential energy densities of phi = psi/tau
 * (no reference counterpart). */
int axs_energies(axs_lattice *h, double out[3]);
/* *finite = 1 when no NaN/Inf is in the fields (the check of s_run.cpp:4-12). */
int axs_check_finite(axs_lattice *h, int *finite);

/* Distance between the synchronised states of two lattices of the same shape
 * (any precisions; no reference counterpart): for each field f of (phi1, phi2,
 * phidot1, phidot2), out[2f] = sum (a_f - b_f)^2 and out[2f+1] = sum b_f^2,
 * FP64 with a fixed reduction order. Used to state FP32 errors against FP64. */
int axs_field_distance(axs_lattice *a, axs_lattice *b, double out[8]);

/* ---- checkpoint / resume (no reference counterpart on the standard path) ----------- */

/* Bytes needed for a checkpoint of this lattice. */
int axs_checkpoint_size(axs_lattice *h, size_t *bytes);
/* Serialise the exact device state (including the leapfrog stage) into buf;
 * axs_restore continues bit-identically. */
int axs_checkpoint(axs_lattice *h, void *buf, size_t bytes);
int axs_restore(axs_lattice *h, const void *buf, size_t bytes);

/* ---- batched ensembles ----------------------------------------------------------------- */

/* n independent lattices (sizes, lambdas, seeds may differ; dt, dx,
 * precision and dimension must agree) stepped together by one persistent
 * kernel launch per step. Member results are bit-identical to the same
 * lattice stepped alone. */
int axs_ensemble_create(const axs_params *members, int n, axs_ensemble **out);
int axs_ensemble_destroy(axs_ensemble *e);
/* Borrowed handle of member i for init, transfer, strings, spectra and
 * reductions; do not destroy it. Do not evolve it alone while it belongs
 * to an ensemble. */
int axs_ensemble_member(axs_ensemble *e, int i, axs_lattice **out);
int axs_ensemble_evolve(axs_ensemble *e, int nsteps);
int axs_ensemble_evolve_timed(axs_ensemble *e, int nsteps, double *ms);
/* axs_find_strings of every member in one call (cores2/cores3,
 * string_finding.cpp:3-86, per member): n_plaquettes[i], num_cores[i] for
 * member i. The members' kernels run back to back with one synchronisation;
 * the results are those of the per-member calls. */
int axs_ensemble_find_strings(axs_ensemble *e, int64_t *n_plaquettes, int64_t *num_cores);
/* axs_axion_spectrum of every member in one call: member i's bins at
 * kmean/pk/count[i*nbins ..]; one synchronisation, the per-member bits. */
int axs_ensemble_axion_spectrum(axs_ensemble *e, int nbins, double *kmean, double *pk, int64_t *count);

/* ---- tuning and diagnostics ------------------------------------------------------------ */

/* Time the candidate tile shapes / pipeline depths for this lattice with
 * dt = 0 steps (the state is unchanged) and keep the fastest. Runs once
 * automatically before the first step unless AXS_AUTOTUNE=0. */
int axs_autotune(axs_lattice *h);
/* Fault injection for tests of the failure path (no reference counterpart):
 * the next step's TMA loads expect 16 bytes more than they deliver, so the
 * step kernel's bounded mbarrier waits (about a second each) run out; the
 * kernel records the timeout, drains its own copies and returns, and the next
 * synchronising call (axs_evolve_timed, axs_download, ...) returns
 * AXS_ERR_TIMEOUT. The CUDA context stays usable; the lattice's state after
 * that step is undefined. Requires the TMA step kernel (AXS_ERR_STATE
 * otherwise). */
int axs_inject_wait_timeout(axs_lattice *h);
/* Describe the step kernel configuration in use (for logs and benches). */
int axs_describe(axs_lattice *h, char *buf, size_t len);
/* The same for an ensemble's one launch per step (no reference counterpart). */
int axs_ensemble_describe(axs_ensemble *e, char *buf, size_t len);
/* Number of kernels this library launched since load (graph replays count
 * every kernel node they run). */
int64_t axs_kernel_launches(void);

/* Make CUDA device `device` current for this thread (handles are created on
 * the current device). */
int axs_set_device(int device);

/* Page-locked host buffers for fast transfers (cudaMallocHost). */
int axs_host_alloc(size_t bytes, void **out);
int axs_host_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
