/*
 * s2d.h -- C-ABI of the GB300 (sm_103a) Spectral2D time-step library.
 *
 * Drop-in replacement for the hot path of mpclay/Spectral2D: the
 * vorticity-streamfunction right-hand side and the TVD (Shu-Osher) RK3 step.
 * Plain C types only (no C++ or framework types), so Fortran binds it through
 * ISO_C_BINDING (scalars by VALUE, arrays as assumed-size or TYPE(C_PTR)),
 * and Python through ctypes.
 *
 * Array conventions at the boundary are the reference's:
 *   - a spectral field is the Fortran array COMPLEX(C_DOUBLE_COMPLEX)
 *     (cISize, nyG), i.e. interleaved (re, im) doubles with the kx index
 *     contiguous; cISize = nxG/2+1, nyG = 3*ny/2 (src/Spectral.F90:162-190);
 *   - row j holds ky = j for j <= nyG/2 and j - nyG above
 *     (src/Spectral.F90:209-218);
 *   - forward transforms are normalised by nxG*nyG, inverse transforms are
 *     not (src/Spectral.F90:749-781).
 *
 * Every entry point returns S2D_OK (0) or a negative S2D_ERR_* code and sets a
 * per-thread message readable with s2d_last_error().  A handle owns all its
 * device memory and one CUDA stream; it is not thread-safe, separate handles
 * may be used from separate threads.  Host arrays are borrowed for the
 * duration of a call only.
 */
#ifndef S2D_H
#define S2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define S2D_API __declspec(dllexport)
#else
#define S2D_API __attribute__((visibility("default")))
#endif

/* ---- status codes ------------------------------------------------------ */
#define S2D_OK                 0
#define S2D_ERR_INVALID       -1   /* bad argument, size or null pointer      */
#define S2D_ERR_CUDA          -2   /* a CUDA runtime call failed              */
#define S2D_ERR_NONFINITE     -3   /* NaN/Inf detected in the state           */
#define S2D_ERR_TIMEOUT       -4   /* a bounded device wait gave up           */
#define S2D_ERR_UNSUPPORTED   -5   /* option the reference leaves unimplemented */
#define S2D_ERR_NOMEM         -6   /* device or host allocation failed        */

/* ---- dealiasing (values of src/Spectral.F90:41-47) --------------------- */
#define S2D_NO_DEALIASING      0
#define S2D_DEALIAS_3_2_RULE   1

/* ---- arithmetic of the FFTs and products ------------------------------- */
#define S2D_FP64               0   /* the reference's precision (RWPC=C_DOUBLE) */
#define S2D_FP32               1   /* FP32 FFTs/products; 1/k^2 stays FP64      */

/* ---- form of the nonlinear term ---------------------------------------- *
 * BASDEVANT: N = (kx^2-ky^2) F[uv] + kx ky F[v^2-u^2]  (4 FFTs per RHS).
 * CONSERVATIVE: N = -i kx F[u w] - i ky F[v w]         (5 FFTs per RHS), the
 * reference's form (src/Spectral.F90:424-479).  The two are the same
 * polynomial identity for divergence-free fields, and on the 3/2 grid the
 * only aliased products that reach retained modes (|k| = nx/2 on an axis)
 * are multiplied by zero in both, so they agree to round-off.            */
#define S2D_NL_BASDEVANT       0
#define S2D_NL_CONSERVATIVE    1

/* ---- initial-condition spectra ----------------------------------------- */
#define S2D_SPECTRUM_SCHUMANN  0   /* 1.5 urms^2 (k/k0) exp(-k/k0), SetIC.F90:374-381 */
#define S2D_SPECTRUM_K4_GAUSS  1   /* k^4 exp(-2 (k/k0)^2)                             */

/* Output of GetGridSize (src/Spectral.F90:117-219). */
typedef struct s2d_grid {
    int32_t nx, ny, dealias;
    int32_t nxG, nyG;
    int32_t kxLG, kyLG, kxMG, kyMG;
    int32_t kxLU, kyLU, kxMU, kyMU;
    double  kMax;
    int32_t rISize, cISize;
} s2d_grid;

/* Run-time configuration.  The reference fixes these as compile-time
 * PARAMETERs of the driver (src/Spectral2D.F90:70-127). */
typedef struct s2d_config {
    int32_t nx, ny;          /* nominal grid; nx == ny, multiple of 8          */
    int32_t dealias;         /* S2D_DEALIAS_3_2_RULE (the only working option) */
    int32_t precision;       /* S2D_FP64 or S2D_FP32                           */
    double  nu;              /* kinematic viscosity                            */
    double  alpha;           /* linear drag: dW -= alpha*w (0 = off)           */
    double  forcing_amp;     /* vorticity source amp*cos(kf*y) (0 = off)       */
    int32_t forcing_k;       /* kf                                             */
    int32_t device;          /* CUDA device ordinal                            */
    int32_t nonlinear_form;  /* S2D_NL_BASDEVANT (default) or S2D_NL_CONSERVATIVE */
} s2d_config;

typedef struct s2d_handle s2d_handle;

/* Library version (major*10000 + minor*100 + patch). */
S2D_API int s2d_version(void);

/* Message of the last failing call on this thread ("" if none). */
S2D_API const char* s2d_last_error(void);

/* GetGridSize -- src/Spectral.F90:117-219.  Host only. */
S2D_API int s2d_get_grid_size(int32_t nx, int32_t ny, int32_t dealias, s2d_grid* out);

/* Set up one simulation: replaces GetGridSize + GetAllocSize + SetupMask +
 * SetupTruncation + TimeIntegrationSetup + SetupPlans
 * (src/Spectral2D.F90:263-307; src/Alloc.F90:62-122; src/Spectral.F90:229-353;
 * src/TimeIntegration.F90:79-108).  The state starts at zero. */
S2D_API int s2d_create(const s2d_config* cfg, s2d_handle** out);

/* Free all device memory of the handle (SpectralFinalize +
 * TimeIntegrationFinalize, src/Spectral.F90:805-813,
 * src/TimeIntegration.F90:218-233). */
S2D_API void s2d_destroy(s2d_handle* h);

/* Load the vorticity wC from a host array in the reference layout
 * (cISize, nyG) complex128.  Modes outside |k| <= nx/2 are dropped (the
 * reference truncates them at the end of every step,
 * src/TimeIntegration.F90:208). psiC is derived from wC
 * (src/Spectral.F90:508-560) and is not an input. */
S2D_API int s2d_set_state(s2d_handle* h, const double* wC, int32_t cISize, int32_t nyG);

/* Store wC and psiC (either may be NULL) into host arrays in the reference
 * layout; every mode outside the retained set is written as zero.  psiC is
 * ComputePsi + Truncate of wC (src/TimeIntegration.F90:205-209). */
S2D_API int s2d_get_state(s2d_handle* h, double* wC, double* psiC, int32_t cISize, int32_t nyG);

/* IntegrateOneStep -- src/TimeIntegration.F90:130-210.  Advances the
 * device-resident state by one TVD-RK3 step of size dt.  Asynchronous on the
 * handle's stream. */
S2D_API int s2d_integrate_one_step(s2d_handle* h, double dt);

/* n calls of IntegrateOneStep, replayed from a CUDA graph of one step
 * (the graph is rebuilt when dt changes).  Asynchronous. */
S2D_API int s2d_integrate_steps(s2d_handle* h, int32_t n, double dt);

/* IntegrateOneStep with the reference's host arrays, for callers that keep
 * wC/psiC on the host: wC (in/out) and psiC (out), reference layout.  Only
 * the retained rectangle of wC is read; the truncated part of both outputs is
 * written as zero while the step runs.  Synchronises before returning.
 *
 * Host arrays in every call of this header (set/get_state, compute_rhs, this
 * one) are read and written in place by the kernels where the device can
 * address them: page-locked memory, and ordinary pageable memory whose pages
 * are resident on systems whose GPU reads the host page tables (Grace,
 * cudaDevAttrPageableMemoryAccess); otherwise through staging copies.  The
 * environment variable S2D_HOST_IO=copy, read by s2d_create, forces the
 * copies for that handle.
 *
 * Every kernel of a step is launched as a programmatic dependent of the one
 * before it on the handle's stream (it waits for its predecessor to complete
 * before touching memory, so results are the same bit for bit);
 * S2D_PDL=0, read by s2d_create, gives plain stream order. */
S2D_API int s2d_integrate_one_step_host(s2d_handle* h, double* wC, double* psiC,
                                        int32_t cISize, int32_t nyG, double dt);

/* ComputeRHS -- src/Spectral.F90:396-482.  dW of the current state, written
 * to a host array in the reference layout (zero outside the retained set). */
S2D_API int s2d_compute_rhs(s2d_handle* h, double* dW, int32_t cISize, int32_t nyG);

/* ComputeSpectrum -- src/Analysis.F90:267-460 (velocity from psi as in
 * src/Analysis.F90:230-234).  Ek has nbins entries (bin centres 0..nbins-1);
 * nbins must equal s2d_spectrum_bins().  Any output may be NULL. */
S2D_API int s2d_spectrum_bins(const s2d_handle* h);
S2D_API int s2d_spectrum(s2d_handle* h, double* Ek, int32_t nbins,
                         double* tke, double* eps, double* enstDiss);

/* Mean enstrophy 1/2 <omega^2> of the current state (no reference counterpart). */
S2D_API int s2d_enstrophy(s2d_handle* h, double* enstrophy);

/* max|wC|, min|wC|, max|psiC|, min|psiC| over the reference array, as the
 * driver prints every printPeriod steps (src/Spectral2D.F90:358-367). */
S2D_API int s2d_minmax_abs(s2d_handle* h, double out[4]);

/* SetTaylorGreen -- src/SetIC.F90:70-101 (with the 1-based grid offset of
 * :91-94).  Sets the device state. */
S2D_API int s2d_set_taylor_green(s2d_handle* h);

/* SetTurbulentVelocity -- src/SetIC.F90:125-151, :175-364, with a
 * reproducible counter-based phase per (seed, kx, ky), a Hermitian kx=0
 * column, and omega scaled so that ComputeSpectrum's TKE equals tke
 * (no scaling when tke <= 0).  Sets the device state. */
S2D_API int s2d_set_turbulent(s2d_handle* h, uint64_t seed, int32_t spectrum,
                              double k0, double urms, double tke);

/* The same generator writing wC into a host array (reference layout);
 * needs no GPU. */
S2D_API int s2d_turbulent_ic_host(int32_t nx, uint64_t seed, int32_t spectrum,
                                  double k0, double urms, double tke, double* wC);

/* CFL time step cfl / max(|u|/dx + |v|/dy) over the nxG x nyG collocation
 * grid of the current state.  Fills the empty ComputeTimeStep stub
 * (src/TimeIntegration.F90:213-215).  Synchronises. */
S2D_API int s2d_cfl_dt(s2d_handle* h, double cfl, double* dt);

/* x and y vorticity-gradient skewness of Analysis (src/Analysis.F90:135-225):
 * -2 <a b^2> / (sqrt(<a^2>) <b^2>) with (a, b) = (du/dx, dw/dx) and
 * (dv/dy, dw/dy) on the collocation grid.  Either output may be NULL. */
S2D_API int s2d_skewness(s2d_handle* h, double* xskew, double* yskew);

/* S2D_ERR_NONFINITE if a NaN/Inf was written to the state since the last
 * call (flag raised on the device by the stage update); clears the flag. */
S2D_API int s2d_check_finite(s2d_handle* h);

/* Block until all work queued on the handle's stream has finished. */
S2D_API int s2d_synchronize(s2d_handle* h);

/* Run n steps and time them with CUDA events on the handle's stream;
 * *ms receives the elapsed time.  If kernel_ms is non-NULL it receives the
 * summed device time of each kernel class over the n steps:
 * [0] inverse y-pass, [1] x-pass with product, [2] forward y-pass with the
 * stage update. */
S2D_API int s2d_time_steps(s2d_handle* h, int32_t n, double dt, double* ms,
                           double* kernel_ms);

/* Radix order of the handle's FFTs (M = 2^a 3^b): plan 0 (the default) runs
 * the radix-3 passes first -- the first one pruned for the truncated
 * spectra of the inverse transforms -- then a radix-2 pass when a is odd,
 * then radix-4 passes; plan 1 puts the radix-2 pass last; plan 2 runs the
 * radix-2 and radix-4 passes first and the radix-3 passes last (no pruned
 * pass).  Plans round differently (results agree to round-off, not bit for
 * bit).  s2d_set_fft_plan rebuilds the twiddle tables (synchronises; not
 * with a closure attached); s2d_tune_fft_plan times every plan on this
 * handle's step with time step dt (its state is restored), keeps the
 * fastest, and writes it and, when ms is not NULL, each plan's ms per step
 * (S2D_FFT_PLANS entries) -- the autotuner of the radix schedule, the part
 * of FFTW_MEASURE planning (src/Spectral.F90:340-349) that applies here. */
#define S2D_FFT_PLANS 3
S2D_API int s2d_set_fft_plan(s2d_handle* h, int32_t plan);
S2D_API int s2d_get_fft_plan(const s2d_handle* h, int32_t* plan);
S2D_API int s2d_tune_fft_plan(s2d_handle* h, double dt, int32_t* plan, double* ms);

/* Kernels launched per RK3 step (for launch accounting). */
S2D_API int s2d_kernels_per_step(const s2d_handle* h);

/* Page-locked host memory for fast host<->device copies. */
S2D_API int s2d_host_alloc(size_t bytes, void** ptr);
S2D_API int s2d_host_free(void* ptr);

/* Measured FP64 throughput of this GPU (a register-resident FMA loop),
 * in TFLOP/s (2 flops per FMA). */
S2D_API int s2d_probe_fp64_peak(int32_t device, double* tflops);

/* ---- checkpoints and restart files -------------------------------------- *
 * Checkpoint: the spectral state and run parameters; reading it back resumes
 * the run bit for bit (the reference writes restarts but cannot read them,
 * src/IO.F90:98-143).
 * Restart: the physical fields Omega, Psi, u, v on the collocation grid with
 * nx, ny, nadv, time, nu (the content of src/IO.F90:306-424) as
 * <root>_<num:08d>.bin (64-byte header, four little-endian float64 arrays,
 * x fastest) plus an XDMF sidecar <root>_<num:08d>.xmf.  s2d_read_restart
 * reloads Omega through the forward transform. */
S2D_API int s2d_checkpoint_write(s2d_handle* h, const char* path, int64_t nadv, double time);
S2D_API int s2d_checkpoint_read(s2d_handle* h, const char* path, int64_t* nadv, double* time);
S2D_API int s2d_write_restart(s2d_handle* h, const char* root, int32_t num, int64_t nadv, double time);
S2D_API int s2d_read_restart(s2d_handle* h, const char* path, int64_t* nadv, double* time);

/* ---- ensembles of independent runs (no reference counterpart) ----------- *
 * A batch advances nruns independent simulations of uneven sizes (nx a power
 * of two in [16, 2048]; each run its own nu, drag and forcing; one precision
 * and device for all) with one persistent kernel launch per RK3 stage, the
 * three launches of a step replayed from a CUDA graph.  Each run is an
 * ordinary handle (s2d_batch_run) on the batch's stream, so the single-run
 * calls (set/get state, ICs, CFL, spectrum) work on it; they are ordered
 * with the batch's launches. */
typedef struct s2d_batch s2d_batch;
S2D_API int s2d_batch_create(int32_t nruns, const s2d_config* cfgs, s2d_batch** out);
S2D_API void s2d_batch_destroy(s2d_batch* b);
S2D_API int s2d_batch_size(const s2d_batch* b);
S2D_API int s2d_batch_run(s2d_batch* b, int32_t i, s2d_handle** h);
/* per-run time steps dt[nruns] used by the following steps */
S2D_API int s2d_batch_set_dt(s2d_batch* b, const double* dt);
/* n RK3 steps of every run (asynchronous) */
S2D_API int s2d_batch_integrate_steps(s2d_batch* b, int32_t n);
/* n steps timed with CUDA events on the batch stream */
S2D_API int s2d_batch_time_steps(s2d_batch* b, int32_t n, double* ms);
/* S2D_ERR_TIMEOUT if a dependency wait of the persistent kernel gave up,
 * S2D_ERR_NONFINITE if a run produced NaN/Inf; clears the flags. */
S2D_API int s2d_batch_status(s2d_batch* b);
S2D_API int s2d_batch_synchronize(s2d_batch* b);
/* Autotuner: first the FFT radix plan of each run size (every plan of
 * s2d_set_fft_plan, one size at a time; skipped with a closure attached),
 * then the tile schedule (128/256/512 threads per CTA, i.e. transforms per
 * tile, and 1-4 CTAs per SM), each timed on this ensemble; keeps the fastest
 * and restores every run's state.  The chosen plans are read with
 * s2d_get_fft_plan on the run handles.  Any output may be NULL. */
S2D_API int s2d_batch_tune(s2d_batch* b, int32_t* threads, int32_t* ctas_per_sm, double* ms_per_step);
/* Fault injection for tests, made on the host: the x-pass tiles of run
 * `run` wait for an inverse y-pass tile that does not exist, so every step
 * takes about one bounded wait (~1 s) per stage and s2d_batch_status then
 * reports S2D_ERR_TIMEOUT; that run's state is not advanced correctly, the
 * others are.  run = -1 removes the stall. */
S2D_API int s2d_batch_inject_stall(s2d_batch* b, int32_t run);

/* ---- learned subgrid closure for coarse LES (no reference counterpart) -- *
 * Sharp spectral filter of a DNS state to an LES grid (a Truncate-style mask
 * of radius nx_les/2, src/Spectral.F90:788-802), the subgrid vorticity flux
 * Pi^ = T[N_dns(w)] - N_les(T w) (N = F[u . grad w]), and a 6-layer circular
 * 3x3 CNN (2 -> 32 x 5 -> 1 channels, GELU, BF16 activations and weights,
 * FP32 accumulation, Adam) that predicts Pi from the filtered (w, psi) on the
 * LES collocation grid.  Handles that make training data (DNS and LES) must
 * be FP64; an LES advanced with a closure may be FP64 or FP32. */
typedef struct s2d_cnn s2d_cnn;
/* grid = LES collocation grid (3*nx_les/2); max_batch = largest batch
 * (max_batch * grid^2 * 32 < 2^31) */
S2D_API int s2d_cnn_create(int32_t grid, int32_t max_batch, uint64_t seed, int32_t device, s2d_cnn** out);
S2D_API void s2d_cnn_destroy(s2d_cnn* c);
S2D_API int s2d_cnn_num_params(const s2d_cnn* c);
/* parameters per layer: W[co][tap][ci] (tap = 3(dy+1)+(dx+1)) then b[co], FP32 */
S2D_API int s2d_cnn_get_params(s2d_cnn* c, float* params);
S2D_API int s2d_cnn_set_params(s2d_cnn* c, const float* params);
/* normalisation: rms of w, psi and Pi (inputs divided, output multiplied) */
S2D_API int s2d_cnn_set_scales(s2d_cnn* c, const double* rms3);
S2D_API int s2d_cnn_get_scales(const s2d_cnn* c, double* rms3);
/* band of the closure term in the LES: modes with |k| < k_min get none
 * (default 0: every retained mode) */
S2D_API int s2d_cnn_set_band(s2d_cnn* c, double k_min);
S2D_API int s2d_cnn_get_band(const s2d_cnn* c, double* k_min);
/* x: batch x grid x grid x 2 (w, psi); y: batch x grid x grid (Pi) */
S2D_API int s2d_cnn_forward_host(s2d_cnn* c, const float* x, int32_t batch, float* y);
/* Forward passes without a gradient (s2d_cnn_forward_host, s2d_cnn_eval, the
 * LES closure term): on != 0 (the default) runs all six layers in one
 * persistent cooperative launch with the activations in two images carrying
 * a circular one-pixel frame; 0 runs one launch per layer, the kernels of the
 * gradient path.  Both give the same bits. */
S2D_API int s2d_cnn_set_fused(s2d_cnn* c, int32_t on);
/* Fault injection for tests, made on the host: with on != 0, CTA 0 of every
 * fused forward skips its first grid-barrier arrival, so the other CTAs'
 * bounded waits (about 1 s) run out, the forward's output is garbage and
 * s2d_cnn_status reports S2D_ERR_TIMEOUT; on = 0 removes it (each launch
 * starts its barrier count from zero, so the next forward is clean). */
S2D_API int s2d_cnn_inject_stall(s2d_cnn* c, int32_t on);
/* MSE loss of the normalised output against target/rms_Pi and its gradient
 * (same layout as the parameters) */
S2D_API int s2d_cnn_grad_host(s2d_cnn* c, const float* x, const float* target, int32_t batch, float* grads,
                              double* loss);
/* Introspection for tests and debugging.  With keep != 0 the gradient calls
 * that follow keep dL/dz of every hidden layer in buffers of their own (five
 * more activation-sized buffers; keep = 0 frees them).  s2d_cnn_get_tensor
 * copies, as float, a BF16 tensor of the last gradient call (or per-layer
 * forward: the fused forward keeps no per-layer tensors) for the
 * first `batch` images, layout [batch][grid][grid][channels padded to 16 or
 * 32]: kind 0 = the input activations of `layer` (layer 0: the normalised
 * network input), 1 = its pre-activation z (layers 0-4, after a gradient
 * call), 2 = dL/dz of its output (layer 5 always; layers 0-4 when kept). */
S2D_API int s2d_cnn_keep_layer_grads(s2d_cnn* c, int32_t keep);
S2D_API int s2d_cnn_get_tensor(s2d_cnn* c, int32_t kind, int32_t layer, int32_t batch, float* out);
/* device-resident training set of (w, psi, Pi) snapshots */
S2D_API int s2d_cnn_dataset_reserve(s2d_cnn* c, int32_t capacity);
S2D_API int s2d_cnn_dataset_size(const s2d_cnn* c);
S2D_API int s2d_cnn_dataset_add(s2d_cnn* c, s2d_handle* les);   /* after s2d_subgrid_flux */
S2D_API int s2d_cnn_dataset_stats(s2d_cnn* c, double* rms3);
/* one epoch over samples [first, first+count) in seeded random order */
S2D_API int s2d_cnn_train_epoch(s2d_cnn* c, int32_t first, int32_t count, int32_t batch, double lr,
                                uint64_t seed, double* mean_loss);
S2D_API int s2d_cnn_eval(s2d_cnn* c, int32_t first, int32_t count, double* mean_loss);
/* S2D_ERR_TIMEOUT if a tensor-core completion wait of the network's kernels
 * gave up since the last call (the forward/gradient/train/eval calls check
 * this themselves; LES runs call it after their steps); clears the flag. */
S2D_API int s2d_cnn_status(s2d_cnn* c);
/* les state := sharp-filtered dns state */
S2D_API int s2d_filter_state(s2d_handle* dns, s2d_handle* les);
/* les state := filtered dns state, and the subgrid flux of the DNS state on
 * the LES grid is kept in the LES handle (and written to pi_host in the
 * reference layout when not NULL) */
S2D_API int s2d_subgrid_flux(s2d_handle* dns, s2d_handle* les, double* pi_host);
/* attach (c != NULL) or detach the closure network of an LES handle */
S2D_API int s2d_les_set_closure(s2d_handle* les, s2d_cnn* c);
/* the closure source -Pi^ of the current LES state (asynchronous) */
S2D_API int s2d_les_closure_term(s2d_handle* les);
/* n steps; with a closure attached, -Pi^ of the state at the start of each
 * step is added to dW in its three RK3 stages */
S2D_API int s2d_les_integrate_steps(s2d_handle* les, int32_t n, double dt);
/* as s2d_les_integrate_steps with a closure attached, timed: *ms = device
 * time of the n steps on the handle's stream (CUDA events) */
S2D_API int s2d_les_time_steps(s2d_handle* les, int32_t n, double dt, double* ms);
/* attach (c != NULL) or detach one closure network for every run of a batch:
 * all runs on the network's grid, at most its max_batch runs.  Each batch
 * step then starts with the closure terms of all runs -- one network forward
 * over the whole batch, the transforms batched over runs -- before the three
 * persistent stage launches, all in the step's CUDA graph. */
S2D_API int s2d_batch_set_closure(s2d_batch* b, s2d_cnn* c);

/* ---- one run decomposed over several ranks (slabs) --------------------- *
 * The reference runs one simulation on several MPI ranks in slabs, with an
 * all-to-all transpose inside every FFTW-MPI transform (src/Alloc.F90:90-100,
 * src/Spectral.F90:340-349, :760, :780).  A slab here is one rank's share of
 * a run: the kx columns [kx0, kx0 + nkx) of the spectral state, for the
 * inverse y-pass (K1) and the forward y-pass with the stage update (K3),
 * and the physical rows [y0, y0 + ny) for the x-pass (K2).  Each stage of
 * IntegrateOneStep is three phases with two all-to-alls between them, which
 * the CALLER performs (MPI_Alltoallv, NCCL, or copies between slabs of one
 * process) on the slab's device buffers:
 *
 *   for stage in 1..3:
 *     s2d_slab_phase(s, stage, 0, dt)   K1 on my columns, pack exchange 0
 *     synchronise; all-to-all of exchange 0 (s2d_slab_exchange)
 *     s2d_slab_phase(s, stage, 1, dt)   unpack, K2 on my rows, pack exchange 1
 *     synchronise; all-to-all of exchange 1
 *     s2d_slab_phase(s, stage, 2, dt)   unpack, K3 and the stage update
 *
 * Segment q of a send buffer goes to rank q; segment q of a receive buffer
 * comes from rank q; segments follow one another in rank order with the
 * byte counts s2d_slab_exchange gives.  Phases run asynchronously on the
 * slab handle's stream (s2d_synchronize).  Every rank's handle holds
 * full-size arrays: set the same initial state on every rank (s2d_set_state,
 * s2d_set_turbulent, ... on s2d_slab_handle); after steps only the rank's
 * own columns of its state are current, and s2d_slab_get_columns writes them
 * (and psi) into reference-layout host arrays, leaving the other columns
 * untouched.  The kernels are the single-run kernels on a column view or a
 * row range, so a decomposed run equals the single run bit for bit.
 * Basdevant form only. */
#define S2D_SLAB_MAX_RANKS 16
typedef struct s2d_slab s2d_slab;
/* part = {kx0, nkx, y0, ny} of rank `rank` of nranks for an nx grid */
S2D_API int s2d_slab_partition(int32_t nx, int32_t nranks, int32_t rank, int32_t part[4]);
S2D_API int s2d_slab_create(const s2d_config* cfg, int32_t rank, int32_t nranks, s2d_slab** out);
S2D_API void s2d_slab_destroy(s2d_slab* s);
/* the slab's handle: initial conditions, set_state, CFL, s2d_synchronize */
S2D_API int s2d_slab_handle(s2d_slab* s, s2d_handle** h);
/* device send / receive buffers of exchange 0 or 1 (the same two buffers
 * serve both) and the bytes per peer (arrays of nranks; either may be NULL) */
S2D_API int s2d_slab_exchange(s2d_slab* s, int32_t exchange, void** send, void** recv, int64_t* send_bytes,
                              int64_t* recv_bytes);
/* phase 0, 1 or 2 of RK3 stage 1..3 (asynchronous on the slab's stream) */
S2D_API int s2d_slab_phase(s2d_slab* s, int32_t stage, int32_t phase, double dt);
/* the rank's columns of wC and psiC (either may be NULL, not both), reference
 * layout; synchronises */
S2D_API int s2d_slab_get_columns(s2d_slab* s, double* wC, double* psiC, int32_t cISize, int32_t nyG);

/* ---- allocation-free right-hand side ----------------------------------- *
 * No counterpart in the reference.  For callers that must not allocate
 * device memory -- host codes whose device memory belongs to another
 * runtime or a fixed pool, plug-ins that may only use the buffers they are
 * handed, or code paths where an allocation (and the device synchronisation
 * it can bring) is not allowed.
 *
 * dW = ComputeRHS(wC) (src/Spectral.F90:396-482, Basdevant form, viscosity
 * nu, no drag or forcing) for one grid of nx = ny points, on the current CUDA
 * device.  wC_dev and dW_dev are DEVICE arrays in the reference layout
 * (cISize, nyG) complex128, owned by the caller; modes of wC outside
 * |k| <= nx/2 are ignored, modes of dW outside it are written as zero.
 * stream is a cudaStream_t (NULL = the legacy default stream); the call is
 * asynchronous on it.
 *
 * All scratch lives in one static device array of
 * S2D_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * the process exits; the call makes no cudaMalloc, cudaFree or other
 * allocation.  nx must be a multiple of 8 and at most S2D_NOALLOC_MAX_NX,
 * else S2D_ERR_INVALID.  The first call on a device resolves the array's
 * device address (cudaGetSymbolAddress) and sets kernel attributes: make it
 * before any stream capture.  The first call with a given nx on a device
 * (and the first after a call with another nx) also queues the upload of
 * that grid's twiddle and 1/k^2 tables into the array on the same stream;
 * later calls with the same nx reuse them.  Every call shares the one
 * array, so calls that overlap on the GPU (other streams, other host
 * threads) race; serialise them.  The library remembers which tables the
 * array holds, so do not use this entry point on a device after
 * cudaDeviceReset (the array's contents are lost while that record stays).
 * Errors are reported by the return code only; a NaN or Inf in wC gives a
 * non-finite dW that is not detected or reported.
 */
#define S2D_NOALLOC_MAX_NX          256
#define S2D_NOALLOC_SCRATCH_BYTES   (3u << 20)
S2D_API int s2d_compute_rhs_noalloc(int32_t nx, double nu, const double* wC_dev, double* dW_dev,
                                    void* stream);

#ifdef __cplusplus
}
#endif

#endif /* S2D_H */
