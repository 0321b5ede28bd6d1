/*
 * nufft3d.h -- C ABI of libnufft3d.so, the sm_103a (GB300) implementation of
 * the @nufft_3d hot path of marcsous/nufft_3d: Kaiser-Bessel interpolation
 * set-up, forward fNUFT, adjoint aNUFT, density compensation and the iNUFT
 * iterative reconstruction.
 *
 * Every entry point replaces one piece of the reference's MATLAB interface
 * (file:line relative to the reference project root).  The layouts are the
 * reference's: column-major MATLAB arrays, complex values interleaved
 * (re, im) as MATLAB's interleaved complex API stores them.
 *
 *   om   [3 x M]            double, cycles/FOV (nufft_3d.m:11)
 *   x    [N1 N2 N3 nc]      complex single image
 *   k    [M nc]             complex single samples
 *   W, d [M]                real single weights
 *
 * Pointers named *_dev are device pointers on the plan's device; *_host are
 * host pointers (pinned memory gives the fastest copies).  `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).  All calls
 * return NUFFT3D_SUCCESS (0) or a negative status; nufft3d_last_error()
 * returns a thread-local message for the last failure on the calling thread.
 *
 * A plan is immutable after creation except for its internal scratch buffers:
 * calls on the same plan must not overlap (serialise them on one stream, or
 * create one plan per stream).  Plans on different devices or different plans
 * on one device are independent.
 */
#ifndef NUFFT3D_H
#define NUFFT3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NUFFT3D_SUCCESS 0
#define NUFFT3D_ERR_ARG (-1)          /* invalid argument (reference error() conditions) */
#define NUFFT3D_ERR_SIZE (-2)         /* size mismatch or prod(K) >= 2^31 */
#define NUFFT3D_ERR_CUDA (-3)         /* CUDA runtime failure */
#define NUFFT3D_ERR_NOMEM (-4)        /* device or host allocation failed */
#define NUFFT3D_ERR_UNSUPPORTED (-5)  /* option outside what this build implements */
#define NUFFT3D_ERR_TIMEOUT (-6)      /* a bounded wait expired */

#define NUFFT3D_SOLVER_MINRES 0       /* iNUFT.m:136 (reference default) */
#define NUFFT3D_SOLVER_CG 1           /* conjugate gradients, FP64 scalars */

typedef struct nufft3d_plan nufft3d_plan;

/* Constructor options: the reference's name/value pairs (nufft_3d.m:26-43,
 * 70-76) plus tuning knobs.  Fill with nufft3d_opts_default() first. */
typedef struct nufft3d_opts {
    double J;          /* kernel width ('J', default 4) */
    double u;          /* oversampling ('u', default 2) */
    double alpha;      /* Kaiser-Bessel alpha ('alpha', 0 = Beatty formula) */
    int radial;        /* 1 = radial kernel, 0 = separable ('radial', default 1) */
    int gpu;           /* 'gpu': 1 = single-precision GPU (the only path built);
                          0 (CPU) and 2 (double GPU) return NUFFT3D_ERR_UNSUPPORTED */
    int device;        /* CUDA device ordinal for the plan (default: current) */
    const float *d;    /* 'd': optional host density [M] (NULL = density.m) */
    int density_iters; /* density.m:5 maxit (default 20) */
    int tile[3];       /* interpolation tile shape (0 = autotune/default) */
    int max_coils_per_pass; /* coils handled per interpolation pass (0 = auto) */
    int max_samples_per_block; /* samples per interpolation block (0 = 4096) */
    int verbose;       /* print the reference's set-up summary to stdout */
    int tap_table;     /* stored interpolation matrix H (nufft_3d.m:153-212) in
                          tile order, read by the 8-coil gather passes of fNUFT
                          (see spread_table for H'): 1 = build it, 0 = evaluate
                          the kernel on the fly, -1 = auto (default: build it
                          when it takes at most half of the free device memory) */
    int wait_polls;    /* polls of each bounded wait of the interpolation
                          kernels (the tile copy of the gather) before it gives
                          up and reports NUFFT3D_ERR_TIMEOUT (default 2^22, well
                          under a second); 0 gives up at once: every bulk tile
                          copy is then still allowed to land, but its tile is
                          skipped and the timeout reported, which exercises the
                          error path without a fault */
    int spread_table;  /* stored transpose H' (built from the stored H, so only
                          with it), read by the 8-coil spread passes of aNUFT
                          (full passes of an even coil count): per tile piece
                          of at most 2048 samples, each grid point's row of
                          (sample, weight); 1 = build it, 0 = evaluate the
                          kernel on the fly, -1 = auto (default: build it when
                          it takes at most half of the free device memory) */
} nufft3d_opts;

/* Read-only properties (nufft_3d.m:26-43). */
typedef struct nufft3d_info {
    int32_t N[3];      /* image size (N3 = 1 in 2D, nufft_3d.m:104-106) */
    int32_t K[3];      /* oversampled grid, K = 2*ceil(N*u/2) (nufft_3d.m:109) */
    int64_t M;         /* number of samples (rows of H) */
    int64_t nnz;       /* samples within bounds (nufft_3d.m:126) */
    double J, u, alpha;
    int radial;
    int tile[3];       /* interpolation tile shape in use */
    int64_t n_blocks;  /* interpolation blocks (tile pieces) */
    double taps_per_sample; /* mean nonzeros per row of H */
    int64_t device_bytes;   /* device memory held by the plan (tables + scratch) */
    int64_t tap_table_bytes; /* part of device_bytes held by the stored H (0 = none) */
    int kernel_polynomial;   /* 1: the device evaluates kernel.m's weights as a
                                polynomial fitted at plan time (max error < 4e-6);
                                0: with the Numerical Recipes branches of kernel.m */
    int64_t spread_table_bytes; /* part of device_bytes held by the stored H' (0 = none) */
} nufft3d_info;

/* Fills *opts with the reference defaults: J=4, u=2, alpha=0 (Beatty),
 * radial=1, gpu=1, density_iters=20 (nufft_3d.m:27-36, density.m:5),
 * tap_table=-1, spread_table=-1. */
int nufft3d_opts_default(nufft3d_opts *opts);

/* obj = nufft_3d(om, N, name, value, ...)  -- nufft_3d.m:54-251.
 * om_host: [3 x M] doubles (cycles/FOV).  N: 1 or 3 even integers
 * (n_N = 1 or 3).  Builds the sorted interpolation plan, the deapodization U
 * (deap.m) and, unless opts->d is given, the density d (density.m). */
int nufft3d_plan_create(const double *om_host, int64_t M, const int32_t *N, int n_N,
                        const nufft3d_opts *opts, nufft3d_plan **plan);

int nufft3d_plan_destroy(nufft3d_plan *plan);

/* A second handle on the same trajectory: shares the source plan's device
 * tables (sorted samples, tiles, U, d, twiddles; freed with the last handle)
 * and has its own work buffers and stream, so calls on the two handles may
 * run concurrently.  Used by the serving loop for concurrent reconstructions
 * of one resident trajectory.  nufft3d_density on any handle changes the
 * shared d. */
int nufft3d_plan_share(const nufft3d_plan *src, nufft3d_plan **plan);

/* Caps the persistent interpolation kernels (gather and spread: one block
 * per multiprocessor) of this handle at `sms` multiprocessors; 0 = all.  The
 * others stay free for kernels on other streams -- e.g. the host-link-bound
 * stages of another handle's host-pointer call, so that two threads calling
 * nufft3d_forward_host / _adjoint_host on two handles overlap one call's
 * transfers with the other's compute.  No counterpart in the reference. */
int nufft3d_plan_set_sms(nufft3d_plan *plan, int sms);

/* How this handle's host-pointer calls (nufft3d_*_host) move page-locked
 * host buffers: mode 0 = the first and last kernels of the chain read and
 * write them in place over the host link (no copies, no staging memory);
 * mode 1 = copy-engine transfers (cudaMemcpyAsync) through device staging
 * buffers, which run beside other handles' kernels without occupying SMs.
 * Pageable buffers are always staged.  No counterpart in the reference. */
int nufft3d_plan_set_host_copy(nufft3d_plan *plan, int mode);

/* Result of nufft3d_plan_tune. */
typedef struct nufft3d_tune_result {
    int samples_per_block;  /* chosen largest tile piece (samples) */
    int coils_per_pass;     /* chosen coils per interpolation pass */
    double ms_best;         /* fNUFT+aNUFT of nc coils with the choice (ms) */
    double ms_default;      /* the same with the plan's settings before tuning (0 if cached) */
    int candidates;         /* settings timed (0 if the choice came from the cache) */
    int from_cache;         /* 1: taken from an earlier search of the same shape */
} nufft3d_tune_result;

/* Autotuner: times fNUFT + aNUFT of nc coils (synthetic data) on this plan
 * for tile pieces of 1024, 2048 or 4096 samples and 2 / 4 / 8 coils per
 * interpolation pass, keeps the fastest and caches it for the process under
 * the plan's shape, coil count and sample-density class (later plans of the
 * same class take it without timing unless force = 1).  The tile shape is
 * fixed by the kernels and not searched.  Replaces this handle's piece table
 * (tune before nufft3d_batch_create or nufft3d_plan_share, which copy it).
 * No counterpart in the reference (sparse H has no blocking to tune). */
int nufft3d_plan_tune(nufft3d_plan *plan, int nc, int force, nufft3d_tune_result *result);

/* Device bytes a handle allocates for work buffers at nc coils (FFT and
 * interpolation scratch; plus the iNUFT solver vectors if with_solver). */
int nufft3d_plan_footprint(const nufft3d_plan *plan, int nc, int with_solver, int64_t *bytes);

int nufft3d_plan_info(const nufft3d_plan *plan, nufft3d_info *info);

/* obj.U (deap.m:2-36,98): [N1 N2 N3] real single, copied to host. */
int nufft3d_get_deap(const nufft3d_plan *plan, float *U_host);

/* obj.d (density.m:2-42, or the user density, zero out of bounds): [M]. */
int nufft3d_get_density(const nufft3d_plan *plan, float *d_host);

/* k = obj.fNUFT(x)  -- fNUFT.m:2-9: k = H*fft3_pad(U.*x)/sqrt(nnz). */
int nufft3d_forward(nufft3d_plan *plan, const float *x_dev, float *k_dev, int nc,
                    void *stream);

/* x = obj.aNUFT(k)  -- aNUFT.m:2-9: x = U.*ifft3_crop(H'*k)/sqrt(nnz). */
int nufft3d_adjoint(nufft3d_plan *plan, const float *k_dev, float *x_dev, int nc,
                    void *stream);

/* y = iprojection(x, damp, W) -- nufft_3d.m:305-313:
 * y = aNUFT(W.*fNUFT(x)) + damp^2*x.  W_dev: [M] or NULL for W = d. */
int nufft3d_normal(nufft3d_plan *plan, const float *x_dev, float *y_dev, int nc,
                   double damp, const float *W_dev, void *stream);

/* k = obj.fNUFT(x) without any device allocation in the call.  No counterpart
 * in the reference (MATLAB allocates freely); it exists for callers that must
 * not trigger cudaMalloc -- it synchronises the whole device and can fail under
 * memory pressure -- such as a latency-critical reconstruction loop or a host
 * application that owns all GPU memory through its own pool.  Same arguments
 * and result as nufft3d_forward.  Work buffers come from one fixed array in
 * the library's device image, nufft3d_forward_noalloc_scratch_bytes() bytes
 * per GPU (held by every GPU that loads the library until exit); plans/coil
 * counts that need more return NUFFT3D_ERR_SIZE.  Every call on a device
 * shares that array: calls that overlap on the GPU race and must be
 * serialised by the caller.  The first call on each device looks up the
 * array's address (cudaGetSymbolAddress); make it before any stream capture.
 * The plan itself is created beforehand with nufft3d_plan_create. */
int nufft3d_forward_noalloc(nufft3d_plan *plan, const float *x_dev, float *k_dev, int nc,
                            void *stream);

/* Size in bytes of the fixed scratch array used by nufft3d_forward_noalloc. */
size_t nufft3d_forward_noalloc_scratch_bytes(void);

/* Host-pointer variants of fNUFT / aNUFT: copy in, run, copy out, synchronise. */
int nufft3d_forward_host(nufft3d_plan *plan, const float *x_host, float *k_host, int nc);
int nufft3d_adjoint_host(nufft3d_plan *plan, const float *k_host, float *x_host, int nc);

/* im = obj.iNUFT(raw, maxit, damp, W)  -- iNUFT.m:2-138,224-227 default path.
 * raw_dev [M nc]; W_dev [M] sample weights multiplied by d (iNUFT.m:72), or
 * NULL for W = d; maxit = 0 is regridding aNUFT(W.*raw) (iNUFT.m:119-122).
 * Each coil is solved as its own system (A'WA + damp^2 I) x = A'W raw with
 * x0 = 0; solver MINRES (reference) or CG; tol as iNUFT.m:114 (1e-4), tol = 0
 * runs exactly maxit iterations.  iters_host (optional, [nc]) receives the
 * iteration count per coil. */
int nufft3d_inverse(nufft3d_plan *plan, const float *raw_dev, float *x_dev, int nc,
                    int maxit, double damp, const float *W_dev, int solver, double tol,
                    int *iters_host, void *stream);

int nufft3d_inverse_host(nufft3d_plan *plan, const float *raw_host, float *x_host, int nc,
                         int maxit, double damp, const float *W_host, int solver,
                         double tol, int *iters_host);

/* The same solve started from x0 instead of 0 -- minres(A, b, tol, maxit,
 * [], [], x0) as discrep.m:55-58 calls it, warm-starting each damp update
 * from the previous image.  x holds x0 on entry and the image on return; the
 * stop test stays relative to |A'W raw| as in MATLAB minres/pcg with x0.
 * maxit = 0 is regridding (x0 ignored), as in nufft3d_inverse. */
int nufft3d_inverse_x0(nufft3d_plan *plan, const float *raw_dev, float *x_dev, int nc,
                       int maxit, double damp, const float *W_dev, int solver, double tol,
                       int *iters_host, void *stream);
/* im = obj.iNUFT(raw, maxit, damp, W, 'phase-constraint', lambda) --
 * iNUFT.m:140-168 with pprojection (nufft_3d.m:325-334): after the MINRES
 * solve, P = exp(i angle(convn(x, ones(3), 'same'))) (a 3x3 box in x-y per
 * slice), then (P'A'WAP + damp^2 I + i lambda^2 imag) y = P'A'W raw is solved
 * from 0 and im = P y.  The reference's solver pcgpc is external; this is CG
 * with real inner products (FP64 scalars, stop |r| <= tol |b|).  maxit <= 1
 * returns the plain result (iNUFT.m:77-78).  iters_host receives the
 * constrained solve's iteration counts. */
int nufft3d_inverse_phase(nufft3d_plan *plan, const float *raw_dev, float *x_dev, int nc, int maxit,
                          double damp, double lambda, const float *W_dev, double tol, int *iters_host,
                          void *stream);
int nufft3d_inverse_phase_host(nufft3d_plan *plan, const float *raw_host, float *x_host, int nc, int maxit,
                               double damp, double lambda, const float *W_host, double tol, int *iters_host);
int nufft3d_inverse_x0_host(nufft3d_plan *plan, const float *raw_host, float *x_host, int nc,
                            int maxit, double damp, const float *W_host, int solver,
                            double tol, int *iters_host);

/* ---- Batches: many volumes (different N, trajectories, coil counts) per launch.
 * No single counterpart in the reference, which handles one object at a time;
 * each volume's result equals what fNUFT / aNUFT / iNUFT of its own plan
 * gives.  plans[v] must be distinct handles (nufft3d_plan_share for repeated
 * trajectories) sharing the kernel (J, u, alpha, radial) and 2-D/3-D; the batch
 * uses their work buffers, so do not use those handles concurrently with it.
 * The batched kernels read each volume's stored H (tap_table) but not its
 * stored H' (the batched spread evaluates the kernel): plans made only for
 * batches can set spread_table = 0 and save that memory. */
typedef struct nufft3d_batch nufft3d_batch;
int nufft3d_batch_create(nufft3d_plan *const *plans, const int *nc, int nvol, nufft3d_batch **batch);
int nufft3d_batch_destroy(nufft3d_batch *batch);
/* x_dev[v] [N1 N2 N3 nc_v] -> k_dev[v] [M_v nc_v] for every volume, one launch per stage. */
int nufft3d_batch_forward(nufft3d_batch *batch, const float *const *x_dev, float *const *k_dev, void *stream);
/* k_dev[v] -> x_dev[v] for every volume. */
int nufft3d_batch_adjoint(nufft3d_batch *batch, const float *const *k_dev, float *const *x_dev, void *stream);
/* iNUFT of every (volume, coil) system with conjugate gradients, W = d, x0 = 0
 * (iNUFT.m:119-136 with the CG solver), FP64 scalars; iters_host
 * (optional) receives the iteration count of each system, volume-major. */
int nufft3d_batch_inverse(nufft3d_batch *batch, const float *const *raw_dev, float *const *x_dev, int maxit,
                          double damp, double tol, int *iters_host, void *stream);

/* Re-runs density.m on the plan (maxit iterations) and stores it as obj.d. */
int nufft3d_density(nufft3d_plan *plan, int maxit);

/* Stage timing with CUDA events on the launching stream (the reference's
 * tic/toc around its phases, nufft_3d.m:130,213 and iNUFT.m:117,227).
 * enable = 1 starts (and resets) timing, 0 stops it.  Stages captured into a
 * CUDA graph are not timed. */
int nufft3d_profile(nufft3d_plan *plan, int enable);

/* Writes the accumulated stage times as a JSON object into buf:
 * {"gather": {"calls": C, "launches": L, "ms": T}, ...}.  Synchronises on the
 * recorded events. */
int nufft3d_profile_read(nufft3d_plan *plan, char *buf, int cap);

/* Status of the asynchronous work of a plan: reads and clears the plan's
 * status flag after the work queued on `stream` (the stream the device-pointer
 * calls ran on; NULL = the legacy default stream) and synchronises that
 * stream.  Returns NUFFT3D_ERR_TIMEOUT if a bounded wait in an interpolation
 * kernel expired since the last check (the affected tiles were skipped, so
 * those results are incomplete), else NUFFT3D_SUCCESS.  Device-pointer calls
 * (nufft3d_forward, _adjoint, _normal, _inverse*, nufft3d_forward_noalloc and
 * the batch calls, which report on the plans of their volumes) return before
 * their kernels run and report through this call; the host-pointer calls and
 * nufft3d_density check it themselves.  No counterpart in the reference,
 * whose MATLAB operators are synchronous. */
int nufft3d_check_status(nufft3d_plan *plan, void *stream);

/* The plan's Kaiser-Bessel weights as the device kernels evaluate them
 * (kernel.m:2-34): w_dev[i] = kernel(d2_dev[i]) for squared distances in grid
 * units, 0 <= d2 <= (J/2)^2 (larger d2 gives the value at (J/2)^2, whose
 * taps the interpolation never keeps).  For checking the single-precision
 * kernel against the reference's FP64 kernel.m; no counterpart in the
 * reference. */
int nufft3d_kernel_eval(const nufft3d_plan *plan, const float *d2_dev, float *w_dev, int64_t n, void *stream);

/* Message of the last failed call on this thread ("" if none). */
const char *nufft3d_last_error(void);

/* Library version string. */
const char *nufft3d_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NUFFT3D_H */
