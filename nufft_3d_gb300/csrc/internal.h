// Internal declarations shared by the libnufft3d translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/nufft3d.h"

namespace nufft3d {

// ------------------------------------------------------ device lock
// CUDA graph capture on one thread is invalidated when another thread makes a
// device-wide synchronising call (cudaFree, cudaDeviceSynchronize).  Every
// allocation, free and device-wide synchronisation in the library, and every
// capture, holds this lock, so plans can be built, freed and used from several
// threads at once (the serving loop does).
std::recursive_mutex &device_lock();
#define NUFFT_DEVICE_LOCK std::lock_guard<std::recursive_mutex> nufft_dlk_(::nufft3d::device_lock())

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
void clear_error();
int fail(int code, const std::string &msg);

#define NUFFT_CUDA_TRY(expr)                                                        \
    do {                                                                            \
        cudaError_t e_ = (expr);                                                    \
        if (e_ != cudaSuccess)                                                      \
            return ::nufft3d::fail(NUFFT3D_ERR_CUDA, std::string(#expr) + ": " +    \
                                   cudaGetErrorString(e_));                         \
    } while (0)

#define NUFFT_TRY(expr)                                                             \
    do {                                                                            \
        int s_ = (expr);                                                            \
        if (s_ != NUFFT3D_SUCCESS) return s_;                                       \
    } while (0)

// ----------------------------------------------------------- KB kernel
// Kaiser-Bessel kernel of kernel.m:2-11 evaluated in registers:
//   w(d2) = I0(alpha*sqrt(1 - d2/(J/2)^2)) / I0(alpha)
// with the Numerical Recipes I0 polynomial (kernel.m:14-30).  The large-
// argument branch is rearranged as exp(ax - alpha) * rsqrt(ax) * poly *
// (exp(alpha)/I0(alpha)) so no intermediate leaves single-precision range.
// Degree of the plan-time polynomial fit of the Kaiser-Bessel kernel.
constexpr int kKBDeg = 14;

struct KBParams {
    float alpha;        // KB alpha
    float inv_half2;    // 1/(J/2)^2
    float a2_over;      // alpha^2 / 3.75^2 (small-branch test/argument)
    float inv_i0a;      // 1/I0(alpha)
    float exp_over_i0a; // exp(alpha)/I0(alpha)
    float half2;        // (J/2)^2: tap kept iff dist2 <= half2 (4*dist2 <= J^2)
    int poly;           // 1: use the polynomial c below (fitted at plan time)
    float c[kKBDeg + 1]; // kernel(t) ~ sum_k c[k] t^k, t = 1 - dist2/(J/2)^2
};

// exp(x) for x <= 0 by Cody-Waite range reduction: x*log2(e) = hi + lo with
// hi = rn(x*L2E) and lo its rounding residual (exact by FMA) plus the tail of
// log2(e); 2^hi comes from ex2.approx and 2^lo ~ 1 + lo*ln2 (|lo| <= 2^-24*|hi|).
__device__ __forceinline__ float exp_neg(float x)
{
    const float L2E = 1.44269504088896341f;
    const float L2E_LO = 1.925963033500e-8f;   // log2(e) - L2E
    const float hi = x * L2E;
    const float lo = fmaf(x, L2E, -hi) + x * L2E_LO;
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(hi));
    return fmaf(e, lo * 0.69314718055994531f, e);
}

__device__ __forceinline__ float kb_weight(float dist2, const KBParams &p)
{
    // (J/2)^2 - dist2 is exact for dist2 in [(J/2)^2/2, (J/2)^2] (Sterbenz)
    const float t = fmaxf((p.half2 - dist2) * p.inv_half2, 0.0f);
    if (p.poly) {
        // branch-free: a degree-14 polynomial in t interpolating the same
        // kernel at Chebyshev nodes (max error checked at plan time with the
        // same Horner steps); an Estrin form, shorter dependency chain but
        // more instructions, measured slower in these issue-bound kernels.
        // Indexed directly (no pointer to the parameter) so the coefficients
        // stay in the constant bank.
        float s = p.c[kKBDeg];
#pragma unroll
        for (int k = kKBDeg - 1; k >= 0; --k) s = fmaf(s, t, p.c[k]);
        return s;
    }
    const float y = p.a2_over * t; // (ax/3.75)^2
    if (y < 1.0f) {
        float s = fmaf(y, 0.45813e-2f, 0.360768e-1f);
        s = fmaf(y, s, 0.2659732f);
        s = fmaf(y, s, 1.2067492f);
        s = fmaf(y, s, 3.0899424f);
        s = fmaf(y, s, 3.5156229f);
        s = fmaf(y, s, 1.0f);
        return s * p.inv_i0a;
    }
    // large branch: t >= 3.75^2/alpha^2 > 0, so the rsqrt forms are exact enough
    const float st = t * rsqrtf(t);              // sqrt(t)
    const float ax = p.alpha * st;               // alpha*sqrt(t)
    const float ra = rsqrtf(ax);                 // ax^(-1/2)
    const float z = 3.75f * (ra * ra);           // 3.75/ax
    // ax - alpha = -alpha (1 - t) / (1 + sqrt(t)) with 1 - t = dist2/(J/2)^2
    // taken from the distance itself: no cancellation between ax and alpha
    const float em = -p.alpha * (dist2 * p.inv_half2) / (1.0f + st);
    float s = fmaf(z, 0.392377e-2f, -0.1647633e-1f);
    s = fmaf(z, s, 0.2635537e-1f);
    s = fmaf(z, s, -0.2057706e-1f);
    s = fmaf(z, s, 0.916281e-2f);
    s = fmaf(z, s, -0.157565e-2f);
    s = fmaf(z, s, 0.225319e-2f);
    s = fmaf(z, s, 0.1328592e-1f);
    s = fmaf(z, s, 0.39894228f);
    return exp_neg(em) * ra * s * p.exp_over_i0a;
}

// ------------------------------------------------------------ geometry
struct Geom {
    int K[3];
    int T[3];     // tile shape
    int P[3];     // padded tile = T + 2*Ra
    int Ra[3];    // halo per axis (R, or 0 along z in 2D)
    int nt[3];    // tiles per axis
    int R;        // ceil(J/2)
    int radial;
    int is2d;
};

// ------------------------------------------------------------------ FFT
struct FFTDesc {
    int n;
    int nst;
    int rad[16];
    const float2 *tw; // tw[j] = exp(-2 pi i j / n), j < n
};

bool fft_factor(int n, FFTDesc &d);

// Strided line pass over rows of contiguous complex vectors (FY/FZ/IY/IZ).
struct LinePass {
    int n_in, n_out, Nimg, pad_in, crop_out, vec, nchunks;
    int64_t in_axis_stride, out_axis_stride, in_outer_stride, out_outer_stride;
};

// ------------------------------------------------------- batched stages
// One descriptor per volume and stage for the batched (multi-volume) launches.
struct BatchFFT {
    const float2 *in;
    float2 *out;
    const float *U;
    const float2 *addend;
    int N1, N23, nc, inv;
    float scale, add_coef;
    LinePass lp;
    FFTDesc fd;
};

// Candidate taps of a plan (see the interpolation kernels): packed offsets
// (dx'+8) | (dy'+8)<<4 | (dz'+8)<<8 of the 8 sub-cube lists back to back.
struct Cand {
    const int *list;
    int n;          // total entries
    int start[8];   // first entry of sub-cube q's list
    int cnt[8];     // its length
    int core[8];    // its first core[q] entries are inside the support for every sample of the sub-cube
};

// Status of the interpolation kernels of one plan: where an expired bounded
// wait is reported and how many polls a wait makes.
struct InterpStatus {
    int *err;   // the plan's status flag (set to 1 on expiry), or null
    int polls;  // polls of each bounded wait
};

// Slots of a plan's small device work buffer (int[16]).
constexpr int kWorkGather = 0;   // work counter of the persistent gather
constexpr int kWorkSpread = 1;   // work counter of the persistent spread
constexpr int kWorkTapFill = 2;  // stored-H build: fill disagrees with count
constexpr int kWorkStatus = 3;   // interpolation status (a bounded wait expired)
constexpr int kDefaultWaitPolls = 1 << 22;

struct BatchInterp {
    const float2 *in;   // gather: grid; spread: sorted samples
    float2 *out;        // gather: sorted samples; spread: grid
    const float4 *samples;
    const int4 *blocks;
    const float *wsample;
    Geom g;
    KBParams kb;
    Cand cand;
    const CUtensorMap *tmaps;  // gather: [4] maps of the grid for coil widths 1, 2, 4, 8 (device memory)
    int tmap_ok;               // bit log2(width): that map is valid
    int nc;
    float scale;
    const uint32_t *tap_rows;  // the volume's stored H (8-coil gather entries), or null
    const int2 *tap_ent;
    InterpStatus status;       // the volume's plan: its status flag and wait polls
};

struct BatchPerm {
    const float2 *in;
    float2 *out;
    const int32_t *inv;
    const float *w;     // permute_in weights (sorted order) or null
    int64_t M;
    int nc;
    float scale;
};

LinePass make_linepass(int n_outer, int64_t rowlen, int n_in, int n_out, int Nimg, int pad_in, int crop_out,
                       int64_t in_axis, int64_t out_axis, int64_t in_outer, int64_t out_outer, int64_t *nblk);
int line_vec(int64_t rowlen);
size_t line_smem(int vec, int K);
bool needs_rare(const FFTDesc &f);
constexpr int kMaxLineCoilsHost = 16;
// Descriptors of up to kBatchParamVols volumes of one batched FFT launch,
// passed by value as the kernel parameter: blocks find their volume by a
// search over `first` in the parameter bank instead of dependent loads from
// global memory before they can touch data.
constexpr int kBatchParamVols = 48;
struct BatchFFTParams {
    int nvol;
    int first[kBatchParamVols + 1];  // first block of each volume; first[nvol] = total
    int nch[kBatchParamVols];        // coil chunks per line (x passes)
    BatchFFT v[kBatchParamVols];
};

int batch_four_step(int K, bool all_vec16);
int launch_fft_batch_p(const BatchFFTParams &P, int kind, size_t smem, bool rare, int r1, cudaStream_t s);
// stored_h: every volume has its stored H (the 8-coil gather group then reads it)
int launch_interp_batch(bool gather, int cb, int R, bool radial, const BatchInterp *vols, const int4 *table,
                        int nblocks, size_t smem, const KBParams &kb, int *work, int nsm, cudaStream_t s,
                        bool stored_h);
int launch_perm_batch(bool out, const BatchPerm *vols, const int4 *table, int nblocks, cudaStream_t s);

// ----------------------------------------------------------------- plan
struct Scratch {
    int nc = 0;
    float2 *B1 = nullptr, *B2 = nullptr, *G = nullptr, *ks = nullptr;
    size_t bytes = 0;
};

struct HostStage {
    size_t bytes_in = 0, bytes_out = 0;
    float *in = nullptr, *out = nullptr;   // device staging for host-pointer calls
};

// Per-stage CUDA-event timing (nufft3d_profile): events are recorded on the
// launching stream around each stage and resolved when read.
enum Stage {
    ST_FFT_X_FWD, ST_FFT_Y_FWD, ST_FFT_Z_FWD, ST_GATHER, ST_PERMUTE_OUT, ST_PERMUTE_IN,
    ST_GRID_ZERO, ST_SPREAD, ST_FFT_Z_ADJ, ST_FFT_Y_ADJ, ST_FFT_X_ADJ, ST_COUNT
};
extern const char *const kStageNames[ST_COUNT];

struct Profiler {
    bool on = false;
    struct Rec {
        int stage;
        int launches;
        cudaEvent_t a, b;
    };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    double ms[ST_COUNT] = {0};
    long long launches[ST_COUNT] = {0};
    long long calls[ST_COUNT] = {0};
};

struct SolverWork {
    int nc = 0;
    size_t nimg = 0;
    float2 *x = nullptr, *r = nullptr, *p = nullptr, *q = nullptr, *v = nullptr,
           *vprev = nullptr, *w1 = nullptr, *w2 = nullptr;
    double *partial = nullptr;  // [nc * nchunk]
    double *bpart = nullptr;    // [nc * nchunk] |b|^2 partial sums of a warm start
    double *scal = nullptr;     // per-coil scalar state
    int *iters = nullptr;       // per-coil iteration counts
    int nchunk = 0;
};

// Device tables of a plan that never change after creation (sorted samples,
// tile pieces, candidate taps, U, d, twiddles).  Plans made with
// nufft3d_plan_share hold the same TableOwner; the last one frees them.
struct TableOwner {
    int device = 0;
    std::vector<void *> ptrs;
    ~TableOwner();
};

} // namespace nufft3d

struct nufft3d_plan {
    int device = 0;
    int N[3] = {0, 0, 0};
    int64_t M = 0, nnz = 0;
    double J = 4, u = 2, alpha = 0, i0a = 1;
    int radial = 1;
    nufft3d::Geom geom{};
    nufft3d::KBParams kb{};
    // sorted samples
    float4 *samples = nullptr;  // (fx, fy, fz, packed local coords), sorted by tile
    int32_t *perm = nullptr;    // sorted -> original
    int32_t *inv = nullptr;     // original -> sorted, -1 out of bounds
    int4 *blocks = nullptr;     // (tile, start, count, float bits of max summed weight)
    int4 *own_blocks = nullptr; // a piece table of this handle alone (after nufft3d_plan_tune), else null
    int *cand = nullptr;        // candidate tap offsets (reflected octant), packed
    int n_cand = 0;             // total entries of the 8 sub-cube lists
    nufft3d::Cand cand_desc{};         // device list + per-sub-cube starts and lengths
    int64_t n_blocks = 0;
    std::vector<int32_t> tile_counts;  // in-bounds samples per tile (host copy; pieces are rebuilt from it)
    int piece_samples = 0;      // largest piece (samples) of the current piece table
    int coils_per_pass = 8;
    int max_coils_per_pass = 8; // the largest coil width the plan's shared memory allows
    int use_tma = 1;            // bulk tensor copies for interior gather tiles
    int sm_count = 148;         // multiprocessors of the plan's device
    int interp_sms = 0;         // SMs the persistent interpolation kernels may use (0 = all)
    int host_copy = 0;          // host-pointer calls: 0 = kernels use page-locked buffers in place,
                                // 1 = copy-engine transfers through device staging buffers
    int *work = nullptr;        // [16]: work counters of the persistent interpolation kernels and the
                                // plan's status flags (slots kWork*)
    int wait_polls = nufft3d::kDefaultWaitPolls;  // polls of each bounded wait in the gather
    // stored H in tile order (8-coil passes): row of sorted sample s = entries
    // [8*tap_rows[s], 8*tap_rows[s+1]) of tap_ent, (weight bits, tile offset),
    // padded with zero weights to whole chunks of 8
    uint32_t *tap_rows = nullptr;
    int2 *tap_ent = nullptr;
    int64_t tap_bytes = 0;
    // stored H' for the 8-coil spread (tables.cu): pieces of at most
    // kSpreadCap samples, (tile, first sample, count, first line); the warps'
    // first lines (33 per piece); the bundles of 128-byte lines
    int4 *spread_pieces = nullptr;
    uint32_t *spread_wstart = nullptr;
    int2 *spread_ent = nullptr;
    int64_t n_spread_pieces = 0;
    int64_t spread_bytes = 0;
    int threads = 256;
    double taps = 0;
    float *U = nullptr;         // deapodization [N1 N2 N3]
    float *d = nullptr;         // density, sorted order [nnz]
    float *d_orig = nullptr;    // density, original order [M] (0 out of bounds)
    float2 *tw[3] = {nullptr, nullptr, nullptr};
    nufft3d::FFTDesc fft[3];
    nufft3d::Scratch scratch;
    nufft3d::HostStage stage;
    nufft3d::SolverWork solver;
    float *wbuf = nullptr;      // sorted sample weights for iNUFT (W.*d)
    int64_t table_bytes = 0;
    cudaStream_t own_stream = nullptr;
    nufft3d::Profiler prof;
    std::shared_ptr<nufft3d::TableOwner> tables;  // owner of the pointers above marked as tables
};

namespace nufft3d {

// Default largest tile piece (samples): larger pieces measured slightly faster
// at 128^3 (fewer halo flushes); nufft3d_plan_tune searches around it.
constexpr int kDefaultPieceSamples = 4096;
// Tile pieces of at most S samples per tile (split evenly), largest first.
std::vector<int4> make_pieces(const std::vector<int32_t> &counts, int S);
// Replaces the plan's piece table with pieces of at most S samples and
// recomputes their summed-weight bounds (synchronises the plan's stream).
int rebuild_pieces(nufft3d_plan *p, int S);

// Launchers (stream-ordered, no synchronisation).
int ensure_scratch(nufft3d_plan *p, int nc);
int launch_fx(nufft3d_plan *p, const float2 *img, float2 *B1, int nc, cudaStream_t s);
int launch_fy(nufft3d_plan *p, const float2 *B1, float2 *B2, int nc, cudaStream_t s);
int launch_fz(nufft3d_plan *p, const float2 *B2, float2 *G, int nc, cudaStream_t s);
int launch_iz(nufft3d_plan *p, const float2 *G, float2 *B2, int nc, cudaStream_t s);
int launch_iy(nufft3d_plan *p, const float2 *B2, float2 *B1, int nc, cudaStream_t s);
// IX: img = scale*U*ifft_x(B1) + add_coef*addend (addend may be null)
int launch_ix(nufft3d_plan *p, const float2 *B1, float2 *img, int nc, float scale,
              const float2 *addend, float add_coef, cudaStream_t s);

// gather: ks[s*nc + c] = scale * w_s * sum_taps w * G[...]  (wsample may be null)
int launch_gather(nufft3d_plan *p, const float2 *G, float2 *ks, int nc, float scale,
                  const float *wsample, cudaStream_t s);
// plan time: per-block bound on summed weights (blocks[b].w) for the spread
int launch_weight_sum(nufft3d_plan *p, cudaStream_t s);
// plan time, stored H: rows[s] = chunks of 8 entries in sample s's row
int launch_tap_count(nufft3d_plan *p, uint32_t *rows, cudaStream_t s);
// plan time, stored H: the entries of every row (rows = chunk offsets)
int launch_tap_fill(nufft3d_plan *p, const uint32_t *rows, int2 *taps, cudaStream_t s);
// the stored-H kernels serve this plan (8-coil passes, R <= 3)
bool tap_table_applies(const nufft3d_plan *p);
// spread: G += H' ks (G zeroed by caller)
int launch_spread(nufft3d_plan *p, const float2 *ks, float2 *G, int nc, cudaStream_t s);
// Largest spread piece of the stored H' (samples staged in shared memory,
// two pieces at a time).
constexpr int kSpreadCap = 1664;
// stored H' (tables.cu): plan-time build from the stored H, the 8-coil
// spread pass that reads it, and whether it serves coils c0..c0+7 of nc
int build_spread_table(nufft3d_plan *p, int mode, cudaStream_t s);
int launch_spread_tab(nufft3d_plan *p, const float2 *ks, float2 *G, int nc, int c0, cudaStream_t s);
bool spread_tab_applies(const nufft3d_plan *p, int nc, int c0);
int configure_spread_tab_kernels();
// multiprocessors the persistent interpolation kernels of a handle may use
int interp_grid_sms(const nufft3d_plan *p);
// user [M nc] <-> sorted [nnz][nc]
int launch_permute_out(nufft3d_plan *p, const float2 *ks, float2 *k, int nc, float scale,
                       cudaStream_t s);
int launch_permute_in(nufft3d_plan *p, const float2 *k, float2 *ks, int nc,
                      const float *wsorted, cudaStream_t s);

// whole operators on the plan's scratch
int op_forward(nufft3d_plan *p, const float2 *x, float2 *k, int nc, cudaStream_t s);
int op_adjoint(nufft3d_plan *p, const float2 *k, float2 *x, int nc, cudaStream_t s);
// y = A'WA x + damp^2 x, wsorted = W.*d in sorted order (null = d)
int op_normal(nufft3d_plan *p, const float2 *x, float2 *y, int nc, double damp,
              const float *wsorted, cudaStream_t s);

int op_adjoint_weighted(nufft3d_plan *p, const float2 *k, float2 *x, int nc, const float *wsorted,
                        cudaStream_t s);
// iNUFT.m:72: W.*d in sorted order (d itself when W_orig is null)
int prepare_weights(nufft3d_plan *p, const float *W_orig, const float **wsorted, cudaStream_t s);
int refresh_density_orig(nufft3d_plan *p, cudaStream_t s);

int run_density(nufft3d_plan *p, int maxit, cudaStream_t s);
// iNUFT work vectors of a plan handle for nc coils (r, p, q, v, vprev, w1, w2, scalars)
int ensure_solver(nufft3d_plan *p, int nc);
int run_inverse(nufft3d_plan *p, const float2 *raw, float2 *x, int nc, int maxit,
                double damp, const float *W_orig, int solver, double tol, int *iters_host,
                cudaStream_t s, bool warm = false);

size_t smem_interp_bytes(const Geom &g, int cb);
size_t cand_smem_bytes(int n);
// shared memory of the spread's pair-interleaved candidate tables
size_t cand_pairs_bytes(const Cand &cd);
// Reads and clears the plan's interpolation status flag on stream s (after
// the work queued there): NUFFT3D_ERR_TIMEOUT if a bounded wait expired.
int plan_check_status(nufft3d_plan *p, cudaStream_t s);
InterpStatus plan_status(const nufft3d_plan *p);
bool encode_gather_map(const nufft3d_plan *p, const float2 *G, int nc, int cb, CUtensorMap *m);
size_t smem_plane_bytes(int R, int cb);

// Stage timing scope: records an event pair on stream s when profiling is on
// (and the stream is not being captured into a graph).
struct StageTimer {
    nufft3d_plan *p;
    int stage;
    int launches;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    StageTimer(nufft3d_plan *p_, int stage_, int launches_, cudaStream_t s_);
    ~StageTimer();
};
int coil_passes(const nufft3d_plan *p, int nc);
int profile_resolve(nufft3d_plan *p);
void profile_release(nufft3d_plan *p);
int configure_kernels();

} // namespace nufft3d
