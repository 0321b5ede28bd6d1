// Batched operators over many volumes of different sizes and coil counts.
//
// Each stage of fNUFT / aNUFT / iprojection is one launch for the whole batch:
// the launch's blocks come from a table of (volume, block, coil offset)
// entries and each block reads its volume's descriptor (geometry, tables,
// buffers) from device memory.  Volumes use the work buffers of their own plan
// handle, so a batch needs one handle per volume (nufft3d_plan_share gives
// several handles on one trajectory).  All volumes must share the kernel
// half-width R = ceil(J/2), the kernel type (radial or separable) and 2-D/3-D.
//
// The batched iNUFT runs conjugate gradients for every (volume, coil) system
// in lockstep: vector kernels walk a table of (system, chunk) blocks, every dot
// product and recurrence scalar is FP64 per system, and one iteration is
// captured as a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace nufft3d {

enum { FX, FY, FZ, IZ, IY, IX, NFFT };

struct BatchSys {
    float2 *x, *r, *p, *q;
    int64_t n;
    int first, nblk;  // this system's blocks in the vector-kernel table
};

constexpr int kVecChunk = 8192;  // elements per vector-kernel block
constexpr int kS = 8;            // per-system scalars
enum { B_RR, B_BN2, B_ALPHA, B_BETA, B_DONE, B_ITERS, B_TOL };

} // namespace nufft3d

using namespace nufft3d;

struct nufft3d_batch {
    int device = 0, nvol = 0, R = 0, radial = 1, is2d = 0, cb = 8;
    bool rare = false;
    bool stored_h = false;  // every volume's plan holds its stored H
    std::vector<nufft3d_plan *> plans;
    std::vector<int> nc;
    // descriptor arrays (device) and their host mirrors
    std::vector<BatchFFT> h_fft[NFFT];
    std::vector<char> chain;  // per volume: FFT passes as its own chain of launches
    // FFT launch groups: volumes with the same FFT length share a launch
    struct FGroup {
        int K = 0;                // transform length of the group
        size_t smem = 0;          // dynamic shared memory of the Stockham launch
        bool all_vec16 = true;    // every volume has 16-wide line chunks
        int r1 = 0;               // > 0: strided pass by the register four-step FFT (K = 16 r1)
        std::vector<int> vols;    // volumes of the group, in launch order
        std::vector<int> blocks;  // their block counts
        std::vector<int> nch;     // their coil chunks per line (x passes)
    };
    std::vector<FGroup> fgroups[NFFT];
    BatchInterp *gat = nullptr, *spr = nullptr;
    std::vector<CUtensorMap> h_tmaps;   // [nvol][4] gather maps (coil widths 1, 2, 4, 8)
    CUtensorMap *d_tmaps = nullptr;     // their device copy (start of the descriptor buffer)
    int *work = nullptr;                // work counter of the persistent interpolation launches
    std::vector<BatchInterp> h_gat, h_spr;
    // interpolation launch groups: one per coil-pass width
    struct IGroup {
        int cb;
        int4 *tab;
        int n;
        size_t smem;
    };
    std::vector<IGroup> igroups;
    BatchPerm *pout = nullptr, *pin = nullptr;
    std::vector<BatchPerm> h_pout, h_pin;
    int4 *ptab = nullptr;
    int pn = 0;
    // upload staging (pinned) and its completion event
    void *stage = nullptr;
    size_t stage_bytes = 0;
    void *dstage = nullptr;
    cudaEvent_t up_done = nullptr;
    cudaStream_t own = nullptr;
    // batched CG
    BatchSys *sys = nullptr;
    int nsys = 0;
    int2 *vtab = nullptr;  // (system, chunk)
    int vn = 0;
    double *partial = nullptr, *scal = nullptr;
    std::vector<void *> frees;
};

namespace nufft3d {

// ------------------------------------------------------------ vector kernels
__device__ __forceinline__ double rdotb(float2 a, float2 b) { return (double)fmaf(a.x, b.x, a.y * b.y); }

__device__ __forceinline__ void bred(double acc, double *out)
{
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += ws[i];
        *out = s;
    }
}

#define BLOOP(i, e, S)                                                                          \
    const int2 e = vtab[blockIdx.x];                                                            \
    const BatchSys &S = sys[e.x];                                                               \
    const int64_t i0_ = (int64_t)e.y * kVecChunk;                                               \
    const int64_t i1_ = min((int64_t)(e.y + 1) * kVecChunk, S.n);                               \
    for (int64_t i = i0_ + threadIdx.x; i < i1_; i += blockDim.x)

// which: 0 = <p, q>, 1 = <r, r>
__global__ void __launch_bounds__(256) k_bdot(const BatchSys *__restrict__ sys, const int2 *__restrict__ vtab,
                                              int which, double *__restrict__ partial)
{
    double acc = 0;
    BLOOP(i, e, S) acc += which == 0 ? rdotb(S.p[i], S.q[i]) : rdotb(S.r[i], S.r[i]);
    bred(acc, &partial[blockIdx.x]);
}

__device__ __forceinline__ double sys_sum(const BatchSys &S, const double *partial)
{
    double s = 0;
    for (int b = 0; b < S.nblk; ++b) s += partial[S.first + b];
    return s;
}

__global__ void k_bcg_init(const BatchSys *__restrict__ sys, int nsys, const double *__restrict__ partial,
                           double *__restrict__ scal, double tol)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    double *T = scal + s * kS;
    const double rr = sys_sum(sys[s], partial);
    for (int i = 0; i < kS; ++i) T[i] = 0;
    T[B_RR] = rr;
    T[B_BN2] = rr;
    T[B_DONE] = rr == 0 ? 1 : 0;
    T[B_TOL] = tol;
}

__global__ void k_bcg_alpha(const BatchSys *__restrict__ sys, int nsys, const double *__restrict__ partial,
                            double *__restrict__ scal)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    double *T = scal + s * kS;
    const double pq = sys_sum(sys[s], partial);
    if (T[B_DONE] != 0 || !(pq > 0)) {
        T[B_DONE] = 1;
        T[B_ALPHA] = 0;
    } else {
        T[B_ALPHA] = T[B_RR] / pq;
    }
}

__global__ void __launch_bounds__(256) k_bcg_xr(const BatchSys *__restrict__ sys, const int2 *__restrict__ vtab,
                                                const double *__restrict__ scal, double *__restrict__ partial)
{
    double acc = 0;
    const float a = (float)scal[vtab[blockIdx.x].x * kS + B_ALPHA];
    BLOOP(i, e, S)
    {
        float2 xv = S.x[i], rv = S.r[i];
        const float2 pv = S.p[i], qv = S.q[i];
        if (a != 0.f) {
            xv.x = fmaf(a, pv.x, xv.x);
            xv.y = fmaf(a, pv.y, xv.y);
            rv.x = fmaf(-a, qv.x, rv.x);
            rv.y = fmaf(-a, qv.y, rv.y);
            S.x[i] = xv;
            S.r[i] = rv;
        }
        acc += rdotb(rv, rv);
    }
    bred(acc, &partial[blockIdx.x]);
}

__global__ void k_bcg_beta(const BatchSys *__restrict__ sys, int nsys, const double *__restrict__ partial,
                           double *__restrict__ scal)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    double *T = scal + s * kS;
    const double rr_new = sys_sum(sys[s], partial);
    if (T[B_DONE] != 0) {
        T[B_BETA] = 0;
        return;
    }
    T[B_ITERS] += 1;
    const double tol = T[B_TOL];
    if ((tol > 0 && sqrt(rr_new) <= tol * sqrt(T[B_BN2])) || rr_new == 0) T[B_DONE] = 1;
    T[B_BETA] = rr_new / T[B_RR];
    T[B_RR] = rr_new;
}

__global__ void __launch_bounds__(256) k_bcg_p(const BatchSys *__restrict__ sys, const int2 *__restrict__ vtab,
                                               const double *__restrict__ scal)
{
    const int sid = vtab[blockIdx.x].x;
    if (scal[sid * kS + B_DONE] != 0) return;
    const float b = (float)scal[sid * kS + B_BETA];
    BLOOP(i, e, S)
    {
        const float2 rv = S.r[i], pv = S.p[i];
        S.p[i] = make_float2(fmaf(b, pv.x, rv.x), fmaf(b, pv.y, rv.y));
    }
}

__global__ void k_biters(const double *__restrict__ scal, int nsys, int *__restrict__ out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsys) out[s] = (int)scal[s * kS + B_ITERS];
}

// ----------------------------------------------------------------- host
template <typename T>
static int dalloc(nufft3d_batch *b, T **p, size_t n)
{
    NUFFT_DEVICE_LOCK;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) return fail(NUFFT3D_ERR_NOMEM, std::string("batch: ") + cudaGetErrorString(e));
    b->frees.push_back(*p);
    return NUFFT3D_SUCCESS;
}

static void fill_fft(nufft3d_batch *b, int v, BatchFFT *d, int stage)
{
    nufft3d_plan *p = b->plans[v];
    const int nc = b->nc[v];
    const int64_t K1 = p->geom.K[0], K2 = p->geom.K[1], K3 = p->geom.K[2];
    const int64_t N2 = p->N[1], N3 = p->N[2];
    const int64_t row = K1 * nc;
    int64_t nblk = 0;
    std::memset(d, 0, sizeof(*d));
    d->U = p->U;
    d->N1 = p->N[0];
    d->N23 = (int)(N2 * N3);
    d->nc = nc;
    switch (stage) {
    case FX: d->fd = p->fft[0]; break;
    case IX: d->fd = p->fft[0]; d->scale = 1.f; break;
    case FY:
        d->fd = p->fft[1];
        d->lp = make_linepass((int)N3, row, (int)N2, (int)K2, (int)N2, 1, 0, row, row, N2 * row, K2 * row, &nblk);
        break;
    case FZ:
        d->fd = p->fft[2];
        d->lp = make_linepass((int)K2, row, (int)N3, (int)K3, (int)N3, 1, 0, K2 * row, K2 * row, row, row, &nblk);
        break;
    case IZ:
        d->fd = p->fft[2];
        d->inv = 1;
        d->lp = make_linepass((int)K2, row, (int)K3, (int)N3, (int)N3, 0, 1, K2 * row, K2 * row, row, row, &nblk);
        break;
    case IY:
        d->fd = p->fft[1];
        d->inv = 1;
        d->lp = make_linepass((int)N3, row, (int)K2, (int)N2, (int)N2, 0, 1, row, row, K2 * row, N2 * row, &nblk);
        break;
    }
}

static int64_t fft_blocks(const nufft3d_plan *p, const BatchFFT &d, int stage, int nc)
{
    if (stage == FX || stage == IX) return (int64_t)d.N23 * ((nc + kMaxLineCoilsHost - 1) / kMaxLineCoilsHost);
    if (stage == FY || stage == IY) return (int64_t)p->N[2] * d.lp.nchunks;
    return (int64_t)p->geom.K[1] * d.lp.nchunks;  // FZ, IZ
}

static int upload(nufft3d_batch *b, cudaStream_t s)
{
    // host staging layout: gather tensor maps, gat, spr, pout, pin
    size_t off = 0;
    char *h = static_cast<char *>(b->stage);
    NUFFT_CUDA_TRY(cudaEventSynchronize(b->up_done));  // previous upload has left the staging buffer
    std::memcpy(h, b->h_tmaps.data(), b->h_tmaps.size() * sizeof(CUtensorMap));
    off += b->h_tmaps.size() * sizeof(CUtensorMap);
    std::memcpy(h + off, b->h_gat.data(), b->h_gat.size() * sizeof(BatchInterp));
    off += b->h_gat.size() * sizeof(BatchInterp);
    std::memcpy(h + off, b->h_spr.data(), b->h_spr.size() * sizeof(BatchInterp));
    off += b->h_spr.size() * sizeof(BatchInterp);
    std::memcpy(h + off, b->h_pout.data(), b->h_pout.size() * sizeof(BatchPerm));
    off += b->h_pout.size() * sizeof(BatchPerm);
    std::memcpy(h + off, b->h_pin.data(), b->h_pin.size() * sizeof(BatchPerm));
    off += b->h_pin.size() * sizeof(BatchPerm);
    NUFFT_CUDA_TRY(cudaMemcpyAsync(b->dstage, b->stage, off, cudaMemcpyHostToDevice, s));
    NUFFT_CUDA_TRY(cudaEventRecord(b->up_done, s));
    return NUFFT3D_SUCCESS;
}

// Set the per-call pointers of every stage.  mode 0: forward x -> k;
// 1: adjoint k -> x (wsorted = per-volume weights or null); 2: normal
// x -> y with y = A'WA x + damp^2 x (W = d).
static void set_io(nufft3d_batch *b, int mode, const float2 *const *in, float2 *const *out, double damp)
{
    for (int v = 0; v < b->nvol; ++v) {
        nufft3d_plan *p = b->plans[v];
        Scratch &S = p->scratch;
        BatchFFT *f = nullptr;
        // forward FFT chain: in -> B1 -> B2 -> G
        f = &b->h_fft[FX][v];
        f->in = in[v];
        f->out = S.B1;
        f = &b->h_fft[FY][v];
        f->in = S.B1;
        f->out = S.B2;
        f = &b->h_fft[FZ][v];
        f->in = S.B2;
        f->out = S.G;
        // adjoint FFT chain: G -> B2 -> B1 -> out
        f = &b->h_fft[IZ][v];
        f->in = S.G;
        f->out = S.B2;
        f = &b->h_fft[IY][v];
        f->in = S.B2;
        f->out = S.B1;
        f = &b->h_fft[IX][v];
        f->in = S.B1;
        f->out = out[v];
        f->addend = mode == 2 ? in[v] : nullptr;
        f->add_coef = (float)(damp * damp);
        f->scale = mode == 1 ? (float)(1.0 / std::sqrt((double)p->nnz)) : 1.f;
        BatchInterp &g = b->h_gat[v];
        g.in = S.G;
        g.out = S.ks;
        // bulk tile copies: maps of this call's grid (encoded per call, so a
        // grid reallocated between calls never leaves a stale map)
        g.tmap_ok = 0;
        g.tmaps = b->d_tmaps + 4 * v;
        for (int lw = 1; lw < 4; ++lw)
            if (encode_gather_map(p, S.G, b->nc[v], 1 << lw, &b->h_tmaps[4 * v + lw])) g.tmap_ok |= 1 << lw;
        g.scale = mode == 2 ? (float)(1.0 / (double)p->nnz) : (float)(1.0 / std::sqrt((double)p->nnz));
        g.wsample = mode == 2 ? p->d : nullptr;
        BatchInterp &sp = b->h_spr[v];
        sp.in = S.ks;
        sp.out = S.G;
        BatchPerm &po = b->h_pout[v];
        po.in = S.ks;
        po.out = out[v];
        po.scale = 1.f;
        BatchPerm &pi = b->h_pin[v];
        pi.in = in[v];
        pi.out = S.ks;
        pi.w = mode == 3 ? p->d : nullptr;  // mode 3: adjoint of W.*raw (iNUFT right-hand side)
    }
}

static int zero_grids(nufft3d_batch *b, cudaStream_t s)
{
    for (int v = 0; v < b->nvol; ++v) {
        nufft3d_plan *p = b->plans[v];
        const size_t bytes = (size_t)p->geom.K[0] * p->geom.K[1] * p->geom.K[2] * b->nc[v] * sizeof(float2);
        NUFFT_CUDA_TRY(cudaMemsetAsync(p->scratch.G, 0, bytes, s));
    }
    return NUFFT3D_SUCCESS;
}

// FFT passes.  A volume whose x pass fills the GPU on its own (at least 4
// blocks per SM) runs its chain of passes volume by volume (x -> y -> z, or
// back), so each intermediate is still in L2 when the next pass reads it;
// running a stage for all volumes first would evict it.  The smaller volumes
// share one launch per stage and transform length (descriptors by value as
// kernel parameters, kBatchParamVols volumes per launch).
static int run_fft_small(nufft3d_batch *b, int st, int kind, cudaStream_t s)
{
    BatchFFTParams P;
    for (auto &g : b->fgroups[st]) {
        std::vector<size_t> small;
        for (size_t i = 0; i < g.vols.size(); ++i)
            if (!b->chain[g.vols[i]]) small.push_back(i);
        for (size_t i0 = 0; i0 < small.size(); i0 += kBatchParamVols) {
            std::memset(&P, 0, sizeof(P));
            const size_t i1 = std::min(small.size(), i0 + kBatchParamVols);
            P.nvol = (int)(i1 - i0);
            int acc = 0;
            for (size_t i = i0; i < i1; ++i) {
                const int j = (int)(i - i0);
                P.first[j] = acc;
                P.nch[j] = g.nch[small[i]];
                P.v[j] = b->h_fft[st][g.vols[small[i]]];
                acc += g.blocks[small[i]];
            }
            P.first[P.nvol] = acc;
            NUFFT_TRY(launch_fft_batch_p(P, kind, g.smem, b->rare, kind == 1 ? g.r1 : 0, s));
        }
    }
    return NUFFT3D_SUCCESS;
}

static int run_fft_chains(nufft3d_batch *b, bool forward, cudaStream_t s)
{
    for (int v = 0; v < b->nvol; ++v) {
        if (!b->chain[v]) continue;
        nufft3d_plan *p = b->plans[v];
        const int nc = b->nc[v];
        if (forward) {
            const BatchFFT &x = b->h_fft[FX][v], &y = b->h_fft[FY][v], &z = b->h_fft[FZ][v];
            NUFFT_TRY(launch_fx(p, x.in, x.out, nc, s));
            NUFFT_TRY(launch_fy(p, y.in, y.out, nc, s));
            if (!b->is2d) NUFFT_TRY(launch_fz(p, z.in, z.out, nc, s));
        } else {
            const BatchFFT &z = b->h_fft[IZ][v], &y = b->h_fft[IY][v], &x = b->h_fft[IX][v];
            if (!b->is2d) NUFFT_TRY(launch_iz(p, z.in, z.out, nc, s));
            NUFFT_TRY(launch_iy(p, y.in, y.out, nc, s));
            NUFFT_TRY(launch_ix(p, x.in, x.out, nc, x.scale, x.addend, x.add_coef, s));
        }
    }
    return NUFFT3D_SUCCESS;
}

static int run_interp(nufft3d_batch *b, bool gather, cudaStream_t s)
{
    for (auto &g : b->igroups)
        NUFFT_TRY(launch_interp_batch(gather, g.cb, b->R, b->radial, gather ? b->gat : b->spr, g.tab, g.n, g.smem,
                                      b->plans[0]->kb, b->work, b->plans[0]->sm_count, s, b->stored_h));
    return NUFFT3D_SUCCESS;
}

static int run_fwd_chain(nufft3d_batch *b, cudaStream_t s)
{
    NUFFT_TRY(run_fft_chains(b, true, s));
    NUFFT_TRY(run_fft_small(b, FX, 0, s));
    NUFFT_TRY(run_fft_small(b, FY, 1, s));
    if (!b->is2d) NUFFT_TRY(run_fft_small(b, FZ, 1, s));
    return run_interp(b, true, s);
}

static int run_adj_chain(nufft3d_batch *b, cudaStream_t s)
{
    NUFFT_TRY(zero_grids(b, s));
    NUFFT_TRY(run_interp(b, false, s));
    NUFFT_TRY(run_fft_chains(b, false, s));
    if (!b->is2d) NUFFT_TRY(run_fft_small(b, IZ, 1, s));
    NUFFT_TRY(run_fft_small(b, IY, 1, s));
    return run_fft_small(b, IX, 2, s);
}

static void free_batch(nufft3d_batch *b)
{
    NUFFT_DEVICE_LOCK;
    for (void *q : b->frees) cudaFree(q);
    b->frees.clear();
    if (b->stage) cudaFreeHost(b->stage);
    if (b->up_done) cudaEventDestroy(b->up_done);
    if (b->own) cudaStreamDestroy(b->own);
}

} // namespace nufft3d

extern "C" int nufft3d_batch_create(nufft3d_plan *const *plans, const int *nc, int nvol, nufft3d_batch **out)
{
    clear_error();
    if (!plans || !nc || !out || nvol < 1) return fail(NUFFT3D_ERR_ARG, "invalid batch arguments");
    *out = nullptr;
    for (int v = 0; v < nvol; ++v) {
        if (!plans[v] || nc[v] < 1) return fail(NUFFT3D_ERR_ARG, "invalid plan or coil count in batch");
        for (int u = 0; u < v; ++u)
            if (plans[u] == plans[v])
                return fail(NUFFT3D_ERR_ARG, "a batch needs one plan handle per volume (use nufft3d_plan_share)");
        if (plans[v]->device != plans[0]->device) return fail(NUFFT3D_ERR_ARG, "batch plans on different devices");
        if (plans[v]->geom.R != plans[0]->geom.R || plans[v]->geom.radial != plans[0]->geom.radial ||
            plans[v]->geom.is2d != plans[0]->geom.is2d ||
            std::memcmp(&plans[v]->kb, &plans[0]->kb, sizeof(KBParams)) != 0)
            return fail(NUFFT3D_ERR_UNSUPPORTED,
                        "batch volumes must share the kernel (J, u, alpha, radial) and 2-D/3-D");
    }
    NUFFT_DEVICE_LOCK;
    int prev = -1;
    cudaGetDevice(&prev);
    const int dev = plans[0]->device;
    if (prev != dev) cudaSetDevice(dev);
    struct Restore {
        int prev, dev;
        ~Restore()
        {
            if (prev >= 0 && prev != dev) cudaSetDevice(prev);
        }
    } restore{prev, dev};

    nufft3d_batch *b = new nufft3d_batch();
    b->device = dev;
    b->nvol = nvol;
    b->plans.assign(plans, plans + nvol);
    b->nc.assign(nc, nc + nvol);
    b->R = plans[0]->geom.R;
    b->radial = plans[0]->geom.radial;
    b->is2d = plans[0]->geom.is2d;
    int maxnc = 1;
    for (int v = 0; v < nvol; ++v) maxnc = std::max(maxnc, nc[v]);
    int cb = 1;
    while (cb < maxnc && cb < 8) cb *= 2;
    if (b->R >= 4 && cb > 4) cb = 4;
    b->cb = cb;
    auto bail = [&](int st) {
        std::string msg = nufft3d_last_error();
        free_batch(b);
        delete b;
        return fail(st, msg);
    };
    for (int v = 0; v < nvol; ++v) {
        int st = ensure_scratch(plans[v], nc[v]);
        if (st != NUFFT3D_SUCCESS) return bail(st);
        if (needs_rare(plans[v]->fft[0]) || needs_rare(plans[v]->fft[1]) || needs_rare(plans[v]->fft[2]))
            b->rare = true;
    }
    // FFT launches grouped by transform length: per group its volumes, their
    // block counts and coil chunks (descriptors go by value at launch)
    for (int st = 0; st < NFFT; ++st) {
        b->h_fft[st].resize(nvol);
        for (int v = 0; v < nvol; ++v) {
            fill_fft(b, v, &b->h_fft[st][v], st);
            const BatchFFT &d = b->h_fft[st][v];
            auto &groups = b->fgroups[st];
            size_t gi = 0;
            while (gi < groups.size() && groups[gi].K != d.fd.n) ++gi;
            if (gi == groups.size()) {
                nufft3d_batch::FGroup fg;
                fg.K = d.fd.n;
                groups.push_back(fg);
            }
            nufft3d_batch::FGroup &g = groups[gi];
            g.vols.push_back(v);
            if (st == FX || st == IX) {
                const int nch = (nc[v] + kMaxLineCoilsHost - 1) / kMaxLineCoilsHost;
                g.blocks.push_back(d.N23 * nch);
                g.nch.push_back(nch);
                g.smem = std::max(g.smem, line_smem(std::min(nc[v], kMaxLineCoilsHost), d.fd.n));
            } else {
                g.blocks.push_back((int)fft_blocks(plans[v], d, st, nc[v]));
                g.nch.push_back(1);
                g.smem = std::max(g.smem, line_smem(d.lp.vec, d.fd.n));
                if (d.lp.vec != 16) g.all_vec16 = false;
            }
        }
        for (auto &g : b->fgroups[st])
            g.r1 = (st == FX || st == IX) ? 0 : batch_four_step(g.K, g.all_vec16);
    }
    b->chain.assign(nvol, 0);
    for (int v = 0; v < nvol; ++v) {
        const int nch = (nc[v] + kMaxLineCoilsHost - 1) / kMaxLineCoilsHost;
        b->chain[v] = (int64_t)b->h_fft[FX][v].N23 * nch >= 4 * (int64_t)plans[v]->sm_count;
    }
    {
        // interpolation: (volume, piece, first coil), heaviest pieces first
        struct E {
            int count;
            int4 e;
        };
        std::vector<E> ents;
        int maxcand = 0;
        b->h_gat.resize(nvol);
        b->h_spr.resize(nvol);
        for (int v = 0; v < nvol; ++v) {
            nufft3d_plan *p = plans[v];
            std::vector<int4> blk(p->n_blocks);
            if (p->n_blocks && cudaMemcpy(blk.data(), p->blocks, sizeof(int4) * p->n_blocks, cudaMemcpyDeviceToHost) != cudaSuccess)
                return bail(fail(NUFFT3D_ERR_CUDA, "batch: reading tile pieces failed"));
            for (int64_t k = 0; k < p->n_blocks; ++k)
                for (int c0 = 0; c0 < nc[v]; c0 += cb) {
                    int w = 1;  // this chunk's width: smallest power of two covering its coils
                    while (w < nc[v] - c0 && w < cb) w *= 2;
                    ents.push_back({blk[k].z, make_int4(v, (int)k, c0, w)});
                }
            BatchInterp d;
            std::memset(&d, 0, sizeof(d));
            d.samples = p->samples;
            d.blocks = p->blocks;
            d.g = p->geom;
            d.kb = p->kb;
            d.cand = p->cand_desc;
            d.tap_rows = p->tap_rows;
            d.tap_ent = p->tap_ent;
            d.status = plan_status(p);  // timeouts are reported on the volume's plan
            if (v == 0) b->stored_h = true;
            if (!p->tap_ent) b->stored_h = false;
            d.nc = nc[v];
            b->h_gat[v] = d;
            b->h_spr[v] = d;
            maxcand = std::max(maxcand, p->n_cand);
        }
        std::stable_sort(ents.begin(), ents.end(), [](const E &a, const E &c) { return a.count > c.count; });
        for (int w = cb; w >= 1; w /= 2) {
            std::vector<int4> tab;
            for (auto &e : ents)
                if (e.e.w == w) tab.push_back(make_int4(e.e.x, e.e.y, e.e.z, 0));
            if (tab.empty()) continue;
            nufft3d_batch::IGroup ig;
            ig.cb = w;
            ig.n = (int)tab.size();
            const size_t plane = smem_plane_bytes(b->R, w);
            const size_t iplane = (size_t)(((plane / (w * sizeof(float2)) + 29) / 32) * 32 + 2) * w * 2 * sizeof(int);
            // + tile alignment; the spread keeps its candidates as packed pairs
            ig.smem = std::max(plane, iplane) +
                      std::max(cand_smem_bytes(maxcand), cand_pairs_bytes(b->h_spr[0].cand)) + 128;
            int s2 = dalloc(b, &ig.tab, tab.size());
            if (s2 != NUFFT3D_SUCCESS) return bail(s2);
            if (cudaMemcpy(ig.tab, tab.data(), tab.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess)
                return bail(fail(NUFFT3D_ERR_CUDA, "batch table upload failed"));
            b->igroups.push_back(ig);
        }
    }
    {
        std::vector<int4> tab;
        b->h_pout.resize(nvol);
        b->h_pin.resize(nvol);
        for (int v = 0; v < nvol; ++v) {
            nufft3d_plan *p = plans[v];
            for (int64_t k = 0; k < (p->M + 255) / 256; ++k) tab.push_back(make_int4(v, (int)k, 0, 0));
            BatchPerm d;
            std::memset(&d, 0, sizeof(d));
            d.inv = p->inv;
            d.M = p->M;
            d.nc = nc[v];
            d.scale = 1.f;
            b->h_pout[v] = d;
            b->h_pin[v] = d;
        }
        b->pn = (int)tab.size();
        int s2 = dalloc(b, &b->ptab, tab.size());
        if (s2 != NUFFT3D_SUCCESS) return bail(s2);
        if (!tab.empty() && cudaMemcpy(b->ptab, tab.data(), tab.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(NUFFT3D_ERR_CUDA, "batch table upload failed"));
    }
    // one device buffer for all descriptors, mirrored by pinned staging
    b->h_tmaps.assign((size_t)4 * nvol, CUtensorMap{});
    size_t bytes = 4 * nvol * sizeof(CUtensorMap) + 2 * nvol * sizeof(BatchInterp) + 2 * nvol * sizeof(BatchPerm);
    b->stage_bytes = bytes;
    if (cudaMallocHost(&b->stage, bytes) != cudaSuccess) return bail(fail(NUFFT3D_ERR_NOMEM, "batch staging"));
    char *base = nullptr;
    int s2 = dalloc(b, &base, bytes);
    if (s2 != NUFFT3D_SUCCESS) return bail(s2);
    b->dstage = base;
    b->d_tmaps = reinterpret_cast<CUtensorMap *>(base);  // cudaMalloc alignment covers the 64-byte rule
    size_t off = 4 * nvol * sizeof(CUtensorMap);
    b->gat = reinterpret_cast<BatchInterp *>(base + off);
    off += nvol * sizeof(BatchInterp);
    b->spr = reinterpret_cast<BatchInterp *>(base + off);
    off += nvol * sizeof(BatchInterp);
    b->pout = reinterpret_cast<BatchPerm *>(base + off);
    off += nvol * sizeof(BatchPerm);
    b->pin = reinterpret_cast<BatchPerm *>(base + off);
    if (cudaEventCreateWithFlags(&b->up_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(b->up_done, 0) != cudaSuccess)
        return bail(fail(NUFFT3D_ERR_CUDA, "batch event"));
    if (cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(NUFFT3D_ERR_CUDA, "batch stream"));
    s2 = dalloc(b, &b->work, 16);
    if (s2 != NUFFT3D_SUCCESS) return bail(s2);
    *out = b;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_batch_destroy(nufft3d_batch *b)
{
    clear_error();
    if (!b) return NUFFT3D_SUCCESS;
    {
        NUFFT_DEVICE_LOCK;
        cudaStreamSynchronize(b->own);
        for (int v = 0; v < b->nvol; ++v)
            if (b->plans[v]->own_stream) cudaStreamSynchronize(b->plans[v]->own_stream);
        cudaDeviceSynchronize();
    }
    free_batch(b);
    delete b;
    return NUFFT3D_SUCCESS;
}

static int batch_guard_check(nufft3d_batch *b, const void *a, const void *c)
{
    if (!b) return fail(NUFFT3D_ERR_ARG, "batch is NULL");
    if (!a || !c) return fail(NUFFT3D_ERR_ARG, "NULL pointer array");
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_batch_forward(nufft3d_batch *b, const float *const *x, float *const *k, void *stream)
{
    clear_error();
    NUFFT_TRY(batch_guard_check(b, x, k));
    cudaStream_t s = (cudaStream_t)stream;
    for (int v = 0; v < b->nvol; ++v)
        if (!x[v] || !k[v]) return fail(NUFFT3D_ERR_ARG, "NULL data pointer in batch");
    set_io(b, 0, reinterpret_cast<const float2 *const *>(x), reinterpret_cast<float2 *const *>(k), 0.0);
    NUFFT_TRY(upload(b, s));
    NUFFT_TRY(run_fwd_chain(b, s));
    return launch_perm_batch(true, b->pout, b->ptab, b->pn, s);
}

extern "C" int nufft3d_batch_adjoint(nufft3d_batch *b, const float *const *k, float *const *x, void *stream)
{
    clear_error();
    NUFFT_TRY(batch_guard_check(b, k, x));
    cudaStream_t s = (cudaStream_t)stream;
    for (int v = 0; v < b->nvol; ++v)
        if (!x[v] || !k[v]) return fail(NUFFT3D_ERR_ARG, "NULL data pointer in batch");
    set_io(b, 1, reinterpret_cast<const float2 *const *>(k), reinterpret_cast<float2 *const *>(x), 0.0);
    NUFFT_TRY(upload(b, s));
    NUFFT_TRY(launch_perm_batch(false, b->pin, b->ptab, b->pn, s));
    return run_adj_chain(b, s);
}

// Batched iNUFT (CG, W = d): raw[v] [M_v nc_v] -> x[v] [N_v^3 nc_v] on the device.
extern "C" int nufft3d_batch_inverse(nufft3d_batch *b, const float *const *raw, float *const *x, int maxit,
                                     double damp, double tol, int *iters_host, void *stream)
{
    clear_error();
    NUFFT_TRY(batch_guard_check(b, raw, x));
    if (maxit < 0) return fail(NUFFT3D_ERR_ARG, "maxit must be a nonnegative integer");
    if (!std::isfinite(damp) || damp < 0) return fail(NUFFT3D_ERR_ARG, "damp must be finite and nonnegative");
    cudaStream_t user = (cudaStream_t)stream;
    cudaStream_t s = b->own;
    cudaEvent_t ev = nullptr;
    NUFFT_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    struct EvG {
        cudaEvent_t e;
        ~EvG() { cudaEventDestroy(e); }
    } evg{ev};
    NUFFT_CUDA_TRY(cudaEventRecord(ev, user));
    NUFFT_CUDA_TRY(cudaStreamWaitEvent(s, ev, 0));
    // per-volume solver vectors and the system table
    std::vector<BatchSys> sys;
    std::vector<int2> vtab;
    for (int v = 0; v < b->nvol; ++v) {
        nufft3d_plan *p = b->plans[v];
        NUFFT_TRY(ensure_solver(p, b->nc[v]));
        SolverWork &w = p->solver;
        const size_t n = (size_t)p->N[0] * p->N[1] * p->N[2];
        for (int c = 0; c < b->nc[v]; ++c) {
            BatchSys S;
            S.x = reinterpret_cast<float2 *>(x[v]) + c * n;
            S.r = w.r + c * n;
            S.p = w.p + c * n;
            S.q = w.q + c * n;
            S.n = (int64_t)n;
            S.first = (int)vtab.size();
            S.nblk = (int)((n + kVecChunk - 1) / kVecChunk);
            for (int k = 0; k < S.nblk; ++k) vtab.push_back(make_int2((int)sys.size(), k));
            sys.push_back(S);
        }
    }
    if (b->nsys < (int)sys.size() || b->vn < (int)vtab.size()) {
        NUFFT_TRY(dalloc(b, &b->sys, sys.size()));
        NUFFT_TRY(dalloc(b, &b->vtab, vtab.size()));
        NUFFT_TRY(dalloc(b, &b->partial, vtab.size()));
        NUFFT_TRY(dalloc(b, &b->scal, sys.size() * kS));
    }
    b->nsys = (int)sys.size();
    b->vn = (int)vtab.size();
    NUFFT_CUDA_TRY(cudaMemcpyAsync(b->sys, sys.data(), sys.size() * sizeof(BatchSys), cudaMemcpyHostToDevice, s));
    NUFFT_CUDA_TRY(cudaMemcpyAsync(b->vtab, vtab.data(), vtab.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
    // b = A'W raw (W = d) into r; p = r; x = 0
    std::vector<float2 *> rptr(b->nvol), pptr(b->nvol), qptr(b->nvol);
    for (int v = 0; v < b->nvol; ++v) {
        rptr[v] = b->plans[v]->solver.r;
        pptr[v] = b->plans[v]->solver.p;
        qptr[v] = b->plans[v]->solver.q;
    }
    set_io(b, 3, reinterpret_cast<const float2 *const *>(raw), rptr.data(), 0.0);
    for (int v = 0; v < b->nvol; ++v) b->h_fft[IX][v].scale = (float)(1.0 / std::sqrt((double)b->plans[v]->nnz));
    NUFFT_TRY(upload(b, s));
    NUFFT_TRY(launch_perm_batch(false, b->pin, b->ptab, b->pn, s));
    NUFFT_TRY(run_adj_chain(b, s));
    for (int v = 0; v < b->nvol; ++v) {
        const size_t bytes = (size_t)b->plans[v]->solver.nimg * b->nc[v] * sizeof(float2);
        NUFFT_CUDA_TRY(cudaMemcpyAsync(pptr[v], rptr[v], bytes, cudaMemcpyDeviceToDevice, s));
        NUFFT_CUDA_TRY(cudaMemsetAsync(x[v], 0, bytes, s));
    }
    const int tb = 128, nsb = (b->nsys + tb - 1) / tb;
    if (maxit > 0) {
        k_bdot<<<b->vn, 256, 0, s>>>(b->sys, b->vtab, 1, b->partial);
        k_bcg_init<<<nsb, tb, 0, s>>>(b->sys, b->nsys, b->partial, b->scal, tol);
        NUFFT_CUDA_TRY(cudaGetLastError());
        // normal operator p -> q for every volume
        set_io(b, 2, reinterpret_cast<const float2 *const *>(pptr.data()), qptr.data(), damp);
        NUFFT_TRY(upload(b, s));
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        NUFFT_DEVICE_LOCK;
        NUFFT_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int st = run_fwd_chain(b, s);
        if (st == NUFFT3D_SUCCESS) st = run_adj_chain(b, s);
        if (st == NUFFT3D_SUCCESS) {
            k_bdot<<<b->vn, 256, 0, s>>>(b->sys, b->vtab, 0, b->partial);
            k_bcg_alpha<<<nsb, tb, 0, s>>>(b->sys, b->nsys, b->partial, b->scal);
            k_bcg_xr<<<b->vn, 256, 0, s>>>(b->sys, b->vtab, b->scal, b->partial);
            k_bcg_beta<<<nsb, tb, 0, s>>>(b->sys, b->nsys, b->partial, b->scal);
            k_bcg_p<<<b->vn, 256, 0, s>>>(b->sys, b->vtab, b->scal);
            if (cudaGetLastError() != cudaSuccess) st = fail(NUFFT3D_ERR_CUDA, "batched CG launch failed");
        }
        cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (st != NUFFT3D_SUCCESS) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (ce != cudaSuccess) return fail(NUFFT3D_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return fail(NUFFT3D_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(ce));
        for (int it = 0; it < maxit && ce == cudaSuccess; ++it) ce = cudaGraphLaunch(exec, s);
        cudaGraphExecDestroy(exec);
        if (ce != cudaSuccess) return fail(NUFFT3D_ERR_CUDA, std::string("batch graph launch: ") + cudaGetErrorString(ce));
    } else {
        // regridding: x = A'W raw
        for (int v = 0; v < b->nvol; ++v) {
            const size_t bytes = (size_t)b->plans[v]->solver.nimg * b->nc[v] * sizeof(float2);
            NUFFT_CUDA_TRY(cudaMemcpyAsync(x[v], rptr[v], bytes, cudaMemcpyDeviceToDevice, s));
        }
    }
    if (iters_host) {
        int *di = nullptr;
        NUFFT_DEVICE_LOCK;
        NUFFT_CUDA_TRY(cudaMalloc(&di, sizeof(int) * b->nsys));
        k_biters<<<nsb, tb, 0, s>>>(b->scal, b->nsys, di);
        cudaMemcpyAsync(iters_host, di, sizeof(int) * b->nsys, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        cudaFree(di);
        if (maxit == 0)
            for (int i = 0; i < b->nsys; ++i) iters_host[i] = 0;
    }
    NUFFT_CUDA_TRY(cudaEventRecord(ev, s));
    NUFFT_CUDA_TRY(cudaStreamWaitEvent(user, ev, 0));
    return NUFFT3D_SUCCESS;
}
