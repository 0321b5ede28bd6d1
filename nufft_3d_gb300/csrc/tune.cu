// Plan-time autotuner: picks the interpolation piece size (the largest
// number of samples one block takes from a tile) and the coils handled per
// interpolation pass by timing fNUFT + aNUFT on the plan itself.
//
// The tile shape is not searched: the kernels' tiles are compile-time shapes
// (8^3 in 3-D, 32x32 in 2-D) whose shared-memory planes and bank layout are
// fixed per kernel instance.  What does vary with the trajectory and the coil
// count is the balance between per-piece overhead (staging the padded tile,
// the spread's scale pass and halo flush) and load balance over the SMs
// (pieces are taken largest first from a work counter), and between sharing
// a candidate evaluation over more coils and the shared memory a wider pass
// needs.  Candidates: pieces of 1024, 2048 or 4096 samples, 2 / 4 / 8 coils
// per pass (within what the plan's shared memory allows).  Larger pieces are
// not tried: the spread's fixed-point scale leaves headroom for the largest
// summed weight at a tile point, which grows with the piece, so each
// doubling of the piece can cost one bit of the adjoint's precision
// (16384-sample pieces measured 3.9e-6 against FP64 at 128^3, 4096 about
// 1e-6, for a 0.3 % shorter step).
//
// Results are cached per process under a key of the plan's shape (N, K, J,
// u, kernel, 2-D), the coil count, the number of in-bounds samples and their
// mean count per occupied tile (both rounded to powers of two), and the
// device's SM count: later plans with the same key take the cached choice
// without timing (the serving loop builds many plans of a few shapes).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>

#include "internal.h"

namespace nufft3d {

// Deterministic nonzero complex values (timing data: the spread skips pieces
// whose values are all zero, so zeros would not time the real work).
__global__ void k_fill_pattern(float2 *__restrict__ a, int64_t n, unsigned seed)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned h = (unsigned)i * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    a[i] = make_float2((float)(h & 0xFFFF) * (1.f / 65536.f) - 0.5f, (float)(h >> 16) * (1.f / 65536.f) - 0.5f);
}

struct TuneChoice {
    int S, cpp;
    double ms;
};

static std::mutex g_tune_mu;
static std::map<std::string, TuneChoice> g_tune_cache;

static int log2_bucket(double v) { return v > 0 ? (int)std::lround(std::log2(v)) : -1; }

static std::string tune_key(const nufft3d_plan *p, int nc)
{
    int64_t occupied = 0;
    for (int32_t c : p->tile_counts) occupied += c > 0;
    const double per_tile = occupied ? (double)p->nnz / (double)occupied : 0.0;
    char buf[256];
    std::snprintf(buf, sizeof buf, "N%dx%dx%d K%dx%dx%d J%g u%g r%d nc%d nnz%d dens%d sm%d", p->N[0], p->N[1],
                  p->N[2], p->geom.K[0], p->geom.K[1], p->geom.K[2], p->J, p->u, p->radial, nc,
                  log2_bucket((double)p->nnz), log2_bucket(per_tile), p->sm_count);
    return buf;
}

// Milliseconds of one fNUFT + aNUFT of nc coils on the plan's own stream
// (mean of `reps` after one untimed pass).
static int time_pair(nufft3d_plan *p, const float2 *x, float2 *k, float2 *x2, int nc, int reps, double *ms)
{
    cudaStream_t s = p->own_stream;
    NUFFT_TRY(op_forward(p, x, k, nc, s));
    NUFFT_TRY(op_adjoint(p, k, x2, nc, s));
    cudaEvent_t a = nullptr, b = nullptr;
    NUFFT_CUDA_TRY(cudaEventCreate(&a));
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return fail(NUFFT3D_ERR_CUDA, "cudaEventCreate failed");
    }
    int st = NUFFT3D_SUCCESS;
    cudaEventRecord(a, s);
    for (int r = 0; r < reps && st == NUFFT3D_SUCCESS; ++r) {
        st = op_forward(p, x, k, nc, s);
        if (st == NUFFT3D_SUCCESS) st = op_adjoint(p, k, x2, nc, s);
    }
    cudaEventRecord(b, s);
    float t = 0;
    if (st == NUFFT3D_SUCCESS) {
        const cudaError_t e = cudaEventSynchronize(b);
        if (e == cudaSuccess) cudaEventElapsedTime(&t, a, b);
        else st = fail(NUFFT3D_ERR_CUDA, std::string("tuning: ") + cudaGetErrorString(e));
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = t / reps;
    return st;
}

static int apply_choice(nufft3d_plan *p, int S, int cpp)
{
    p->coils_per_pass = cpp;
    if (S != p->piece_samples) NUFFT_TRY(rebuild_pieces(p, S));
    return NUFFT3D_SUCCESS;
}

} // namespace nufft3d

using namespace nufft3d;

extern "C" int nufft3d_plan_tune(nufft3d_plan *p, int nc, int force, nufft3d_tune_result *res)
{
    clear_error();
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    if (nc < 1) return fail(NUFFT3D_ERR_ARG, "number of coils must be >= 1");
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return fail(NUFFT3D_ERR_CUDA, "no CUDA device");
    if (prev != p->device && cudaSetDevice(p->device) != cudaSuccess)
        return fail(NUFFT3D_ERR_CUDA, "cannot select the plan's device");
    struct Restore {
        int dev, prev;
        ~Restore()
        {
            if (prev >= 0 && prev != dev) cudaSetDevice(prev);
        }
    } restore{p->device, prev};
    nufft3d_tune_result r{};
    r.samples_per_block = p->piece_samples;
    r.coils_per_pass = p->coils_per_pass;
    if (p->nnz == 0) {
        if (res) *res = r;
        return NUFFT3D_SUCCESS;
    }
    const std::string key = tune_key(p, nc);
    if (!force) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            NUFFT_TRY(apply_choice(p, it->second.S, it->second.cpp));
            r.samples_per_block = it->second.S;
            r.coils_per_pass = it->second.cpp;
            r.ms_best = it->second.ms;
            r.from_cache = 1;
            if (res) *res = r;
            return NUFFT3D_SUCCESS;
        }
    }
    // timing buffers: an image and samples of nc coils with nonzero values
    const size_t nimg = (size_t)p->N[0] * p->N[1] * p->N[2] * nc, nk = (size_t)p->M * nc;
    float2 *x = nullptr, *x2 = nullptr, *k = nullptr;
    {
        NUFFT_DEVICE_LOCK;
        if (cudaMalloc(&x, nimg * sizeof(float2)) != cudaSuccess || cudaMalloc(&x2, nimg * sizeof(float2)) != cudaSuccess ||
            cudaMalloc(&k, nk * sizeof(float2)) != cudaSuccess) {
            if (x) cudaFree(x);
            if (x2) cudaFree(x2);
            cudaGetLastError();
            return fail(NUFFT3D_ERR_NOMEM, "cannot allocate the tuning buffers");
        }
    }
    struct Free {
        float2 *a, *b, *c;
        ~Free()
        {
            NUFFT_DEVICE_LOCK;
            cudaFree(a);
            cudaFree(b);
            cudaFree(c);
        }
    } fr{x, x2, k};
    k_fill_pattern<<<(unsigned)((nimg + 255) / 256), 256, 0, p->own_stream>>>(x, (int64_t)nimg, 0x9E3779B9u);
    NUFFT_CUDA_TRY(cudaGetLastError());
    const int S0 = p->piece_samples, c0 = p->coils_per_pass;
    const int reps = 3;
    double best = 0, t_def = 0;
    int bS = S0, bc = c0;
    NUFFT_TRY(time_pair(p, x, k, x2, nc, reps, &t_def));
    best = t_def;
    int tried = 1;
    static const int kS[] = {1024, 2048, 4096};
    for (int cpp = 2; cpp <= p->max_coils_per_pass; cpp *= 2) {
        for (int S : kS) {
            if (S == S0 && cpp == c0) continue;
            NUFFT_TRY(apply_choice(p, S, cpp));
            double t = 0;
            NUFFT_TRY(time_pair(p, x, k, x2, nc, reps, &t));
            ++tried;
            if (t < best) {
                best = t;
                bS = S;
                bc = cpp;
            }
        }
    }
    NUFFT_TRY(apply_choice(p, bS, bc));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = TuneChoice{bS, bc, best};
    }
    r.samples_per_block = bS;
    r.coils_per_pass = bc;
    r.ms_best = best;
    r.ms_default = t_def;
    r.candidates = tried;
    if (res) *res = r;
    return NUFFT3D_SUCCESS;
}
