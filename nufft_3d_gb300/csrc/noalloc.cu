// Forward transform that allocates no device memory per call.
//
// The regular nufft3d_forward keeps its FFT and interpolation work buffers in
// the plan and allocates them (cudaMalloc) the first time a coil count is
// seen.  Some callers cannot allow that: cudaMalloc synchronises the whole
// device and can fail under memory pressure, so a latency-critical
// reconstruction loop, or a host application that hands the GPU's memory to
// its own pool and forbids other components from allocating, must not trigger
// it.  nufft3d_forward_noalloc runs the same kernels with their work buffers
// carved out of one fixed array in device global memory that is part of the
// library image itself (kNoAllocScratchBytes; every GPU that loads the
// library holds it until the process exits).  The plan is still created
// beforehand, at a point where allocating is acceptable.
//
// The array is shared by every call on a device, and it keeps whatever the
// previous call left in it: calls whose work overlaps on the GPU (two
// streams, two host threads) race on it and must be serialised by the
// caller.  The forward pipeline overwrites every scratch element it later
// reads, so nothing needs clearing between calls.
//
// The device address of the array is looked up once per device, on the first
// call made with that device current (cudaGetSymbolAddress); make that first
// call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "internal.h"

namespace nufft3d {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20; // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device.
static int noalloc_base(int dev, unsigned char **out)
{
    if (dev < 0 || dev >= kMaxDevices) return fail(NUFFT3D_ERR_UNSUPPORTED, "device ordinal too large");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(NUFFT3D_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_noalloc_ptr[dev] = ptr;
    }
    *out = static_cast<unsigned char *>(g_noalloc_ptr[dev]);
    return NUFFT3D_SUCCESS;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

} // namespace nufft3d

using namespace nufft3d;

extern "C" size_t nufft3d_forward_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int nufft3d_forward_noalloc(nufft3d_plan *p, const float *x, float *k, int nc, void *stream)
{
    clear_error();
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    if (!x || !k) return fail(NUFFT3D_ERR_ARG, "NULL data pointer");
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

    const Geom &g = p->geom;
    const size_t K1 = g.K[0], K2 = g.K[1], K3 = g.K[2];
    const size_t N2 = p->N[1], N3 = p->N[2];
    const size_t c8 = sizeof(float2) * (size_t)nc;
    const size_t bB1 = align256(K1 * N2 * N3 * c8), bB2 = align256(K1 * K2 * N3 * c8);
    const size_t bG = g.is2d ? 0 : align256(K1 * K2 * K3 * c8);
    const size_t bks = align256((size_t)(p->nnz > 0 ? p->nnz : 1) * c8);
    const size_t need = bB1 + bB2 + bG + bks;
    if (need > kNoAllocScratchBytes)
        return fail(NUFFT3D_ERR_SIZE, "nufft3d_forward_noalloc needs " + std::to_string(need) +
                                          " bytes of scratch for this plan and nc=" + std::to_string(nc) +
                                          "; the fixed scratch holds " + std::to_string(kNoAllocScratchBytes));
    unsigned char *base = nullptr;
    NUFFT_TRY(noalloc_base(p->device, &base));
    float2 *B1 = reinterpret_cast<float2 *>(base);
    float2 *B2 = reinterpret_cast<float2 *>(base + bB1);
    float2 *G = g.is2d ? B2 : reinterpret_cast<float2 *>(base + bB1 + bB2);
    float2 *ks = reinterpret_cast<float2 *>(base + bB1 + bB2 + bG);
    cudaStream_t s = (cudaStream_t)stream;
    float2 *kout = reinterpret_cast<float2 *>(k);
    if (p->nnz == 0) {
        NUFFT_CUDA_TRY(cudaMemsetAsync(kout, 0, (size_t)p->M * c8, s));
        return NUFFT3D_SUCCESS;
    }
    // fNUFT.m:4-9 with the same kernels as nufft3d_forward
    NUFFT_TRY(launch_fx(p, reinterpret_cast<const float2 *>(x), B1, nc, s));
    NUFFT_TRY(launch_fy(p, B1, B2, nc, s));
    if (!g.is2d) NUFFT_TRY(launch_fz(p, B2, G, nc, s));
    NUFFT_TRY(launch_gather(p, G, ks, nc, (float)(1.0 / std::sqrt((double)p->nnz)), nullptr, s));
    NUFFT_TRY(launch_permute_out(p, ks, kout, nc, 1.f, s));
    return NUFFT3D_SUCCESS;
}
