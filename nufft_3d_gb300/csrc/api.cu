// Operators and C-ABI entry points: fNUFT, aNUFT, iprojection, density.m.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "internal.h"

namespace nufft3d {

struct DevGuard {
    int prev = -1;
    explicit DevGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DevGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

static size_t img_elems(const nufft3d_plan *p) { return (size_t)p->N[0] * p->N[1] * p->N[2]; }

int ensure_scratch(nufft3d_plan *p, int nc)
{
    Scratch &s = p->scratch;
    if (s.nc >= nc) return NUFFT3D_SUCCESS;
    NUFFT_DEVICE_LOCK;
    const Geom &g = p->geom;
    const size_t K1 = g.K[0], K2 = g.K[1], K3 = g.K[2];
    const size_t N2 = p->N[1], N3 = p->N[2];
    const size_t nB1 = K1 * N2 * N3 * nc, nB2 = K1 * K2 * N3 * nc, nG = K1 * K2 * K3 * nc;
    const size_t nks = (size_t)(p->nnz > 0 ? p->nnz : 1) * nc;
    if (s.G && s.G != s.B2) cudaFree(s.G); // 2D: G aliases B2
    if (s.B1) cudaFree(s.B1);
    if (s.B2) cudaFree(s.B2);
    if (s.ks) cudaFree(s.ks);
    s = Scratch();
    auto A = [](float2 **ptr, size_t n) {
        return cudaMalloc((void **)ptr, n * sizeof(float2)) == cudaSuccess;
    };
    bool ok = A(&s.B1, nB1) && A(&s.B2, nB2) && (g.is2d || A(&s.G, nG)) && A(&s.ks, nks);
    if (!ok) {
        if (s.B1) cudaFree(s.B1);
        if (s.B2) cudaFree(s.B2);
        if (s.G) cudaFree(s.G);
        if (s.ks) cudaFree(s.ks);
        s = Scratch();
        cudaGetLastError();
        return fail(NUFFT3D_ERR_NOMEM, "cannot allocate interpolation/FFT scratch for nc=" + std::to_string(nc));
    }
    if (g.is2d) s.G = s.B2; // K3 = N3 = 1: the y-pass output is the grid
    s.nc = nc;
    s.bytes = (nB1 + nB2 + (g.is2d ? 0 : nG) + nks) * sizeof(float2);
    return NUFFT3D_SUCCESS;
}

static size_t grid_bytes(const nufft3d_plan *p, int nc)
{
    return (size_t)p->geom.K[0] * p->geom.K[1] * p->geom.K[2] * nc * sizeof(float2);
}

// ------------------------------------------------------------ profiling
const char *const kStageNames[ST_COUNT] = {"fft_x_fwd", "fft_y_fwd", "fft_z_fwd", "gather",
                                           "permute_out", "permute_in", "grid_zero", "spread",
                                           "fft_z_adj", "fft_y_adj", "fft_x_adj"};

static cudaEvent_t pool_get(Profiler &pr)
{
    if (!pr.pool.empty()) {
        cudaEvent_t e = pr.pool.back();
        pr.pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

StageTimer::StageTimer(nufft3d_plan *p_, int stage_, int launches_, cudaStream_t s_)
    : p(p_), stage(stage_), launches(launches_), s(s_)
{
    if (!p->prof.on) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    a = pool_get(p->prof);
    if (a) cudaEventRecord(a, s);
}

StageTimer::~StageTimer()
{
    if (!a) return;
    cudaEvent_t b = pool_get(p->prof);
    if (!b) return;
    cudaEventRecord(b, s);
    p->prof.pending.push_back({stage, launches, a, b});
}

int profile_resolve(nufft3d_plan *p)
{
    Profiler &pr = p->prof;
    for (auto &r : pr.pending) {
        NUFFT_CUDA_TRY(cudaEventSynchronize(r.b));
        float ms = 0;
        NUFFT_CUDA_TRY(cudaEventElapsedTime(&ms, r.a, r.b));
        pr.ms[r.stage] += ms;
        pr.launches[r.stage] += r.launches;
        pr.calls[r.stage] += 1;
        pr.pool.push_back(r.a);
        pr.pool.push_back(r.b);
    }
    pr.pending.clear();
    return NUFFT3D_SUCCESS;
}

void profile_release(nufft3d_plan *p)
{
    Profiler &pr = p->prof;
    for (auto &r : pr.pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    pr.pending.clear();
    for (auto e : pr.pool) cudaEventDestroy(e);
    pr.pool.clear();
}

int coil_passes(const nufft3d_plan *p, int nc)
{
    int n = 0;
    for (int c0 = 0; c0 < nc; c0 += p->coils_per_pass) ++n;
    return n;
}

// image -> grid G (fft3_pad of U.*x)
static int to_grid(nufft3d_plan *p, const float2 *x, int nc, cudaStream_t s)
{
    Scratch &S = p->scratch;
    {
        StageTimer t(p, ST_FFT_X_FWD, 1, s);
        NUFFT_TRY(launch_fx(p, x, S.B1, nc, s));
    }
    {
        StageTimer t(p, ST_FFT_Y_FWD, 1, s);
        NUFFT_TRY(launch_fy(p, S.B1, S.B2, nc, s));
    }
    if (!p->geom.is2d) {
        StageTimer t(p, ST_FFT_Z_FWD, 1, s);
        NUFFT_TRY(launch_fz(p, S.B2, S.G, nc, s));
    }
    return NUFFT3D_SUCCESS;
}

// grid G -> image (ifft3_crop, .*U, *scale, + add_coef*addend)
static int from_grid(nufft3d_plan *p, float2 *x, int nc, float scale, const float2 *addend,
                     float add_coef, cudaStream_t s)
{
    Scratch &S = p->scratch;
    if (!p->geom.is2d) {
        StageTimer t(p, ST_FFT_Z_ADJ, 1, s);
        NUFFT_TRY(launch_iz(p, S.G, S.B2, nc, s));
    }
    {
        StageTimer t(p, ST_FFT_Y_ADJ, 1, s);
        NUFFT_TRY(launch_iy(p, S.B2, S.B1, nc, s));
    }
    {
        StageTimer t(p, ST_FFT_X_ADJ, 1, s);
        NUFFT_TRY(launch_ix(p, S.B1, x, nc, scale, addend, add_coef, s));
    }
    return NUFFT3D_SUCCESS;
}

static int gather_timed(nufft3d_plan *p, int nc, float scale, const float *ws, cudaStream_t s)
{
    StageTimer t(p, ST_GATHER, coil_passes(p, nc), s);
    return launch_gather(p, p->scratch.G, p->scratch.ks, nc, scale, ws, s);
}

static int spread_timed(nufft3d_plan *p, int nc, cudaStream_t s)
{
    {
        StageTimer t(p, ST_GRID_ZERO, 0, s);
        NUFFT_CUDA_TRY(cudaMemsetAsync(p->scratch.G, 0, grid_bytes(p, nc), s));
    }
    StageTimer t(p, ST_SPREAD, coil_passes(p, nc), s);
    return launch_spread(p, p->scratch.ks, p->scratch.G, nc, s);
}

int op_forward(nufft3d_plan *p, const float2 *x, float2 *k, int nc, cudaStream_t s)
{
    NUFFT_TRY(ensure_scratch(p, nc));
    if (p->nnz == 0) {
        NUFFT_CUDA_TRY(cudaMemsetAsync(k, 0, (size_t)p->M * nc * sizeof(float2), s));
        return NUFFT3D_SUCCESS;
    }
    NUFFT_TRY(to_grid(p, x, nc, s));
    NUFFT_TRY(gather_timed(p, nc, (float)(1.0 / std::sqrt((double)p->nnz)), nullptr, s));
    StageTimer t(p, ST_PERMUTE_OUT, 1, s);
    NUFFT_TRY(launch_permute_out(p, p->scratch.ks, k, nc, 1.f, s));
    return NUFFT3D_SUCCESS;
}

int op_adjoint_weighted(nufft3d_plan *p, const float2 *k, float2 *x, int nc, const float *wsorted,
                        cudaStream_t s)
{
    NUFFT_TRY(ensure_scratch(p, nc));
    if (p->nnz == 0) {
        NUFFT_CUDA_TRY(cudaMemsetAsync(x, 0, img_elems(p) * nc * sizeof(float2), s));
        return NUFFT3D_SUCCESS;
    }
    {
        StageTimer t(p, ST_PERMUTE_IN, 1, s);
        NUFFT_TRY(launch_permute_in(p, k, p->scratch.ks, nc, wsorted, s));
    }
    NUFFT_TRY(spread_timed(p, nc, s));
    NUFFT_TRY(from_grid(p, x, nc, (float)(1.0 / std::sqrt((double)p->nnz)), nullptr, 0.f, s));
    return NUFFT3D_SUCCESS;
}

int op_adjoint(nufft3d_plan *p, const float2 *k, float2 *x, int nc, cudaStream_t s)
{
    return op_adjoint_weighted(p, k, x, nc, nullptr, s);
}

int op_normal(nufft3d_plan *p, const float2 *x, float2 *y, int nc, double damp,
              const float *wsorted, cudaStream_t s)
{
    NUFFT_TRY(ensure_scratch(p, nc));
    const float d2 = (float)(damp * damp);
    if (p->nnz == 0) {
        // y = damp^2 x
        NUFFT_CUDA_TRY(cudaMemsetAsync(p->scratch.G, 0, grid_bytes(p, nc), s));
        NUFFT_TRY(from_grid(p, y, nc, 0.f, x, d2, s));
        return NUFFT3D_SUCCESS;
    }
    NUFFT_TRY(to_grid(p, x, nc, s));
    NUFFT_TRY(gather_timed(p, nc, (float)(1.0 / (double)p->nnz), wsorted ? wsorted : p->d, s));
    NUFFT_TRY(spread_timed(p, nc, s));
    NUFFT_TRY(from_grid(p, y, nc, 1.f, x, d2, s));
    return NUFFT3D_SUCCESS;
}

// ------------------------------------------------------------- density
__global__ void k_fill(float *a, int64_t n, float v)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

__global__ void k_real_to_complex(const float *__restrict__ a, float2 *__restrict__ b, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = make_float2(a[i], 0.f);
}

// density.m:11-13: d = d ./ max(H*H'*d, eps)
__global__ void k_density_update(float *__restrict__ d, const float2 *__restrict__ hhd, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = d[i] / fmaxf(hhd[i].x, 2.220446049250313e-16f);
}

__global__ void k_sum(const float *__restrict__ a, int64_t n, double *__restrict__ out)
{
    double acc = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc += a[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[blockIdx.x] = acc;
    }
}

__global__ void k_factor(double *__restrict__ parts, int nparts, double num)
{
    double s = 0;
    for (int k = 0; k < nparts; ++k) s += parts[k];
    parts[nparts] = num / s;
}

__global__ void k_scale_by(float *__restrict__ a, int64_t n, const double *__restrict__ factor)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (float)(a[i] * *factor);
}

int refresh_density_orig(nufft3d_plan *p, cudaStream_t s);

int run_density(nufft3d_plan *p, int maxit, cudaStream_t s)
{
    const int64_t n = p->nnz;
    if (n == 0) return refresh_density_orig(p, s);
    NUFFT_TRY(ensure_scratch(p, 1));
    const int th = 256;
    const unsigned nb = (unsigned)((n + th - 1) / th);
    k_fill<<<nb, th, 0, s>>>(p->d, n, 1.f); // density.m:8 (d = ok)
    NUFFT_CUDA_TRY(cudaGetLastError());
    for (int it = 0; it < maxit; ++it) {
        k_real_to_complex<<<nb, th, 0, s>>>(p->d, p->scratch.ks, n);
        NUFFT_CUDA_TRY(cudaGetLastError());
        NUFFT_CUDA_TRY(cudaMemsetAsync(p->scratch.G, 0, grid_bytes(p, 1), s));
        NUFFT_TRY(launch_spread(p, p->scratch.ks, p->scratch.G, 1, s));
        NUFFT_TRY(launch_gather(p, p->scratch.G, p->scratch.ks, 1, 1.f, nullptr, s));
        k_density_update<<<nb, th, 0, s>>>(p->d, p->scratch.ks, n);
        NUFFT_CUDA_TRY(cudaGetLastError());
    }
    // density.m:42: d = d / (sum(d)/nnz)
    const int nparts = 304;
    double *parts = nullptr;
    NUFFT_DEVICE_LOCK;
    NUFFT_CUDA_TRY(cudaMalloc(&parts, sizeof(double) * (nparts + 1)));
    k_sum<<<nparts, th, 0, s>>>(p->d, n, parts);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_factor<<<1, 1, 0, s>>>(parts, nparts, (double)n);
        k_scale_by<<<nb, th, 0, s>>>(p->d, n, parts + nparts);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(parts);
    if (e != cudaSuccess) return fail(NUFFT3D_ERR_CUDA, std::string("density: ") + cudaGetErrorString(e));
    return refresh_density_orig(p, s);
}

} // namespace nufft3d

using namespace nufft3d;

static int check_common(nufft3d_plan *p, const void *a, const void *b, int nc)
{
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    if (!a || !b) return fail(NUFFT3D_ERR_ARG, "NULL data pointer");
    if (nc < 1) return fail(NUFFT3D_ERR_ARG, "number of coils must be >= 1");
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_forward(nufft3d_plan *p, const float *x, float *k, int nc, void *stream)
{
    clear_error();
    NUFFT_TRY(check_common(p, x, k, nc));
    DevGuard g(p->device);
    return op_forward(p, (const float2 *)x, (float2 *)k, nc, (cudaStream_t)stream);
}

extern "C" int nufft3d_adjoint(nufft3d_plan *p, const float *k, float *x, int nc, void *stream)
{
    clear_error();
    NUFFT_TRY(check_common(p, k, x, nc));
    DevGuard g(p->device);
    return op_adjoint(p, (const float2 *)k, (float2 *)x, nc, (cudaStream_t)stream);
}

extern "C" int nufft3d_normal(nufft3d_plan *p, const float *x, float *y, int nc, double damp,
                              const float *W, void *stream)
{
    clear_error();
    NUFFT_TRY(check_common(p, x, y, nc));
    if (!std::isfinite(damp) || damp < 0) return fail(NUFFT3D_ERR_ARG, "damp must be finite and nonnegative");
    DevGuard g(p->device);
    const float *ws = nullptr;
    NUFFT_TRY(prepare_weights(p, W, &ws, (cudaStream_t)stream));
    return op_normal(p, (const float2 *)x, (float2 *)y, nc, damp, ws, (cudaStream_t)stream);
}

static int stage_alloc(nufft3d_plan *p, size_t in_bytes, size_t out_bytes)
{
    HostStage &h = p->stage;
    if (h.bytes_in >= in_bytes && h.bytes_out >= out_bytes) return NUFFT3D_SUCCESS;
    NUFFT_DEVICE_LOCK;
    if (h.bytes_in < in_bytes) {
        if (h.in) cudaFree(h.in);
        h.in = nullptr;
        h.bytes_in = 0;
        NUFFT_CUDA_TRY(cudaMalloc(&h.in, in_bytes));
        h.bytes_in = in_bytes;
    }
    if (h.bytes_out < out_bytes) {
        if (h.out) cudaFree(h.out);
        h.out = nullptr;
        h.bytes_out = 0;
        NUFFT_CUDA_TRY(cudaMalloc(&h.out, out_bytes));
        h.bytes_out = out_bytes;
    }
    return NUFFT3D_SUCCESS;
}

// Device address of a page-locked host buffer (cudaHostAlloc or
// cudaHostRegister), through which kernels read or write it directly over the
// host link; nullptr for pageable memory, which goes through a device staging
// buffer and cudaMemcpyAsync instead.
static void *mapped_device_ptr(const void *h)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Host-pointer operator: page-locked buffers are used in place by the first
// and last kernels of the chain (the input read once by the x pass or the
// permute, the output written once), so the transfers ride inside those
// kernels instead of separate copies (host_copy = 0), or are moved by the
// copy engines through device staging buffers (host_copy = 1); pageable
// buffers are always staged.
template <typename Op>
static int host_call(nufft3d_plan *p, const void *in, void *out, size_t bi, size_t bo, Op &&op)
{
    cudaStream_t s = p->own_stream;
    const void *din = p->host_copy ? nullptr : mapped_device_ptr(in);
    void *dout = p->host_copy ? nullptr : mapped_device_ptr(out);
    NUFFT_TRY(stage_alloc(p, din ? 0 : bi, dout ? 0 : bo));
    if (!din) {
        NUFFT_CUDA_TRY(cudaMemcpyAsync(p->stage.in, in, bi, cudaMemcpyHostToDevice, s));
        din = p->stage.in;
    }
    NUFFT_TRY(op((const float2 *)din, dout ? (float2 *)dout : (float2 *)p->stage.out, s));
    if (!dout) NUFFT_CUDA_TRY(cudaMemcpyAsync(out, p->stage.out, bo, cudaMemcpyDeviceToHost, s));
    NUFFT_TRY(plan_check_status(p, s));
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_forward_host(nufft3d_plan *p, const float *x, float *k, int nc)
{
    clear_error();
    NUFFT_TRY(check_common(p, x, k, nc));
    DevGuard g(p->device);
    const size_t bi = img_elems(p) * nc * sizeof(float2), bo = (size_t)p->M * nc * sizeof(float2);
    return host_call(p, x, k, bi, bo, [&](const float2 *din, float2 *dout, cudaStream_t s) {
        return op_forward(p, din, dout, nc, s);
    });
}

extern "C" int nufft3d_adjoint_host(nufft3d_plan *p, const float *k, float *x, int nc)
{
    clear_error();
    NUFFT_TRY(check_common(p, k, x, nc));
    DevGuard g(p->device);
    const size_t bi = (size_t)p->M * nc * sizeof(float2), bo = img_elems(p) * nc * sizeof(float2);
    return host_call(p, k, x, bi, bo, [&](const float2 *din, float2 *dout, cudaStream_t s) {
        return op_adjoint(p, din, dout, nc, s);
    });
}

extern "C" int nufft3d_density(nufft3d_plan *p, int maxit)
{
    clear_error();
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    if (maxit < 0) return fail(NUFFT3D_ERR_ARG, "maxit must be nonnegative");
    DevGuard g(p->device);
    NUFFT_TRY(run_density(p, maxit, p->own_stream));
    NUFFT_TRY(plan_check_status(p, p->own_stream));
    return NUFFT3D_SUCCESS;
}

namespace nufft3d {
__global__ void k_kernel_eval(const float *__restrict__ d2, float *__restrict__ w, int64_t n, KBParams kb)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w[i] = kb_weight(fminf(d2[i], kb.half2), kb);
}
} // namespace nufft3d

extern "C" int nufft3d_kernel_eval(const nufft3d_plan *p, const float *d2, float *w, int64_t n, void *stream)
{
    clear_error();
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    if (n < 0 || (n > 0 && (!d2 || !w))) return fail(NUFFT3D_ERR_ARG, "NULL data pointer or negative count");
    if (n == 0) return NUFFT3D_SUCCESS;
    DevGuard g(p->device);
    k_kernel_eval<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d2, w, n, p->kb);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_check_status(nufft3d_plan *p, void *stream)
{
    clear_error();
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    DevGuard g(p->device);
    return plan_check_status(p, (cudaStream_t)stream);
}

extern "C" int nufft3d_profile(nufft3d_plan *p, int enable)
{
    clear_error();
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    DevGuard g(p->device);
    NUFFT_TRY(profile_resolve(p));
    Profiler &pr = p->prof;
    for (int i = 0; i < ST_COUNT; ++i) {
        pr.ms[i] = 0;
        pr.launches[i] = 0;
        pr.calls[i] = 0;
    }
    pr.on = enable != 0;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_profile_read(nufft3d_plan *p, char *buf, int cap)
{
    clear_error();
    if (!p || !buf || cap <= 0) return fail(NUFFT3D_ERR_ARG, "NULL argument");
    DevGuard g(p->device);
    NUFFT_TRY(profile_resolve(p));
    std::string out = "{";
    const Profiler &pr = p->prof;
    bool first = true;
    for (int i = 0; i < ST_COUNT; ++i) {
        if (!pr.calls[i]) continue;
        char tmp[256];
        std::snprintf(tmp, sizeof tmp, "%s\"%s\": {\"calls\": %lld, \"launches\": %lld, \"ms\": %.6f}",
                      first ? "" : ", ", kStageNames[i], pr.calls[i], pr.launches[i], pr.ms[i]);
        out += tmp;
        first = false;
    }
    out += "}";
    if ((int)out.size() + 1 > cap) return fail(NUFFT3D_ERR_SIZE, "profile buffer too small");
    std::memcpy(buf, out.c_str(), out.size() + 1);
    return NUFFT3D_SUCCESS;
}
