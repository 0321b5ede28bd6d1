// Interpolation gather (fNUFT) and gridding spread (aNUFT) without a stored H.
//
// The reference builds a sparse matrix H [M x prod(K)] (nufft_3d.m:153-212)
// and multiplies by H (spmv, nufft_3d.m:259-271) and H' (spmv_t,
// nufft_3d.m:274-282) through cuSPARSE.  Here the in-bounds samples are
// sorted by oversampled-grid tile at plan time; one block handles one tile
// piece: it stages the tile plus a halo of R = ceil(J/2) points in shared
// memory, evaluates the Kaiser-Bessel weights of kernel.m in registers and
//   gather: reads the staged grid and writes each sample's value;
//   spread: accumulates into the staged tile (shared-memory atomics) and adds
//           the tile to the grid with vector atomics (halos overlap).
// The neighbour set is the reference's: offsets -R..R around round(u*om),
// kept when 4*dist2 <= J^2 (radial) or per axis (separable).
//
// Sample record (float4): (fx, fy, fz, packed) with f = u*om - round(u*om)
// computed in double at plan time and packed = lx | ly<<8 | lz<<16 the
// sample's rounded position inside the padded tile.
// Grid layout [K3][K2][K1][nc]; sorted sample data layout [nnz][nc].
#include <cuda_runtime.h>

#include "internal.h"

namespace nufft3d {

constexpr int kInterpThreads = 256;

__device__ __forceinline__ int wrap_idx(int x, int K)
{
    x %= K;
    return x < 0 ? x + K : x;
}

// Visit the taps of one sample: BODY sees `w` (weight) and `tp` (offset of
// the tap in the padded tile, in grid points).
template <int R, bool RADIAL, int RZ, typename F>
__device__ __forceinline__ void for_taps(const float4 rec, int Px, int Py, const KBParams &kb,
                                         F &&body)
{
    const int packed = __float_as_int(rec.w);
    const int lx0 = packed & 0xFF, ly0 = (packed >> 8) & 0xFF, lz0 = (packed >> 16) & 0xFF;
    const float h2 = kb.half2;
    float wxs[2 * R + 1];
    if (!RADIAL) {
#pragma unroll
        for (int dx = -R; dx <= R; ++dx) {
            const float ex = dx - rec.x;
            const float ex2 = ex * ex;
            wxs[dx + R] = ex2 <= h2 ? kb_weight(ex2, kb) : 0.f;
        }
    }
#pragma unroll 1
    for (int dz = -RZ; dz <= RZ; ++dz) {
        const float ez = dz - rec.z;
        const float ez2 = ez * ez;
        if (ez2 > h2) continue;
        const float wz = RADIAL ? 1.f : kb_weight(ez2, kb);
#pragma unroll 1
        for (int dy = -R; dy <= R; ++dy) {
            const float ey = dy - rec.y;
            const float ey2 = ey * ey;
            const float eyz2 = RADIAL ? ez2 + ey2 : ey2;
            if (eyz2 > h2) continue;
            const float wyz = RADIAL ? 1.f : wz * kb_weight(ey2, kb);
            const int rowoff = ((lz0 + dz) * Py + (ly0 + dy)) * Px + lx0;
#pragma unroll
            for (int dx = -R; dx <= R; ++dx) {
                const float ex = dx - rec.x;
                if (RADIAL) {
                    const float d2 = fmaf(ex, ex, eyz2);
                    if (d2 <= h2) body(kb_weight(d2, kb), rowoff + dx);
                } else {
                    if (ex * ex <= h2) body(wyz * wxs[dx + R], rowoff + dx);
                }
            }
        }
    }
}

template <int CB>
__device__ __forceinline__ void stage_tile(float2 *tile, const float2 *__restrict__ G, int nc,
                                           int c0, int cb, const Geom &g, int ox, int oy, int oz)
{
    const int Px = g.P[0], Py = g.P[1], Pz = g.P[2];
    const int n = Px * Py * Pz * CB;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int c = t % CB;
        const int pt = t / CB;
        const int lx = pt % Px;
        const int r = pt / Px;
        const int ly = r % Py;
        const int lz = r / Py;
        float2 v = make_float2(0.f, 0.f);
        if (c < cb) {
            const int gx = wrap_idx(ox + lx, g.K[0]);
            const int gy = wrap_idx(oy + ly, g.K[1]);
            const int gz = wrap_idx(oz + lz, g.K[2]);
            v = G[(((size_t)gz * g.K[1] + gy) * g.K[0] + gx) * nc + c0 + c];
        }
        tile[t] = v;
    }
}

template <int CB, int R, bool RADIAL, int RZ>
__global__ void __launch_bounds__(kInterpThreads)
k_gather(const float2 *__restrict__ G, float2 *__restrict__ ks, int nc, int c0,
         const float4 *__restrict__ samples, const int4 *__restrict__ blocks, Geom g,
         KBParams kb, float scale, const float *__restrict__ wsample)
{
    extern __shared__ float2 tile[];
    const int4 bi = blocks[blockIdx.x];
    const int tid = bi.x;
    const int tx = tid % g.nt[0];
    const int ty = (tid / g.nt[0]) % g.nt[1];
    const int tz = tid / (g.nt[0] * g.nt[1]);
    const int cb = min(CB, nc - c0);
    stage_tile<CB>(tile, G, nc, c0, cb, g, tx * g.T[0] - g.Ra[0], ty * g.T[1] - g.Ra[1],
                   tz * g.T[2] - g.Ra[2]);
    __syncthreads();
    const int Px = g.P[0], Py = g.P[1];
    for (int s = bi.y + threadIdx.x; s < bi.y + bi.z; s += blockDim.x) {
        const float4 rec = __ldg(&samples[s]);
        float2 acc[CB];
#pragma unroll
        for (int c = 0; c < CB; ++c) acc[c] = make_float2(0.f, 0.f);
        for_taps<R, RADIAL, RZ>(rec, Px, Py, kb, [&](float w, int off) {
            const float2 *tp = tile + (size_t)off * CB;
#pragma unroll
            for (int c = 0; c < CB; ++c) {
                const float2 v = tp[c];
                acc[c].x = fmaf(w, v.x, acc[c].x);
                acc[c].y = fmaf(w, v.y, acc[c].y);
            }
        });
        const float sc = wsample ? scale * __ldg(&wsample[s]) : scale;
        float2 *o = ks + (size_t)s * nc + c0;
#pragma unroll
        for (int c = 0; c < CB; ++c)
            if (c < cb) o[c] = make_float2(acc[c].x * sc, acc[c].y * sc);
    }
}

template <int CB, int R, bool RADIAL, int RZ>
__global__ void __launch_bounds__(kInterpThreads)
k_spread(const float2 *__restrict__ ks, float2 *__restrict__ G, int nc, int c0,
         const float4 *__restrict__ samples, const int4 *__restrict__ blocks, Geom g,
         KBParams kb)
{
    extern __shared__ float2 tile[];
    const int4 bi = blocks[blockIdx.x];
    const int tid = bi.x;
    const int tx = tid % g.nt[0];
    const int ty = (tid / g.nt[0]) % g.nt[1];
    const int tz = tid / (g.nt[0] * g.nt[1]);
    const int cb = min(CB, nc - c0);
    const int Px = g.P[0], Py = g.P[1], Pz = g.P[2];
    const int n = Px * Py * Pz * CB;
    for (int t = threadIdx.x; t < n; t += blockDim.x) tile[t] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int s = bi.y + threadIdx.x; s < bi.y + bi.z; s += blockDim.x) {
        const float4 rec = __ldg(&samples[s]);
        float2 yv[CB];
        const float2 *src = ks + (size_t)s * nc + c0;
#pragma unroll
        for (int c = 0; c < CB; ++c) yv[c] = c < cb ? src[c] : make_float2(0.f, 0.f);
        for_taps<R, RADIAL, RZ>(rec, Px, Py, kb, [&](float w, int off) {
            float2 *tp = tile + (size_t)off * CB;
#pragma unroll
            for (int c = 0; c < CB; ++c) {
                atomicAdd(&tp[c].x, w * yv[c].x);
                atomicAdd(&tp[c].y, w * yv[c].y);
            }
        });
    }
    __syncthreads();
    const int ox = tx * g.T[0] - g.Ra[0], oy = ty * g.T[1] - g.Ra[1], oz = tz * g.T[2] - g.Ra[2];
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int c = t % CB;
        if (c >= cb) continue;
        const float2 v = tile[t];
        if (v.x == 0.f && v.y == 0.f) continue;
        const int pt = t / CB;
        const int lx = pt % Px;
        const int r = pt / Px;
        const int ly = r % Py;
        const int lz = r / Py;
        const int gx = wrap_idx(ox + lx, g.K[0]);
        const int gy = wrap_idx(oy + ly, g.K[1]);
        const int gz = wrap_idx(oz + lz, g.K[2]);
        atomicAdd(&G[(((size_t)gz * g.K[1] + gy) * g.K[0] + gx) * nc + c0 + c], v);
    }
}

__global__ void k_permute_out(const float2 *__restrict__ ks, float2 *__restrict__ k,
                              const int32_t *__restrict__ inv, int64_t M, int nc, float scale)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const int s = inv[m];
    for (int c = 0; c < nc; ++c) {
        float2 v = make_float2(0.f, 0.f);
        if (s >= 0) {
            v = ks[(size_t)s * nc + c];
            v.x *= scale;
            v.y *= scale;
        }
        k[m + M * c] = v;
    }
}

__global__ void k_permute_in(const float2 *__restrict__ k, float2 *__restrict__ ks,
                             const int32_t *__restrict__ inv, int64_t M, int nc,
                             const float *__restrict__ wsorted)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const int s = inv[m];
    if (s < 0) return;
    const float w = wsorted ? wsorted[s] : 1.f;
    for (int c = 0; c < nc; ++c) {
        float2 v = k[m + M * c];
        ks[(size_t)s * nc + c] = make_float2(v.x * w, v.y * w);
    }
}

// ---------------------------------------------------------------- host
size_t smem_interp_bytes(const Geom &g, int cb)
{
    return (size_t)g.P[0] * g.P[1] * g.P[2] * cb * sizeof(float2);
}

template <int CB, int R, bool RADIAL, int RZ>
static int gather_t(nufft3d_plan *p, const float2 *G, float2 *ks, int nc, int c0, float scale,
                    const float *ws, cudaStream_t s)
{
    const size_t smem = smem_interp_bytes(p->geom, CB);
    k_gather<CB, R, RADIAL, RZ><<<(unsigned)p->n_blocks, kInterpThreads, smem, s>>>(
        G, ks, nc, c0, p->samples, p->blocks, p->geom, p->kb, scale, ws);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

template <int CB, int R, bool RADIAL, int RZ>
static int spread_t(nufft3d_plan *p, const float2 *ks, float2 *G, int nc, int c0, cudaStream_t s)
{
    const size_t smem = smem_interp_bytes(p->geom, CB);
    k_spread<CB, R, RADIAL, RZ><<<(unsigned)p->n_blocks, kInterpThreads, smem, s>>>(
        ks, G, nc, c0, p->samples, p->blocks, p->geom, p->kb);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

// Dispatch over (coils per pass, R, radial, 2D).
template <bool GATHER, int CB, int R>
static int dispatch_rz(nufft3d_plan *p, const float2 *in, float2 *out, int nc, int c0, float scale,
                       const float *ws, cudaStream_t s)
{
    const bool rad = p->geom.radial != 0;
    const bool flat = p->geom.is2d != 0;
    if (GATHER) {
        if (rad) return flat ? gather_t<CB, R, true, 0>(p, in, out, nc, c0, scale, ws, s)
                             : gather_t<CB, R, true, R>(p, in, out, nc, c0, scale, ws, s);
        return flat ? gather_t<CB, R, false, 0>(p, in, out, nc, c0, scale, ws, s)
                    : gather_t<CB, R, false, R>(p, in, out, nc, c0, scale, ws, s);
    }
    if (rad) return flat ? spread_t<CB, R, true, 0>(p, in, out, nc, c0, s)
                         : spread_t<CB, R, true, R>(p, in, out, nc, c0, s);
    return flat ? spread_t<CB, R, false, 0>(p, in, out, nc, c0, s)
                : spread_t<CB, R, false, R>(p, in, out, nc, c0, s);
}

template <bool GATHER, int CB>
static int dispatch_r(nufft3d_plan *p, const float2 *in, float2 *out, int nc, int c0, float scale,
                      const float *ws, cudaStream_t s)
{
    switch (p->geom.R) {
    case 1: return dispatch_rz<GATHER, CB, 1>(p, in, out, nc, c0, scale, ws, s);
    case 2: return dispatch_rz<GATHER, CB, 2>(p, in, out, nc, c0, scale, ws, s);
    case 3: return dispatch_rz<GATHER, CB, 3>(p, in, out, nc, c0, scale, ws, s);
    case 4: return dispatch_rz<GATHER, CB, 4>(p, in, out, nc, c0, scale, ws, s);
    default: return fail(NUFFT3D_ERR_UNSUPPORTED, "kernel half-width ceil(J/2) must be 1..4");
    }
}

template <bool GATHER>
static int interp(nufft3d_plan *p, const float2 *in, float2 *out, int nc, float scale,
                  const float *ws, cudaStream_t s)
{
    if (p->n_blocks == 0) return NUFFT3D_SUCCESS;
    const int cmax = p->coils_per_pass;
    for (int c0 = 0; c0 < nc; c0 += cmax) {
        const int rem = nc - c0;
        int cb = 1;
        while (cb < rem && cb < cmax) cb *= 2;
        int st;
        switch (cb) {
        case 1: st = dispatch_r<GATHER, 1>(p, in, out, nc, c0, scale, ws, s); break;
        case 2: st = dispatch_r<GATHER, 2>(p, in, out, nc, c0, scale, ws, s); break;
        case 4: st = dispatch_r<GATHER, 4>(p, in, out, nc, c0, scale, ws, s); break;
        default: st = dispatch_r<GATHER, 8>(p, in, out, nc, c0, scale, ws, s); break;
        }
        if (st != NUFFT3D_SUCCESS) return st;
        if (cb > rem) break;
    }
    return NUFFT3D_SUCCESS;
}

int launch_gather(nufft3d_plan *p, const float2 *G, float2 *ks, int nc, float scale,
                  const float *wsample, cudaStream_t s)
{
    return interp<true>(p, G, ks, nc, scale, wsample, s);
}

int launch_spread(nufft3d_plan *p, const float2 *ks, float2 *G, int nc, cudaStream_t s)
{
    return interp<false>(p, ks, G, nc, 1.f, nullptr, s);
}

int launch_permute_out(nufft3d_plan *p, const float2 *ks, float2 *k, int nc, float scale,
                       cudaStream_t s)
{
    if (p->M == 0) return NUFFT3D_SUCCESS;
    const int th = 256;
    const int64_t nb = (p->M + th - 1) / th;
    k_permute_out<<<(unsigned)nb, th, 0, s>>>(ks, k, p->inv, p->M, nc, scale);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

int launch_permute_in(nufft3d_plan *p, const float2 *k, float2 *ks, int nc,
                      const float *wsorted, cudaStream_t s)
{
    if (p->M == 0) return NUFFT3D_SUCCESS;
    const int th = 256;
    const int64_t nb = (p->M + th - 1) / th;
    k_permute_in<<<(unsigned)nb, th, 0, s>>>(k, ks, p->inv, p->M, nc, wsorted);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

template <bool GATHER, int CB, int R>
static int cfg_rz()
{
    const int mx = 227 * 1024;
    if (GATHER) {
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_gather<CB, R, true, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_gather<CB, R, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_gather<CB, R, false, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_gather<CB, R, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    } else {
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_spread<CB, R, true, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_spread<CB, R, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_spread<CB, R, false, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_spread<CB, R, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    }
    return NUFFT3D_SUCCESS;
}

template <bool GATHER, int CB>
static int cfg_r()
{
    NUFFT_TRY((cfg_rz<GATHER, CB, 1>()));
    NUFFT_TRY((cfg_rz<GATHER, CB, 2>()));
    NUFFT_TRY((cfg_rz<GATHER, CB, 3>()));
    NUFFT_TRY((cfg_rz<GATHER, CB, 4>()));
    return NUFFT3D_SUCCESS;
}

int configure_interp_kernels()
{
    NUFFT_TRY((cfg_r<true, 1>()));
    NUFFT_TRY((cfg_r<true, 2>()));
    NUFFT_TRY((cfg_r<true, 4>()));
    NUFFT_TRY((cfg_r<true, 8>()));
    NUFFT_TRY((cfg_r<false, 1>()));
    NUFFT_TRY((cfg_r<false, 2>()));
    NUFFT_TRY((cfg_r<false, 4>()));
    NUFFT_TRY((cfg_r<false, 8>()));
    return NUFFT3D_SUCCESS;
}

} // namespace nufft3d
