// Interpolation gather (fNUFT) and gridding spread (aNUFT) without a stored H.
//
// The reference builds a sparse matrix H [M x prod(K)] (nufft_3d.m:153-212)
// and multiplies by H (spmv, nufft_3d.m:259-271) and H' (spmv_t,
// nufft_3d.m:274-282) through cuSPARSE.  Here the in-bounds samples are
// sorted by oversampled-grid tile at plan time and the tiles split into
// pieces; persistent blocks (one per SM) take pieces from a work counter,
// hold the tile plus a halo of R = ceil(J/2) points in shared memory,
// evaluate the Kaiser-Bessel weights of kernel.m in registers and
//   gather: read the staged grid (one bulk tensor copy per interior tile) and
//           write each sample's value;
//   spread: accumulate into the tile (32-bit fixed-point shared-memory
//           reductions) and add the tile to the grid with vector atomics
//           (halos overlap).
// The neighbour set is the reference's: offsets -R..R around round(u*om),
// kept when 4*dist2 <= J^2 (radial) or per axis (separable).
//
// Sample record (float4): (fx, fy, fz, packed) with f = u*om - round(u*om)
// computed in double at plan time and packed = lx | ly<<8 | lz<<16 the
// sample's rounded position inside the padded tile.
// Grid layout [K3][K2][K1][nc]; sorted sample data layout [nnz][nc].
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "internal.h"

namespace nufft3d {

constexpr int kInterpThreads = 1024;
constexpr int kGroup = 8;                 // lanes sharing one sample

// Tile plane stride (points per coil plane) as a compile-time constant per
// half-width R: tiles are 8^3 (3-D) or 32x32x1 (2-D) plus the halo, and the
// stride covers both, so each coil plane is an immediate offset.
template <int R>
struct Plane {
    static constexpr int P3 = (8 + 2 * R) * (8 + 2 * R) * (8 + 2 * R);
    static constexpr int P2 = (32 + 2 * R) * (32 + 2 * R);
    static constexpr int PS = P3 > P2 ? P3 : P2;
};

__device__ __forceinline__ int wrap_idx(int x, int K)
{
    x %= K;
    return x < 0 ? x + K : x;
}

// Candidate taps (struct Cand, built at plan time): a sample's fractional
// offset f from its rounded grid point is reflected into the octant
// |f| in [0, 1/2]^3, which is split into 8 sub-cubes (|f_a| below or above
// 1/4 per axis); each sub-cube has its own list of offsets d' that can fall
// inside the support.  A sample uses the tap s*d' (s = sign(f) per axis) and
// tests (d' - |f|)^2 per axis -- the same value as (s*d' - f)^2.
//
// Per-block copy in shared memory: the 8 list starts and lengths, then every
// offset as floats (dx', dy', dz', 0).  The tile offset of a tap is computed
// from the sample's signed strides, so no per-octant table is needed.
struct CandSmem {
    const int *sc;  // [24]: start[8], cnt[8], core[8]
    float4 *f;      // [n]
};

// Candidate tables at the start of the dynamic shared memory; returns the
// first free 16-byte word after them.
__device__ __forceinline__ float4 *carve_cand(const Cand &cd, CandSmem &cs, float4 *smem4)
{
    cs.sc = reinterpret_cast<const int *>(smem4);
    cs.f = smem4 + 6;
    return smem4 + 6 + cd.n;
}

__device__ __forceinline__ void build_cand(const Cand &cd, CandSmem cs)
{
    int *sc = const_cast<int *>(cs.sc);
    if (threadIdx.x < 8) {
        sc[threadIdx.x] = cd.start[threadIdx.x];
        sc[8 + threadIdx.x] = cd.cnt[threadIdx.x];
        sc[16 + threadIdx.x] = cd.core[threadIdx.x];
    }
    for (int i = threadIdx.x; i < cd.n; i += blockDim.x) {
        const int code = cd.list[i];
        const int dx = (code & 15) - 8, dy = ((code >> 4) & 15) - 8, dz = ((code >> 8) & 15) - 8;
        cs.f[i] = make_float4((float)dx, (float)dy, (float)dz, 0.f);
    }
}

size_t cand_smem_bytes(int n) { return (size_t)(n + 6) * sizeof(float4); }

// The spread's copy of the lists, for packed evaluation of two candidates per
// lane: list q in blocks of 64, entry (b, l) holding its candidates 64b + l
// ("a") and 64b + 32 + l ("b") as two words of bytes (dx'+8, dy'+8, dz'+8, 0),
// one 8-byte shared load per lane and block (the spread is bound by
// shared-memory traffic, not by issue).  Slots past the list's end hold byte
// 255 per axis, an offset so far away that it never passes a support test.
struct CandPairs {
    const int *sc;  // [16]: first entry of list q, length of list q
    const int2 *pc;
};

constexpr int kFarTapCode = 0x00FFFFFF;

__host__ __device__ __forceinline__ int cand_pair_entries(const int *cnt)
{
    int n = 0;
    for (int q = 0; q < 8; ++q) n += ((cnt[q] + 63) >> 6) * 32;
    return n;
}

size_t cand_pairs_bytes(const Cand &cd)
{
    return (size_t)4 * sizeof(float4) + (((size_t)cand_pair_entries(cd.cnt) * sizeof(int2) + 15) & ~(size_t)15);
}

// Pair tables at the start of the dynamic shared memory; returns the first
// free 16-byte word after them.
__device__ __forceinline__ float4 *carve_pairs(const Cand &cd, CandPairs &cp, float4 *smem4)
{
    const int np = cand_pair_entries(cd.cnt);
    cp.sc = reinterpret_cast<const int *>(smem4);
    cp.pc = reinterpret_cast<const int2 *>(smem4 + 4);
    return smem4 + 4 + (np + 1) / 2;
}

__device__ __forceinline__ void build_pairs(const Cand &cd, const CandPairs &cp)
{
    const int np = cand_pair_entries(cd.cnt);
    if (threadIdx.x == 0) {
        int *sc = const_cast<int *>(cp.sc);
        int st = 0;
        for (int q = 0; q < 8; ++q) {
            sc[q] = st;
            sc[8 + q] = cd.cnt[q];
            st += ((cd.cnt[q] + 63) >> 6) * 32;
        }
    }
    int2 *pc = const_cast<int2 *>(cp.pc);
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
        int q = 0, st = 0;
        for (; q < 7; ++q) {
            const int n = ((cd.cnt[q] + 63) >> 6) * 32;
            if (i < st + n) break;
            st += n;
        }
        const int e = i - st, ia = 64 * (e >> 5) + (e & 31), ib = ia + 32;
        int w[2];
        const int idx[2] = {ia, ib};
        for (int h = 0; h < 2; ++h) {
            // the list's codes are 4 bits per axis with a bias of 8: widen to bytes
            const int code = idx[h] < cd.cnt[q] ? cd.list[cd.start[q] + idx[h]] : -1;
            w[h] = code < 0 ? kFarTapCode : (code & 15) | (((code >> 4) & 15) << 8) | (((code >> 8) & 15) << 16);
        }
        pc[i] = make_int2(w[0], w[1]);
    }
}

// Axis k (byte k) of two pair codes as exact floats d' = byte - 8: the byte
// is placed in the low mantissa bits of 1.5*2^23 and that bias removed.
template <int K>
__device__ __forceinline__ float2 pair_axis(const int2 c)
{
    const float2 m = make_float2(__int_as_float(__byte_perm(c.x, 0x4B400000, 0x7650 + K)),
                                 __int_as_float(__byte_perm(c.y, 0x4B400000, 0x7650 + K)));
    return __fadd2_rn(m, make_float2(-12582920.0f, -12582920.0f));
}

// Per-sample reflected coordinates.
struct SampleGeo {
    float fx, fy, fz;  // |f|
    float sx, sy, sz;  // signed tile strides of the sample's octant: +-1, +-Px, +-Px*Py
    float b;           // tile index of the rounded position + 1.5*2^23 (see tap)
    int lbase, ln;     // the sample's sub-cube candidate list
    int lcore;         // its first lcore candidates are inside the support for any f of the sub-cube
};

// Reads the list starts and lengths from shared memory: call after the
// barrier that follows build_cand.
__device__ __forceinline__ SampleGeo sample_geo(const float4 rec, int Px, int Py, const CandSmem &cs)
{
    SampleGeo g;
    const int packed = __float_as_int(rec.w);
    const int lx0 = packed & 0xFF, ly0 = (packed >> 8) & 0xFF, lz0 = (packed >> 16) & 0xFF;
    g.sx = rec.x < 0.f ? -1.f : 1.f;
    g.sy = rec.y < 0.f ? (float)-Px : (float)Px;
    g.sz = rec.z < 0.f ? (float)(-Px * Py) : (float)(Px * Py);
    g.fx = fabsf(rec.x);
    g.fy = fabsf(rec.y);
    g.fz = fabsf(rec.z);
    g.b = (float)((lz0 * Py + ly0) * Px + lx0) + 12582912.0f;
    const int q = (g.fx >= 0.25f ? 1 : 0) | (g.fy >= 0.25f ? 2 : 0) | (g.fz >= 0.25f ? 4 : 0);
    g.lbase = cs.sc[q];
    g.ln = cs.sc[8 + q];
    g.lcore = cs.sc[16 + q];
    return g;
}

// The same for the pair tables: lbase = the list's first pair entry.
__device__ __forceinline__ SampleGeo sample_geo_pairs(const float4 rec, int Px, int Py, const CandPairs &cp)
{
    SampleGeo g;
    const int packed = __float_as_int(rec.w);
    const int lx0 = packed & 0xFF, ly0 = (packed >> 8) & 0xFF, lz0 = (packed >> 16) & 0xFF;
    g.sx = rec.x < 0.f ? -1.f : 1.f;
    g.sy = rec.y < 0.f ? (float)-Px : (float)Px;
    g.sz = rec.z < 0.f ? (float)(-Px * Py) : (float)(Px * Py);
    g.fx = fabsf(rec.x);
    g.fy = fabsf(rec.y);
    g.fz = fabsf(rec.z);
    g.b = (float)((lz0 * Py + ly0) * Px + lx0) + 12582912.0f;
    const int q = (g.fx >= 0.25f ? 1 : 0) | (g.fy >= 0.25f ? 2 : 0) | (g.fz >= 0.25f ? 4 : 0);
    g.lbase = cp.sc[q];
    g.ln = cp.sc[8 + q];
    g.lcore = 0;
    return g;
}

// Tile offset of the candidate with reflected offset cf: base + s*d' summed
// in floating point on top of 1.5*2^23, where every partial sum is an exact
// integer (|values| < 2^22), read back from the bits.
__device__ __forceinline__ int tap_offset(const float4 cf, const SampleGeo &g)
{
    return __float_as_int(fmaf(cf.z, g.sz, fmaf(cf.y, g.sy, fmaf(cf.x, g.sx, g.b)))) - 0x4B400000;
}

// Weight and tile offset of candidate ci (< g.ln) of the sample's list; false
// outside the kernel support (the neighbour test of nufft_3d.m:183-192).
template <bool RADIAL>
__device__ __forceinline__ bool tap(int ci, const SampleGeo &g, const CandSmem &cs, const KBParams &kb,
                                    float &w, int &off)
{
    const float4 cf = cs.f[g.lbase + ci];
    const float ex = cf.x - g.fx, ey = cf.y - g.fy, ez = cf.z - g.fz;
    const float ex2 = ex * ex, ey2 = ey * ey, ez2 = ez * ez;
    const float h2 = kb.half2;
    if (RADIAL) {
        const float d2 = ez2 + ey2 + ex2;
        if (!(d2 <= h2)) return false;
        w = kb_weight(d2, kb);
    } else {
        if (!(ex2 <= h2 && ey2 <= h2 && ez2 <= h2)) return false;
        w = kb_weight(ez2, kb) * kb_weight(ey2, kb) * kb_weight(ex2, kb);
    }
    off = tap_offset(cf, g);
    return true;
}

// Weight and tile offset of a core candidate (ci < g.lcore: inside the
// support for every sample of the sub-cube, so there is nothing to test).
template <bool RADIAL>
__device__ __forceinline__ void tap_core(int ci, const SampleGeo &g, const CandSmem &cs, const KBParams &kb,
                                         float &w, int &off)
{
    const float4 cf = cs.f[g.lbase + ci];
    const float ex = cf.x - g.fx, ey = cf.y - g.fy, ez = cf.z - g.fz;
    const float ex2 = ex * ex, ey2 = ey * ey, ez2 = ez * ez;
    if (RADIAL)
        w = kb_weight(ez2 + ey2 + ex2, kb);
    else
        w = kb_weight(ez2, kb) * kb_weight(ey2, kb) * kb_weight(ex2, kb);
    off = tap_offset(cf, g);
}

// Visit every (tile point, coil) of the padded tile with the grid point it
// maps to: warps take tile rows (one division per row), lanes run along x and
// the coil index (V values per point) so global accesses stay contiguous.
// F(pt, c, gidx) with pt the tile-local point and gidx the grid point.
template <int V, typename F>
__device__ __forceinline__ void for_tile_rows(const Geom &g, int ox, int oy, int oz, F &&f)
{
    const int Px = g.P[0], Py = g.P[1], Pz = g.P[2];
    const int rowlen = Px * V;
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5, lane = threadIdx.x & 31;
    const bool simple = Px <= g.K[0];
    for (int row = warp; row < Py * Pz; row += nwarps) {
        const int ly = row % Py, lz = row / Py;
        const int gy = wrap_idx(oy + ly, g.K[1]), gz = wrap_idx(oz + lz, g.K[2]);
        const size_t rb = ((size_t)gz * g.K[1] + gy) * g.K[0];
        for (int q = lane; q < rowlen; q += 32) {
            const int lx = q / V, c = q - lx * V;
            int gx = ox + lx;
            if (simple) {
                gx += gx < 0 ? g.K[0] : 0;
                gx -= gx >= g.K[0] ? g.K[0] : 0;
            } else {
                gx = wrap_idx(gx, g.K[0]);
            }
            f(row * Px + lx, c, rb + gx);
        }
    }
}

// Work layout of the spread: one warp per sample.  The 32 lanes evaluate 64
// candidate taps at a time, two per lane with packed FP32x2 arithmetic
// (weight + tile offset); the hits are compacted through a per-warp queue
// and then applied by sub-steps in which lane (q, j) handles queued tap j for
// coil pair q (NP pairs, CPS taps per sub-step).  A quarter-warp adds 8 taps
// of one coil plane; the candidate order keeps their offsets distinct modulo
// 8 where it can, so the reductions meet few bank conflicts.  (The gather
// uses 8 lanes per sample instead, below.)
template <int CB>
struct Lanes {
    static constexpr int NP = CB >= 2 ? CB / 2 : 1;  // coil pairs (or one coil)
    static constexpr int CPS = 32 / NP;               // queued taps per sub-step
};

__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// kb_weight for two distances at once: the polynomial with packed FP32x2
// operations (the same rounding as the scalar steps), else two scalar calls.
__device__ __forceinline__ float2 kb_weight2(float2 d2, const KBParams &p)
{
    if (p.poly) {
        float2 t = __fmul2_rn(__fadd2_rn(dup2(p.half2), make_float2(-d2.x, -d2.y)), dup2(p.inv_half2));
        t.x = fmaxf(t.x, 0.f);
        t.y = fmaxf(t.y, 0.f);
        float2 s = dup2(p.c[kKBDeg]);
#pragma unroll
        for (int k = kKBDeg - 1; k >= 0; --k) s = __ffma2_rn(s, t, dup2(p.c[k]));
        return s;
    }
    return make_float2(kb_weight(d2.x, p), kb_weight(d2.y, p));
}

struct TapQueue2 {
    int2 e[64];  // (weight bits, tile offset) of the hits of 64 candidates
};

// Evaluate candidates [base, base+64) of sample sg, two per lane with packed
// FP32x2 arithmetic (lane l: candidates base+l and base+32+l); the hits go to
// the warp's queue in list order.  Returns the hit count.
template <bool RADIAL>
__device__ __forceinline__ int eval_pair(int base, const SampleGeo &sg, const CandPairs &cp,
                                         const KBParams &kb, TapQueue2 &qu, int lane)
{
    const int2 cc = cp.pc[sg.lbase + (base >> 1) + lane];
    const float2 X = pair_axis<0>(cc), Y = pair_axis<1>(cc), Z = pair_axis<2>(cc);
    // tile offsets: base + s*d' summed on top of 1.5*2^23 (exact integers)
    const float2 o = __ffma2_rn(Z, dup2(sg.sz), __ffma2_rn(Y, dup2(sg.sy), __ffma2_rn(X, dup2(sg.sx), dup2(sg.b))));
    const float h2 = kb.half2;
    float2 w;
    bool ha, hb;
    const float2 ex = __fadd2_rn(X, dup2(-sg.fx)), ey = __fadd2_rn(Y, dup2(-sg.fy)),
                 ez = __fadd2_rn(Z, dup2(-sg.fz));
    if (RADIAL) {
        const float2 d2 = __ffma2_rn(ez, ez, __ffma2_rn(ey, ey, __fmul2_rn(ex, ex)));
        ha = d2.x <= h2;
        hb = d2.y <= h2;
        w = kb_weight2(d2, kb);
    } else {
        const float2 ex2 = __fmul2_rn(ex, ex), ey2 = __fmul2_rn(ey, ey), ez2 = __fmul2_rn(ez, ez);
        ha = ex2.x <= h2 && ey2.x <= h2 && ez2.x <= h2;
        hb = ex2.y <= h2 && ey2.y <= h2 && ez2.y <= h2;
        w = __fmul2_rn(__fmul2_rn(kb_weight2(ez2, kb), kb_weight2(ey2, kb)), kb_weight2(ex2, kb));
    }
    const unsigned ma = __ballot_sync(0xffffffffu, ha), mb = __ballot_sync(0xffffffffu, hb);
    const unsigned lt = (1u << lane) - 1u;
    const int na = __popc(ma);
    if (ha) qu.e[__popc(ma & lt)] = make_int2(__float_as_int(w.x), __float_as_int(o.x) - 0x4B400000);
    if (hb) qu.e[na + __popc(mb & lt)] = make_int2(__float_as_int(w.y), __float_as_int(o.y) - 0x4B400000);
    __syncwarp();
    return na + __popc(mb);
}

// Gather: tile staged coil-major ([CB][P^3] complex) -> ks.  kGroup lanes per
// sample walk the candidate list; partial sums are reduced across the group.
// ------------------------------------------------- TMA tile staging
// Interior tiles of the gather (padded tile inside the grid on every axis)
// are staged by one bulk tensor copy of the box [z][y][x][CB coils] of the
// grid [K3][K2][K1][nc] complex (4-D map: 2*nc floats, K1, K2, K3), which
// lands point-major in shared memory.  Tiles that wrap around the grid edge
// use per-element asynchronous copies into the same layout.
// Waits are bounded (a plan option gives the number of polls): on expiry
// the block sets its plan's status flag (read by nufft3d_check_status and
// the host-pointer entry points), lets the copy land with a second bounded
// wait and returns.

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            unsigned bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
                 : "memory");
}

// Origin of the padded tile of tile index tid; true if it lies inside the
// grid on every axis (no wrap-around).
__device__ __forceinline__ bool tile_origin(const Geom &g, int tid, int &ox, int &oy, int &oz)
{
    const int tx = tid % g.nt[0];
    const int ty = (tid / g.nt[0]) % g.nt[1];
    const int tz = tid / (g.nt[0] * g.nt[1]);
    ox = tx * g.T[0] - g.Ra[0];
    oy = ty * g.T[1] - g.Ra[1];
    oz = tz * g.T[2] - g.Ra[2];
    return ox >= 0 && oy >= 0 && oz >= 0 && ox + g.P[0] <= g.K[0] && oy + g.P[1] <= g.K[1] &&
           oz + g.P[2] <= g.K[2];
}

// Bounded wait for the phase of the given parity (at most `polls` polls);
// false if it expired.
constexpr int kDrainPolls = 1 << 22;

__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity, int polls)
{
    for (int i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}


__device__ __forceinline__ float2 *align128(float4 *p)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(p);
    return reinterpret_cast<float2 *>(reinterpret_cast<char *>(p) + ((128u - (sa & 127u)) & 127u));
}

// acc[c] += w * tile(c, off): coil pairs come from one 16-byte load of a pair
// plane; a quarter-warp is one sample's chunk of 8 candidates, whose tile
// words the plan-time candidate order spreads over distinct bank groups.
// Gather tile layout: point-major, one record of CB coils (8*CB bytes) per
// tile point, as the bulk tensor copy lands it.  Lane l of a sample's group
// reads the 16-byte coil pairs of a tap in the rotated order pair = rot ^ k
// (rot = l mod NP, k = 0..NP-1), so that in each load the 8 lanes touch 8
// different 16-byte bank groups when lanes l and l+4 (same rot) hold taps of
// different parity (the candidate order is chosen for that); acc holds the
// pairs in that rotated order until unrotate().
template <int CB>
__device__ __forceinline__ void accumulate(float2 (&acc)[CB], const float2 *tile, int off, float w,
                                           const int (&ko)[CB >= 2 ? CB / 2 : 1])
{
    if constexpr (CB >= 2) {
        const char *pb = reinterpret_cast<const char *>(tile) + (size_t)off * (CB * 8);
        const float2 ww = make_float2(w, w);
#pragma unroll
        for (int k = 0; k < CB / 2; ++k) {
            const float4 v = *reinterpret_cast<const float4 *>(pb + ko[k]);
            // packed FP32x2 FMAs (one instruction per complex value, same rounding as fmaf)
            acc[2 * k] = __ffma2_rn(ww, make_float2(v.x, v.y), acc[2 * k]);
            acc[2 * k + 1] = __ffma2_rn(ww, make_float2(v.z, v.w), acc[2 * k + 1]);
        }
    } else {
        acc[0] = __ffma2_rn(make_float2(w, w), tile[off], acc[0]);
    }
}

// acc[2k..2k+1] (pair rot ^ k) -> acc[2p..2p+1] (pair p): conditional swaps
// of pair k with k^1 (rot bit 0) and k^2 (rot bit 1).
template <int CB>
__device__ __forceinline__ void unrotate(float2 (&acc)[CB], int rot)
{
    if constexpr (CB >= 4) {
#pragma unroll
        for (int b = 1; b < CB / 2; b <<= 1) {
            const bool sw = rot & b;
#pragma unroll
            for (int k = 0; k < CB / 2; ++k) {
                if (k & b) continue;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float2 lo = acc[2 * k + h], hi = acc[2 * (k ^ b) + h];
                    acc[2 * k + h] = sw ? hi : lo;
                    acc[2 * (k ^ b) + h] = sw ? lo : hi;
                }
            }
        }
    }
}

// Stage the padded tile of piece bi: one bulk tensor copy for interior tiles
// (completing phase `phase` of the barrier), else per-element asynchronous
// copies.  Returns false, uniformly over the block, if a bulk copy did not
// complete; the tile is then not to be read.
template <int CB>
__device__ __forceinline__ bool stage_tile(const float2 *__restrict__ G, int nc, int c0, const int4 bi,
                                           const Geom &g, float2 *tile, const CUtensorMap *tmap, unsigned bar_sa,
                                           unsigned &phase, const InterpStatus &st)
{
    int ox, oy, oz;
    const bool inside = tile_origin(g, bi.x, ox, oy, oz);
    const int cb = min(CB, nc - c0);
    const bool bulk = tmap != nullptr && inside;
    if (bulk) {
        if (threadIdx.x == 0) {
            mbar_expect_tx(bar_sa, (unsigned)(g.P[0] * g.P[1] * g.P[2] * CB * sizeof(float2)));
            tma_load_4d((unsigned)__cvta_generic_to_shared(tile), tmap, 2 * c0, ox, oy, oz, bar_sa);
        }
        const bool done = mbar_wait_bounded(bar_sa, phase, st.polls);
        phase ^= 1u;
        if (__syncthreads_or(!done)) {     // block-uniform exit on expiry
            if (threadIdx.x == 0) {
                if (st.err) atomicOr(st.err, 1);
                mbar_wait_bounded(bar_sa, phase ^ 1u, kDrainPolls);  // let the copy land before the block exits
            }
            __syncthreads();
            return false;
        }
    } else {
        // stage the padded tile with asynchronous copies (no register round trip)
        for_tile_rows<CB>(g, ox, oy, oz, [&](int pt, int c, size_t gidx) {
            float2 *dst = &tile[(size_t)pt * CB + c];
            if (c < cb) {
                const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(&G[gidx * nc + c0 + c])
                             : "memory");
            } else {
                *dst = make_float2(0.f, 0.f);
            }
        });
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();
    }
    return true;
}

// One tile piece of the gather: stage the padded tile, then interpolate the
// piece's samples.  Entered and left with the tile free for the next piece
// (the caller's barrier).  Returns false, uniformly over the block, if a
// bulk copy did not complete.
template <int CB, bool RADIAL, int R>
__device__ __forceinline__ bool gather_piece(const float2 *__restrict__ G, float2 *__restrict__ ks, int nc, int c0,
                                             const float4 *__restrict__ samples, const int4 bi, const Geom &g,
                                             const KBParams &kb, float scale, const float *__restrict__ wsample,
                                             const CandSmem &cs, float2 *tile, const CUtensorMap *tmap,
                                             unsigned bar_sa, unsigned &phase, const InterpStatus &st)
{
    if (!stage_tile<CB>(G, nc, c0, bi, g, tile, tmap, bar_sa, phase, st)) return false;
    const int Px = g.P[0];
    const int cb = min(CB, nc - c0);
    const int lane = threadIdx.x & 31;
    const int lig = lane & (kGroup - 1);
    const unsigned gmask = 0xFFu << (lane & ~(kGroup - 1));
    const int rot = CB >= 2 ? lig & (CB / 2 - 1) : 0;
    int ko[CB >= 2 ? CB / 2 : 1];
#pragma unroll
    for (int k = 0; k < (CB >= 2 ? CB / 2 : 1); ++k) ko[k] = (rot ^ k) << 4;
    const int grp = threadIdx.x / kGroup, ngrp = blockDim.x / kGroup;
    const int send = bi.y + bi.z;
    float4 rec_next = bi.y + grp < send ? __ldg(&samples[bi.y + grp]) : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int s = bi.y + grp; s < send; s += ngrp) {
        const SampleGeo sg = sample_geo(rec_next, Px, g.P[1], cs);
        if (s + ngrp < send) rec_next = __ldg(&samples[s + ngrp]);
        const int niter = (sg.ln + kGroup - 1) / kGroup;
        const int ncore = sg.lcore / kGroup;  // steps whose 8 candidates are all core
        float2 acc[CB];
#pragma unroll
        for (int c = 0; c < CB; ++c) acc[c] = make_float2(0.f, 0.f);
        int it = 0;
        // core candidates: no support test, two per step (ILP)
        for (; it + 1 < ncore; it += 2) {
            const int ci0 = it * kGroup + lig, ci1 = ci0 + kGroup;
            float w0, w1;
            int off0, off1;
            tap_core<RADIAL>(ci0, sg, cs, kb, w0, off0);
            tap_core<RADIAL>(ci1, sg, cs, kb, w1, off1);
            accumulate<CB>(acc, tile, off0, w0, ko);
            accumulate<CB>(acc, tile, off1, w1, ko);
        }
        // the rest, two independent candidates per step (ILP)
        for (; it < niter; it += 2) {
            const int ci0 = it * kGroup + lig, ci1 = ci0 + kGroup;
            float w0, w1;
            int off0, off1;
            // (branchy form: a branch-free variant with predicated loads was slower here)
            const bool h0 = ci0 < sg.ln && tap<RADIAL>(ci0, sg, cs, kb, w0, off0);
            const bool h1 = ci1 < sg.ln && tap<RADIAL>(ci1, sg, cs, kb, w1, off1);
            if (h0) accumulate<CB>(acc, tile, off0, w0, ko);
            if (h1) accumulate<CB>(acc, tile, off1, w1, ko);
        }
        unrotate<CB>(acc, rot);
#pragma unroll
        for (int c = 0; c < CB; ++c) {
#pragma unroll
            for (int o = kGroup / 2; o > 0; o >>= 1) {
                acc[c].x += __shfl_xor_sync(gmask, acc[c].x, o);
                acc[c].y += __shfl_xor_sync(gmask, acc[c].y, o);
            }
        }
        const float sc_ = wsample ? scale * __ldg(&wsample[s]) : scale;
        float2 *o = ks + (size_t)s * nc + c0;
#pragma unroll
        for (int c = 0; c < CB; ++c)
            if (c % kGroup == lig && c < cb) o[c] = make_float2(acc[c].x * sc_, acc[c].y * sc_);
    }
    __syncthreads();  // every warp is done with the tile
    return true;
}

// Shared set-up of the gather blocks: candidate tables, tile, barrier.
struct GatherSmem {
    CandSmem cs;
    float2 *tile;
    unsigned bar_sa;
};

__device__ __forceinline__ GatherSmem gather_setup(const Cand &cd, float4 *smem4, unsigned long long *bar)
{
    GatherSmem m;
    m.tile = align128(carve_cand(cd, m.cs, smem4));
    m.bar_sa = bar ? (unsigned)__cvta_generic_to_shared(bar) : 0u;
    build_cand(cd, m.cs);
    if (bar && threadIdx.x == 0) mbar_init(m.bar_sa, 1);
    __syncthreads();
    return m;
}

// Persistent gather: one block per SM takes tile pieces in order (largest
// first) from a work counter, so the candidate tables and the barrier are set
// up once per SM instead of once per piece.
template <int CB, bool RADIAL, int R>
__global__ void __launch_bounds__(kInterpThreads)
k_gather(const float2 *__restrict__ G, float2 *__restrict__ ks, int nc, int c0,
         const float4 *__restrict__ samples, const int4 *__restrict__ blocks, int nblocks, int *__restrict__ work,
         Geom g, KBParams kb, float scale, const float *__restrict__ wsample, const __grid_constant__ Cand cd,
         const __grid_constant__ CUtensorMap tmap, int use_tma, InterpStatus st)
{
    extern __shared__ float4 smem4[];
    __shared__ unsigned long long bar;
    __shared__ int next;
    const GatherSmem m = gather_setup(cd, smem4, &bar);
    unsigned phase = 0;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(work, 1);
        __syncthreads();
        const int b = next;
        if (b >= nblocks) break;
        if (!gather_piece<CB, RADIAL, R>(G, ks, nc, c0, samples, blocks[b], g, kb, scale, wsample, m.cs, m.tile,
                                         use_tma ? &tmap : nullptr, m.bar_sa, phase, st))
            return;
    }
}

// Spread: ks -> tile -> grid.  The tile accumulates in 32-bit fixed point
// with native shared-memory integer reductions (floating-point shared atomics
// are several times slower on this part).  Per piece and coil the scale is a
// power of two 2^F chosen from that coil's largest |Re|,|Im| over the piece's
// samples and the plan-time bound wsum = max over tile points of the summed
// weights, so that every partial sum stays below 2^30 and every product
// w*y*2^F below 2^22; products are rounded to integers exactly by the
// 1.5*2^23 addition.  Each coil keeps its own precision whatever the gain of
// the other coils of the pass (coils of unrelated requests can share a pass).
// Layout [CB][2][P^3] int32 (split real/imaginary planes, so a warp's
// scattered taps spread over all banks).  A warp takes one sample: its hits
// are compacted into a queue and each quarter-warp adds one coil pair of 8
// queued taps per instruction (the candidate order keeps those 8 offsets in
// distinct bank groups where it can).  The tile
// is then added to the grid with vector atomics (neighbouring tiles' halos
// overlap).
__device__ __forceinline__ float block_max(float v, float *red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        float r = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
        if (threadIdx.x == 0) red[32] = r;
    }
    __syncthreads();
    return red[32];
}

// Shared-memory reduction at a 32-bit shared address plus a compile-time
// byte offset (the planes of one tap differ by constant strides).
template <int IMM>
__device__ __forceinline__ void red_add_at(unsigned a, int v)
{
    asm volatile("red.shared.add.u32 [%0+%2], %1;" ::"r"(a), "r"(v), "n"(IMM) : "memory");
}

// round(a*b) for |a*b| < 2^22 with one fused rounding: the exact product is
// added to 1.5*2^23, which leaves an integer in the low mantissa bits; two
// at a time with one packed FP32x2 FMA
__device__ __forceinline__ int2 to_fixed_mul2(float2 a, float2 b)
{
    const float2 r = __ffma2_rn(a, b, make_float2(12582912.0f, 12582912.0f));
    return make_int2(__float_as_int(r.x) - 0x4B400000, __float_as_int(r.y) - 0x4B400000);
}

// Integer planes of the spread: one plane per (coil, re/im); the stride is
// the smallest value >= the tile volume that is 2 mod 32, so a warp's 32
// reductions (8 neighbouring points x 4 planes 2 apart) hit 32 distinct banks.
template <int R>
struct IPlane {
    static constexpr int PS = ((Plane<R>::PS + 29) / 32) * 32 + 2;
};

// Per-coil fixed-point scales of a spread piece: psc[c] = 2^F_c and
// psc[kMaxCB + c] = 2^-F_c from coil c's largest |Re|,|Im| over the piece
// and the plan-time bound on summed weights (coils that are zero over the
// piece get F = 0: they add nothing).  red holds 32*CB floats.  Returns
// false (block-uniform) when the piece adds nothing.  Contains __syncthreads.
constexpr int kMaxCB = 8;

template <int CB>
__device__ __forceinline__ bool piece_scale(const float2 *__restrict__ ks, int nc, int c0, int cb, const int4 bi,
                                            float *red, float *psc)
{
    const int send = bi.y + bi.z;
    float m[CB];
#pragma unroll
    for (int c = 0; c < CB; ++c) m[c] = 0.f;
    for (int s = bi.y + threadIdx.x; s < send; s += blockDim.x) {
        const float2 *src = ks + (size_t)s * nc + c0;
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            if (c < cb) {
                const float2 v = src[c];
                m[c] = fmaxf(m[c], fmaxf(fabsf(v.x), fabsf(v.y)));
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < CB; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m[c] = fmaxf(m[c], __shfl_xor_sync(0xffffffffu, m[c], o));
    }
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < CB; ++c) red[warp * CB + c] = m[c];
    }
    __syncthreads();
    bool any = false;
    if (threadIdx.x < CB) {
        const int c = threadIdx.x;
        float ymax = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) ymax = fmaxf(ymax, red[w * CB + c]);
        int F = 0;
        if (ymax > 0.f) {
            any = true;
            const float wsum = fmaxf(__int_as_float(bi.w), 1.0f);
            int ey, ecy;
            frexpf(ymax, &ey);                     // ymax < 2^ey
            frexpf(ymax * wsum, &ecy);             // wsum*ymax < 2^ecy
            F = max(-126, min(126, min(22 - ey, 30 - ecy)));
        }
        psc[c] = ldexpf(1.f, F);
        psc[kMaxCB + c] = ldexpf(1.f, -F);
    }
    return __syncthreads_or(any) != 0;  // also: psc is visible to the block, red free again
}

// Add the integer planes of piece bi to the grid (vector atomics: the halos
// of neighbouring tiles overlap) and return every plane read to zero.
template <int CB, int R>
__device__ __forceinline__ void flush_tile(float2 *__restrict__ G, int nc, int c0, int cb, const int4 bi,
                                           const Geom &g, int *tile, const float *inv_scale)
{
    constexpr int ps = IPlane<R>::PS;
    int ox, oy, oz;
    tile_origin(g, bi.x, ox, oy, oz);
    if (CB % 2 == 0 && nc % 2 == 0 && c0 % 2 == 0) {
        for_tile_rows<CB / 2>(g, ox, oy, oz, [&](int pt, int cq, size_t gidx) {
            const int cc = 2 * cq;
            if (cc >= cb) return;
            int *t0 = tile + (size_t)(2 * cc) * ps + pt;
            const int a = t0[0], b = t0[ps], e = t0[2 * ps], f = t0[3 * ps];
            if ((a | b | e | f) == 0) return;
            t0[0] = 0;
            t0[ps] = 0;
            t0[2 * ps] = 0;
            t0[3 * ps] = 0;
            const float s0 = inv_scale[cc], s1 = inv_scale[cc + 1];
            atomicAdd(reinterpret_cast<float4 *>(&G[gidx * nc + c0 + cc]),
                      make_float4(a * s0, b * s0, e * s1, f * s1));
        });
    } else {
        for_tile_rows<CB>(g, ox, oy, oz, [&](int pt, int cc, size_t gidx) {
            if (cc >= cb) return;
            int *t0 = tile + (size_t)(2 * cc) * ps + pt;
            const int a = t0[0], b = t0[ps];
            if ((a | b) == 0) return;
            t0[0] = 0;
            t0[ps] = 0;
            const float s0 = inv_scale[cc];
            atomicAdd(&G[gidx * nc + c0 + cc], make_float2(a * s0, b * s0));
        });
    }
}

// One tile piece of the spread into integer planes that are zero on entry
// (the flush returns every plane it reads to zero, so a persistent block
// zeroes its tile only once).  Entered and left with the tile free.
template <int CB, bool RADIAL, int R>
__device__ __forceinline__ void spread_piece(const float2 *__restrict__ ks, float2 *__restrict__ G, int nc, int c0,
                                             const float4 *__restrict__ samples, const int4 bi, const Geom &g,
                                             const KBParams &kb, const CandPairs &cs, int *tile, float *red,
                                             float *psc, TapQueue2 *queues)
{
    constexpr int NP = Lanes<CB>::NP, CPS = Lanes<CB>::CPS;
    constexpr int ps = IPlane<R>::PS;
    const int Px = g.P[0];
    const int cb = min(CB, nc - c0);
    const int send = bi.y + bi.z;
    if (!piece_scale<CB>(ks, nc, c0, cb, bi, red, psc)) return;  // the tile stays zero
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int q = lane / CPS, j = lane % CPS;
    const int c = CB >= 2 ? 2 * q : 0;
    // this lane's coils' scales (c + 1 < CB whenever CB >= 2)
    const float sa = psc[c], sb = CB >= 2 ? psc[c + 1] : 0.f;
    int *pl0 = tile + (size_t)(2 * c) * ps;  // re, im of coil c; then re, im of coil c+1
    const unsigned pl0_sa = (unsigned)__cvta_generic_to_shared(pl0);
    TapQueue2 &qu = queues[warp];
    auto load_y = [&](int s, float4 &y) {
        const float2 *src = ks + (size_t)s * nc + c0;
        const float2 a = c < cb ? src[c] : make_float2(0.f, 0.f);
        const float2 b = (CB >= 2 && c + 1 < cb) ? src[c + 1] : make_float2(0.f, 0.f);
        y = make_float4(a.x * sa, a.y * sa, b.x * sb, b.y * sb);
    };
    float4 rec_next = make_float4(0.f, 0.f, 0.f, 0.f), y_next = make_float4(0.f, 0.f, 0.f, 0.f);
    if (bi.y + warp < send) {
        rec_next = __ldg(&samples[bi.y + warp]);
        load_y(bi.y + warp, y_next);
    }
    for (int s = bi.y + warp; s < send; s += nwarps) {
        const SampleGeo sg = sample_geo_pairs(rec_next, Px, g.P[1], cs);
        const float4 y = y_next;
        if (s + nwarps < send) {
            rec_next = __ldg(&samples[s + nwarps]);
            load_y(s + nwarps, y_next);
        }
        for (int base = 0; base < sg.ln; base += 64) {
            const int nh = eval_pair<RADIAL>(base, sg, cs, kb, qu, lane);
            for (int t = j; t < nh; t += CPS) {
                const int2 qe = qu.e[t];
                const float w = __int_as_float(qe.x);
                const unsigned a = pl0_sa + 4u * (unsigned)qe.y;
                const float2 ww = make_float2(w, w);
                const int2 v0 = to_fixed_mul2(ww, make_float2(y.x, y.y));
                red_add_at<0>(a, v0.x);
                red_add_at<4 * ps>(a, v0.y);
                if (CB >= 2) {
                    const int2 v1 = to_fixed_mul2(ww, make_float2(y.z, y.w));
                    red_add_at<8 * ps>(a, v1.x);
                    red_add_at<12 * ps>(a, v1.y);
                }
            }
            __syncwarp();
        }
    }
    __syncthreads();
    flush_tile<CB, R>(G, nc, c0, cb, bi, g, tile, psc + kMaxCB);
    __syncthreads();  // the tile is zero again
}

template <int R>
__device__ __forceinline__ int *spread_setup(const Cand &cd, CandPairs &cs, float4 *smem4, int cbk)
{
    constexpr int ps = IPlane<R>::PS;
    int *tile = reinterpret_cast<int *>(carve_pairs(cd, cs, smem4));
    // zero the integer planes once, with 16-byte stores (ps * cbk * 2 is a multiple of 4)
    int4 *t4 = reinterpret_cast<int4 *>(tile);
    for (int t = threadIdx.x; t < ps * cbk / 2; t += blockDim.x) t4[t] = make_int4(0, 0, 0, 0);
    build_pairs(cd, cs);
    __syncthreads();
    return tile;
}

// Persistent spread: one block per SM takes tile pieces from a work counter.
template <int CB, bool RADIAL, int R>
__global__ void __launch_bounds__(kInterpThreads)
k_spread(const float2 *__restrict__ ks, float2 *__restrict__ G, int nc, int c0,
         const float4 *__restrict__ samples, const int4 *__restrict__ blocks, int nblocks, int *__restrict__ work,
         Geom g, KBParams kb, const __grid_constant__ Cand cd)
{
    extern __shared__ float4 smem4[];
    __shared__ float red[32 * CB];
    __shared__ float psc[2 * kMaxCB];
    __shared__ TapQueue2 queues[kInterpThreads / 32];
    __shared__ int next;
    CandPairs cs;
    int *tile = spread_setup<R>(cd, cs, smem4, CB);
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(work, 1);
        __syncthreads();
        const int b = next;
        if (b >= nblocks) break;
        spread_piece<CB, RADIAL, R>(ks, G, nc, c0, samples, blocks[b], g, kb, cs, tile, red, psc, queues);
    }
}

// Plan-time bound for the fixed-point spread: for each block, the largest
// sum of kernel weights its samples put on one tile point (float shared
// atomics; runs once per plan).  Written to blocks[b].w as float bits.
template <bool RADIAL>
__global__ void __launch_bounds__(kInterpThreads)
k_weight_sum(const float4 *__restrict__ samples, int4 *__restrict__ blocks, Geom g, KBParams kb,
             const __grid_constant__ Cand cd)
{
    extern __shared__ float4 smem4[];
    __shared__ float red[33];
    const int Px = g.P[0], PxPy = g.P[0] * g.P[1];
    const int pv = PxPy * g.P[2];
    CandSmem cs;
    float *tile = reinterpret_cast<float *>(carve_cand(cd, cs, smem4));
    const int4 bi = blocks[blockIdx.x];
    for (int t = threadIdx.x; t < pv; t += blockDim.x) tile[t] = 0.f;
    build_cand(cd, cs);
    __syncthreads();
    const int lig = threadIdx.x & (kGroup - 1);
    const int grp = threadIdx.x / kGroup, ngrp = blockDim.x / kGroup;
    for (int s = bi.y + grp; s < bi.y + bi.z; s += ngrp) {
        const SampleGeo sg = sample_geo(__ldg(&samples[s]), Px, g.P[1], cs);
        for (int ci = lig; ci < sg.ln; ci += kGroup) {
            float w;
            int off;
            if (tap<RADIAL>(ci, sg, cs, kb, w, off)) atomicAdd(&tile[off], w);
        }
    }
    __syncthreads();
    float m = 0.f;
    for (int t = threadIdx.x; t < pv; t += blockDim.x) m = fmaxf(m, tile[t]);
    m = block_max(m, red);
    // small safety margin over the single-precision sums
    if (threadIdx.x == 0) blocks[blockIdx.x].w = __float_as_int(m * 1.001f + 1e-3f);
}

// ------------------------------------------------------------- stored H
// The reference keeps H as a sparse matrix (nufft_3d.m:153-212).  Its stored
// form here follows the tile sort: the row of sorted sample s is a run of
// (weight bits, tile offset) entries in chunks of 8 taps, padded with zero
// weights to a whole chunk; the rows of a piece are contiguous, so the gather
// streams them with plain loads that run ahead of the taps and evaluates no
// kernel weights.  Inside a row the taps are ordered for the shared-memory
// banks: round-robin over the residue of the tile offset mod 8, and inside
// each chunk even offsets before odd ones (gather lanes k and k+4 read one
// 16-byte column of the point-major tile, conflict-free when their offsets
// differ in parity: about 0.12 collisions per chunk on J=6 radial rows).
// The residue order would also keep a chunk's 8 taps on distinct banks of
// the spread's integer planes (about 1.13 wavefronts per chunk), but a
// spread that streams H through shared memory measured slower than one that
// evaluates the kernel (staging H costs as many instructions as the weights
// it saves), so H' is applied on the fly.  The weights are the on-the-fly
// kernels' (same candidate lists and kernel).

// Streaming load of one stored-H entry (read once: no L1 allocation).
__device__ __forceinline__ int2 ld_tap(const int2 *p)
{
    int2 v;
    asm volatile("ld.global.nc.L1::no_allocate.v2.s32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

// One tile piece of the gather from the stored H (8 coils per pass).  Each
// group of 8 lanes takes a contiguous run of the piece's samples, whose rows
// form one contiguous stream of chunks; lane l of the group applies entry l
// of every chunk (a whole tap: 8 coils, rotated coil-pair reads as in the
// on-the-fly gather) and keeps the next 4 chunks' entries in registers, so
// the loads run ahead across sample boundaries (2, 3 or 6 chunks in
// registers, a 5-deep per-lane shared-memory FIFO filled by asynchronous
// copies, and L2 prefetch windows all measured slower).  At the end of a
// sample the group reduces its 8 partial sums.
template <int R>
__device__ __forceinline__ bool gather_piece_tab(const float2 *__restrict__ G, float2 *__restrict__ ks, int nc,
                                                 int c0, const int4 bi, const Geom &g, float scale,
                                                 const float *__restrict__ wsample,
                                                 const uint32_t *__restrict__ rows, const int2 *__restrict__ taps,
                                                 float2 *tile, const CUtensorMap *tmap, unsigned bar_sa,
                                                 unsigned &phase, const InterpStatus &stat)
{
    constexpr int CB = 8;
    const int lane = threadIdx.x & 31, lig = lane & 7;
    const int grp = threadIdx.x >> 3, ngrp = blockDim.x >> 3;
    const unsigned gmask = 0xFFu << (lane & 24);
    const int s_lo = bi.y + (int)(((long long)bi.z * grp) / ngrp);
    const int s_hi = bi.y + (int)(((long long)bi.z * (grp + 1)) / ngrp);
    uint32_t cA = 0, nchk = 0;
    if (s_lo < s_hi) {
        cA = __ldg(&rows[s_lo]);
        nchk = __ldg(&rows[s_hi]) - cA;
    }
    const int2 *st = taps + (size_t)cA * 8 + lig;
    const int2 z2 = make_int2(0, 0);
    // the first chunks land while the tile does
    int2 e0 = nchk > 0 ? ld_tap(st) : z2;
    int2 e1 = nchk > 1 ? ld_tap(st + 8) : z2;
    int2 e2 = nchk > 2 ? ld_tap(st + 16) : z2;
    int2 e3 = nchk > 3 ? ld_tap(st + 24) : z2;
    if (!stage_tile<CB>(G, nc, c0, bi, g, tile, tmap, bar_sa, phase, stat)) return false;
    const int cb = min(CB, nc - c0);
    const int rot = lig & 3, rot16 = rot << 4;
    float2 acc[CB];
#pragma unroll
    for (int c = 0; c < CB; ++c) acc[c] = make_float2(0.f, 0.f);
    int s = s_lo;
    uint32_t send = s < s_hi ? __ldg(&rows[s + 1]) - cA : 0u;      // chunk where sample s ends
    uint32_t snext = s + 1 < s_hi ? __ldg(&rows[s + 2]) - cA : 0u;  // and sample s+1
    // write sample s, move to the next one.  Reduce-scatter over the group:
    // at each of 3 steps a lane keeps half of its coils (the half named by
    // one bit of its lane index) and adds the partner's copy of them, so lane
    // l ends with coil l summed over the 8 lanes (14 shuffles instead of 48).
    auto finish = [&]() {
        unrotate<CB>(acc, rot);
        float2 h4[4], h2[2], h1;
        const bool b2 = lig & 4, b1 = lig & 2, b0 = lig & 1;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 keep = b2 ? acc[4 + k] : acc[k], give = b2 ? acc[k] : acc[4 + k];
            h4[k].x = keep.x + __shfl_xor_sync(gmask, give.x, 4);
            h4[k].y = keep.y + __shfl_xor_sync(gmask, give.y, 4);
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const float2 keep = b1 ? h4[2 + k] : h4[k], give = b1 ? h4[k] : h4[2 + k];
            h2[k].x = keep.x + __shfl_xor_sync(gmask, give.x, 2);
            h2[k].y = keep.y + __shfl_xor_sync(gmask, give.y, 2);
        }
        {
            const float2 keep = b0 ? h2[1] : h2[0], give = b0 ? h2[0] : h2[1];
            h1.x = keep.x + __shfl_xor_sync(gmask, give.x, 1);
            h1.y = keep.y + __shfl_xor_sync(gmask, give.y, 1);
        }
        const float sc_ = wsample ? scale * __ldg(&wsample[s]) : scale;
        if (lig < cb) ks[(size_t)s * nc + c0 + lig] = make_float2(h1.x * sc_, h1.y * sc_);
#pragma unroll
        for (int c = 0; c < CB; ++c) acc[c] = make_float2(0.f, 0.f);
        ++s;
        send = snext;
        snext = s + 1 < s_hi ? __ldg(&rows[s + 2]) - cA : 0u;
    };
    while (s < s_hi && send == 0u) finish();  // samples without taps
    auto step = [&](int2 &ed, uint32_t ch) {
        const int2 cur = ed;
        ed = ch + 4 < nchk ? ld_tap(st + (size_t)(ch + 4) * 8) : z2;
        // coil pairs in the rotated order rot ^ k (see accumulate); padding
        // entries (weight 0, tile offset 0) add nothing and need no branch
        const float w = __int_as_float(cur.x);
        const float2 ww = make_float2(w, w);
        const char *pb = reinterpret_cast<const char *>(tile) + (size_t)cur.y * (CB * 8);
#pragma unroll
        for (int k = 0; k < CB / 2; ++k) {
            const float4 v = *reinterpret_cast<const float4 *>(pb + (rot16 ^ (k << 4)));
            acc[2 * k] = __ffma2_rn(ww, make_float2(v.x, v.y), acc[2 * k]);
            acc[2 * k + 1] = __ffma2_rn(ww, make_float2(v.z, v.w), acc[2 * k + 1]);
        }
        if (ch + 1 == send) {
            do {
                finish();
            } while (s < s_hi && send == ch + 1);  // and the samples without taps after it
        }
    };
    for (uint32_t ch = 0; ch < nchk; ch += 4) {
        step(e0, ch);
        if (ch + 1 < nchk) step(e1, ch + 1);
        if (ch + 2 < nchk) step(e2, ch + 2);
        if (ch + 3 < nchk) step(e3, ch + 3);
    }
    __syncthreads();  // every warp is done with the tile
    return true;
}

// Persistent gather from the stored H: shared memory = the tile.
template <int R>
__global__ void __launch_bounds__(kInterpThreads)
k_gather_tab(const float2 *__restrict__ G, float2 *__restrict__ ks, int nc, int c0,
             const int4 *__restrict__ blocks, int nblocks, int *__restrict__ work, Geom g, float scale,
             const float *__restrict__ wsample, const uint32_t *__restrict__ rows, const int2 *__restrict__ taps,
             const __grid_constant__ CUtensorMap tmap, int use_tma, InterpStatus st)
{
    extern __shared__ float4 smem4[];
    __shared__ unsigned long long bar;
    __shared__ int next;
    float2 *tile = align128(smem4);
    const unsigned bar_sa = (unsigned)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) mbar_init(bar_sa, 1);
    __syncthreads();
    unsigned phase = 0;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(work, 1);
        __syncthreads();
        const int b = next;
        if (b >= nblocks) break;
        if (!gather_piece_tab<R>(G, ks, nc, c0, blocks[b], g, scale, wsample, rows, taps, tile,
                                 use_tma ? &tmap : nullptr, bar_sa, phase, st))
            return;
    }
}

// Weight and tile offset of candidate ci for the stored H.  The distance is
// formed with explicitly rounded operations (never contracted into FMAs), so
// the count and fill passes, compiled separately, take identical support
// decisions.
template <bool RADIAL>
__device__ __forceinline__ bool tap_exact(int ci, const SampleGeo &g, const CandSmem &cs, const KBParams &kb,
                                          float &w, int &off)
{
    const float4 cf = cs.f[g.lbase + ci];
    const float ex = __fsub_rn(cf.x, g.fx), ey = __fsub_rn(cf.y, g.fy), ez = __fsub_rn(cf.z, g.fz);
    const float ex2 = __fmul_rn(ex, ex), ey2 = __fmul_rn(ey, ey), ez2 = __fmul_rn(ez, ez);
    const float h2 = kb.half2;
    if (RADIAL) {
        const float d2 = __fadd_rn(__fadd_rn(ez2, ey2), ex2);
        if (!(d2 <= h2)) return false;
        w = kb_weight(d2, kb);
    } else {
        if (!(ex2 <= h2 && ey2 <= h2 && ez2 <= h2)) return false;
        w = __fmul_rn(__fmul_rn(kb_weight(ez2, kb), kb_weight(ey2, kb)), kb_weight(ex2, kb));
    }
    off = tap_offset(cf, g);
    return true;
}

// Plan time, pass 1 of the stored H: rows[s] = 8-entry chunks of sample s's
// row (its hits, rounded up).  One warp per sample.
template <bool RADIAL>
__global__ void __launch_bounds__(256)
k_tap_count(const float4 *__restrict__ samples, int64_t nnz, Geom g, KBParams kb, const __grid_constant__ Cand cd,
            uint32_t *__restrict__ rows)
{
    extern __shared__ float4 smem4[];
    CandSmem cs;
    carve_cand(cd, cs, smem4);
    build_cand(cd, cs);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nnz; s += nw) {
        const SampleGeo sg = sample_geo(__ldg(&samples[s]), g.P[0], g.P[1], cs);
        int nh = 0;
        for (int base = 0; base < sg.ln; base += 32) {
            const int ci = base + lane;
            float w;
            int off;
            const bool hit = ci < sg.ln && tap_exact<RADIAL>(ci, sg, cs, kb, w, off);
            nh += __popc(__ballot_sync(0xffffffffu, hit));
        }
        if (lane == 0) rows[s] = (uint32_t)((nh + 7) >> 3);
    }
}

// Plan time, pass 2: the entries of every row in bank order (see above).
// Per warp two shared buffers of cap entries: the hits in candidate order,
// then in round-robin residue order.  *err is set if a row has more hits
// than the count pass found (the row is then cut at its length).
template <bool RADIAL>
__global__ void __launch_bounds__(256)
k_tap_fill(const float4 *__restrict__ samples, int64_t nnz, Geom g, KBParams kb, const __grid_constant__ Cand cd,
           const uint32_t *__restrict__ rows, int2 *__restrict__ taps, int cap, int *__restrict__ err)
{
    extern __shared__ float4 smem4[];
    CandSmem cs;
    int2 *bufs = reinterpret_cast<int2 *>(carve_cand(cd, cs, smem4));
    build_cand(cd, cs);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int2 *A = bufs + (size_t)warp * 2 * cap, *B = A + cap;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nnz; s += nw) {
        const SampleGeo sg = sample_geo(__ldg(&samples[s]), g.P[0], g.P[1], cs);
        int nh = 0;
        for (int base = 0; base < sg.ln; base += 32) {
            const int ci = base + lane;
            float w = 0.f;
            int off = 0;
            const bool hit = ci < sg.ln && tap_exact<RADIAL>(ci, sg, cs, kb, w, off);
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (hit) A[nh + __popc(m & ((1u << lane) - 1u))] = make_int2(__float_as_int(w), off);
            nh += __popc(m);
        }
        __syncwarp();
        // the row holds what the count pass found; never write past it
        const size_t row = (size_t)__ldg(&rows[s]) * 8;
        const int nfill = (int)((size_t)__ldg(&rows[s + 1]) * 8 - row);
        if (nh > nfill) {
            if (lane == 0) atomicOr(err, 1);
            nh = nfill;
        }
        // hits per residue of the tile offset mod 8
        int cnt = 0;
        if (lane < 8)
            for (int i = 0; i < nh; ++i) cnt += (A[i].y & 7) == lane;
        int n[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) n[r] = __shfl_sync(0xffffffffu, cnt, r);
        // round-robin order: level k holds the k-th hit of every residue that
        // has one, the residues with more hits first (they run out last)
        for (int i = lane; i < nh; i += 32) {
            const int2 e = A[i];
            const int r = e.y & 7;
            int rank = 0;
            for (int i2 = 0; i2 < i; ++i2) rank += (A[i2].y & 7) == r;
            int nr = 0;
#pragma unroll
            for (int r2 = 0; r2 < 8; ++r2) nr = r2 == r ? n[r2] : nr;
            int pos = 0;
#pragma unroll
            for (int r2 = 0; r2 < 8; ++r2) {
                const bool before = n[r2] > nr || (n[r2] == nr && r2 < r);
                pos += min(n[r2], rank) + ((before && n[r2] > rank) ? 1 : 0);
            }
            B[pos] = e;
        }
        __syncwarp();
        // inside each chunk: even offsets first, then odd ones; zero padding
        for (int p = lane; p < nfill; p += 32) {
            if (p >= nh) {
                taps[row + p] = make_int2(0, 0);
                continue;
            }
            const int c8 = p & ~7, end = min(c8 + 8, nh);
            int ev = 0, evb = 0;
            for (int k = c8; k < end; ++k) {
                const int even = (B[k].y & 1) == 0;
                ev += even;
                evb += (k < p) ? even : 0;
            }
            const int2 e = B[p];
            const int slot = (e.y & 1) ? ev + ((p - c8) - evb) : evb;
            taps[row + c8 + slot] = e;
        }
        __syncwarp();  // A and B are refilled for the next sample
    }
}

// user layout [M][nc] (coil-major) <-> sorted [nnz][nc] (coil fastest); the
// sorted side is read/written as one contiguous nc-vector per sample.
__global__ void k_permute_out(const float2 *__restrict__ ks, float2 *__restrict__ k,
                              const int32_t *__restrict__ inv, int64_t M, int nc, float scale)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const int s = inv[m];
    int c = 0;
    if ((nc & 1) == 0 && s >= 0) {
        // a sample's coils are one contiguous vector: 16-byte loads of pairs
        const float4 *src = reinterpret_cast<const float4 *>(ks + (size_t)s * nc);
        for (; c < nc; c += 2) {
            const float4 v = src[c >> 1];
            k[m + M * c] = make_float2(v.x * scale, v.y * scale);
            k[m + M * (c + 1)] = make_float2(v.z * scale, v.w * scale);
        }
    }
    for (; c < nc; ++c) {
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
    int c = 0;
    if ((nc & 1) == 0) {
        // write the sample's contiguous coil vector with 16-byte stores
        float4 *dst = reinterpret_cast<float4 *>(ks + (size_t)s * nc);
        for (; c < nc; c += 2) {
            const float2 a = k[m + M * c], b = k[m + M * (c + 1)];
            dst[c >> 1] = make_float4(a.x * w, a.y * w, b.x * w, b.y * w);
        }
    }
    for (; c < nc; ++c) {
        float2 v = k[m + M * c];
        ks[(size_t)s * nc + c] = make_float2(v.x * w, v.y * w);
    }
}

// Batched interpolation, persistent: one block per SM takes (volume, tile
// piece, first coil) entries of `table` (heaviest first) from a work counter.
// Every volume of a batch has the same kernel and tile shape, hence the same
// candidate tables, which are set up once per block.
template <int CB, bool RADIAL, int R>
__global__ void __launch_bounds__(kInterpThreads)
k_gather_batch(const BatchInterp *__restrict__ vols, const int4 *__restrict__ table, int ntab,
               int *__restrict__ work, KBParams kb)
{
    extern __shared__ float4 smem4[];
    __shared__ unsigned long long bar;
    __shared__ int next;
    const GatherSmem m = gather_setup(vols[0].cand, smem4, &bar);
    unsigned phase = 0;
    constexpr int lw = CB >= 8 ? 3 : CB >= 4 ? 2 : CB >= 2 ? 1 : 0;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(work, 1);
        __syncthreads();
        const int t = next;
        if (t >= ntab) break;
        const int4 e = table[t];
        const BatchInterp &b = vols[e.x];
        const CUtensorMap *tm = (b.tmap_ok >> lw) & 1 ? &b.tmaps[lw] : nullptr;
        // the kernel weights come from the parameter bank (shared by the batch)
        if (!gather_piece<CB, RADIAL, R>(b.in, b.out, b.nc, e.z, b.samples, b.blocks[e.y], b.g, kb, b.scale,
                                         b.wsample, m.cs, m.tile, tm, m.bar_sa, phase, b.status))
            return;
    }
}

// Batched 8-coil gather when every volume has its stored H: the table entry
// (volume, piece, first coil) selects the volume's rows; shared memory = the
// tile only.
template <int R>
__global__ void __launch_bounds__(kInterpThreads)
k_gather_batch_tab(const BatchInterp *__restrict__ vols, const int4 *__restrict__ table, int ntab,
                   int *__restrict__ work)
{
    extern __shared__ float4 smem4[];
    __shared__ unsigned long long bar;
    __shared__ int next;
    float2 *tile = align128(smem4);
    const unsigned bar_sa = (unsigned)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) mbar_init(bar_sa, 1);
    __syncthreads();
    unsigned phase = 0;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(work, 1);
        __syncthreads();
        const int t = next;
        if (t >= ntab) break;
        const int4 e = table[t];
        const BatchInterp &b = vols[e.x];
        const CUtensorMap *tm = (b.tmap_ok >> 3) & 1 ? &b.tmaps[3] : nullptr;
        if (!gather_piece_tab<R>(b.in, b.out, b.nc, e.z, b.blocks[e.y], b.g, b.scale, b.wsample, b.tap_rows,
                                 b.tap_ent, tile, tm, bar_sa, phase, b.status))
            return;
    }
}

template <int CB, bool RADIAL, int R>
__global__ void __launch_bounds__(kInterpThreads)
k_spread_batch(const BatchInterp *__restrict__ vols, const int4 *__restrict__ table, int ntab,
               int *__restrict__ work, KBParams kb)
{
    extern __shared__ float4 smem4[];
    __shared__ float red[32 * CB];
    __shared__ float psc[2 * kMaxCB];
    __shared__ TapQueue2 queues[kInterpThreads / 32];
    __shared__ int next;
    CandPairs cs;
    int *tile = spread_setup<R>(vols[0].cand, cs, smem4, CB);
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(work, 1);
        __syncthreads();
        const int t = next;
        if (t >= ntab) break;
        const int4 e = table[t];
        const BatchInterp &b = vols[e.x];
        spread_piece<CB, RADIAL, R>(b.in, b.out, b.nc, e.z, b.samples, b.blocks[e.y], b.g, kb, cs, tile, red,
                                    psc, queues);
    }
}

// Batched permutes: block -> (volume, chunk of 256 samples).
__global__ void k_perm_batch(const BatchPerm *__restrict__ vols, const int4 *__restrict__ table, int out)
{
    const int4 e = table[blockIdx.x];
    const BatchPerm &b = vols[e.x];
    const int64_t m = (int64_t)e.y * blockDim.x + threadIdx.x;
    if (m >= b.M) return;
    const int s = b.inv[m];
    const int nc = b.nc;
    if (out) {
        for (int c = 0; c < nc; ++c) {
            float2 v = make_float2(0.f, 0.f);
            if (s >= 0) {
                v = b.in[(size_t)s * nc + c];
                v.x *= b.scale;
                v.y *= b.scale;
            }
            b.out[m + b.M * c] = v;
        }
    } else {
        if (s < 0) return;
        const float w = b.w ? b.w[s] : 1.f;
        for (int c = 0; c < nc; ++c) {
            const float2 v = b.in[m + b.M * c];
            b.out[(size_t)s * nc + c] = make_float2(v.x * w, v.y * w);
        }
    }
}

// ---------------------------------------------------------------- host
size_t smem_interp_bytes(const Geom &g, int cb)
{
    return (size_t)g.P[0] * g.P[1] * g.P[2] * cb * sizeof(float2);
}

static const Cand &cand_of(const nufft3d_plan *p) { return p->cand_desc; }

size_t smem_plane_bytes(int R, int cb)
{
    int ps = 0;
    switch (R) {
    case 1: ps = Plane<1>::PS; break;
    case 2: ps = Plane<2>::PS; break;
    case 3: ps = Plane<3>::PS; break;
    default: ps = Plane<4>::PS; break;
    }
    return (size_t)ps * cb * sizeof(float2);
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        else
            cudaGetLastError();
    });
    return fn;
}

// The 4-D map of the grid for the gather's bulk tile copies (box of CB
// coils per point); false where it does not apply (odd nc: row strides must
// be multiples of 16 bytes; single coils: the box row must be 16 bytes or
// more) or the driver refuses it.
template <int CB>
static bool gather_tensor_map(const nufft3d_plan *p, const float2 *G, int nc, CUtensorMap *m)
{
    const Geom &g = p->geom;
    if (CB < 2 || nc % 2) return false;
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t row = (cuuint64_t)nc * sizeof(float2);
    cuuint64_t dim[4] = {(cuuint64_t)2 * nc, (cuuint64_t)g.K[0], (cuuint64_t)g.K[1], (cuuint64_t)g.K[2]};
    cuuint64_t str[3] = {row, row * g.K[0], row * g.K[0] * g.K[1]};
    cuuint32_t box[4] = {2 * CB, (cuuint32_t)g.P[0], (cuuint32_t)g.P[1], (cuuint32_t)g.P[2]};
    cuuint32_t es[4] = {1, 1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float2 *>(G), dim, str, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Encodes the gather tensor map of grid G (nc coils) for chunks of cb
// coils; false where the bulk copy does not apply.
bool encode_gather_map(const nufft3d_plan *p, const float2 *G, int nc, int cb, CUtensorMap *m)
{
    switch (cb) {
    case 2: return gather_tensor_map<2>(p, G, nc, m);
    case 4: return gather_tensor_map<4>(p, G, nc, m);
    case 8: return gather_tensor_map<8>(p, G, nc, m);
    default: return false;
    }
}

int plan_check_status(nufft3d_plan *p, cudaStream_t s)
{
    int v = 0;
    int *flag = p->work + kWorkStatus;
    NUFFT_CUDA_TRY(cudaMemcpyAsync(&v, flag, sizeof(v), cudaMemcpyDeviceToHost, s));
    NUFFT_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), s));
    NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    if (!v) return NUFFT3D_SUCCESS;
    return fail(NUFFT3D_ERR_TIMEOUT, "a tile copy in the interpolation did not complete in time");
}

InterpStatus plan_status(const nufft3d_plan *p) { return InterpStatus{p->work + kWorkStatus, p->wait_polls}; }

int interp_grid_sms(const nufft3d_plan *p);

template <int CB, bool RADIAL, int R>
static int gather_t(nufft3d_plan *p, const float2 *G, float2 *ks, int nc, int c0, float scale,
                    const float *ws, cudaStream_t s)
{
    // + 128: the tile is aligned to 128 bytes for the bulk copies
    const size_t smem = smem_plane_bytes(R, CB) + cand_smem_bytes(p->n_cand) + 128;
    alignas(64) CUtensorMap m;
    std::memset(&m, 0, sizeof(m));
    const int use_tma = p->use_tma && gather_tensor_map<CB>(p, G, nc, &m) ? 1 : 0;
    NUFFT_CUDA_TRY(cudaMemsetAsync(p->work, 0, sizeof(int), s));
    const int64_t grid = std::min<int64_t>(p->n_blocks, interp_grid_sms(p));
    k_gather<CB, RADIAL, R><<<(unsigned)grid, kInterpThreads, smem, s>>>(
        G, ks, nc, c0, p->samples, p->blocks, (int)p->n_blocks, p->work, p->geom, p->kb, scale, ws, cand_of(p), m,
        use_tma, plan_status(p));
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

template <int CB, bool RADIAL, int R>
static int spread_t(nufft3d_plan *p, const float2 *ks, float2 *G, int nc, int c0, cudaStream_t s)
{
    const size_t smem = (size_t)IPlane<R>::PS * CB * 2 * sizeof(int) + cand_pairs_bytes(p->cand_desc);
    NUFFT_CUDA_TRY(cudaMemsetAsync(p->work + 1, 0, sizeof(int), s));
    const int64_t grid = std::min<int64_t>(p->n_blocks, interp_grid_sms(p));
    k_spread<CB, RADIAL, R><<<(unsigned)grid, kInterpThreads, smem, s>>>(
        ks, G, nc, c0, p->samples, p->blocks, (int)p->n_blocks, p->work + 1, p->geom, p->kb, cand_of(p));
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

int interp_grid_sms(const nufft3d_plan *p)
{
    return p->interp_sms > 0 && p->interp_sms < p->sm_count ? p->interp_sms : p->sm_count;
}

bool tap_table_applies(const nufft3d_plan *p) { return p->coils_per_pass == 8 && p->geom.R <= 3; }

template <int R>
static int gather_tab_t(nufft3d_plan *p, const float2 *G, float2 *ks, int nc, int c0, float scale,
                        const float *ws, cudaStream_t s)
{
    const size_t smem = smem_plane_bytes(R, 8) + 128;
    alignas(64) CUtensorMap m;
    std::memset(&m, 0, sizeof(m));
    const int use_tma = p->use_tma && gather_tensor_map<8>(p, G, nc, &m) ? 1 : 0;
    NUFFT_CUDA_TRY(cudaMemsetAsync(p->work, 0, sizeof(int), s));
    const int64_t grid = std::min<int64_t>(p->n_blocks, interp_grid_sms(p));
    k_gather_tab<R><<<(unsigned)grid, kInterpThreads, smem, s>>>(G, ks, nc, c0, p->blocks, (int)p->n_blocks,
                                                                 p->work, p->geom, scale, ws, p->tap_rows,
                                                                 p->tap_ent, m, use_tma, plan_status(p));
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

// 8-coil gather passes of a plan with the stored H
static int gather_tab(nufft3d_plan *p, const float2 *in, float2 *out, int nc, int c0, float scale,
                      const float *ws, cudaStream_t s)
{
    switch (p->geom.R) {
    case 1: return gather_tab_t<1>(p, in, out, nc, c0, scale, ws, s);
    case 2: return gather_tab_t<2>(p, in, out, nc, c0, scale, ws, s);
    case 3: return gather_tab_t<3>(p, in, out, nc, c0, scale, ws, s);
    default: return fail(NUFFT3D_ERR_UNSUPPORTED, "stored H with R > 3");
    }
}

template <bool GATHER, int CB, bool RADIAL>
static int dispatch_r(nufft3d_plan *p, const float2 *in, float2 *out, int nc, int c0, float scale,
                      const float *ws, cudaStream_t s)
{
    switch (p->geom.R) {
    case 1: return GATHER ? gather_t<CB, RADIAL, 1>(p, in, out, nc, c0, scale, ws, s)
                          : spread_t<CB, RADIAL, 1>(p, in, out, nc, c0, s);
    case 2: return GATHER ? gather_t<CB, RADIAL, 2>(p, in, out, nc, c0, scale, ws, s)
                          : spread_t<CB, RADIAL, 2>(p, in, out, nc, c0, s);
    case 3: return GATHER ? gather_t<CB, RADIAL, 3>(p, in, out, nc, c0, scale, ws, s)
                          : spread_t<CB, RADIAL, 3>(p, in, out, nc, c0, s);
    default:
        if (CB == 8) return fail(NUFFT3D_ERR_UNSUPPORTED, "8 coils per pass do not fit with R=4 tiles");
        return GATHER ? gather_t<(CB < 8 ? CB : 4), RADIAL, 4>(p, in, out, nc, c0, scale, ws, s)
                      : spread_t<(CB < 8 ? CB : 4), RADIAL, 4>(p, in, out, nc, c0, s);
    }
}

template <bool GATHER, int CB>
static int dispatch(nufft3d_plan *p, const float2 *in, float2 *out, int nc, int c0, float scale,
                    const float *ws, cudaStream_t s)
{
    return p->geom.radial ? dispatch_r<GATHER, CB, true>(p, in, out, nc, c0, scale, ws, s)
                          : dispatch_r<GATHER, CB, false>(p, in, out, nc, c0, scale, ws, s);
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
        case 1: st = dispatch<GATHER, 1>(p, in, out, nc, c0, scale, ws, s); break;
        case 2: st = dispatch<GATHER, 2>(p, in, out, nc, c0, scale, ws, s); break;
        case 4: st = dispatch<GATHER, 4>(p, in, out, nc, c0, scale, ws, s); break;
        default:
            // the stored H serves the gather and the stored H' the spread
            // (full passes of an even coil count), else the kernel is evaluated
            if (GATHER && p->tap_ent)
                st = gather_tab(p, in, out, nc, c0, scale, ws, s);
            else if (!GATHER && spread_tab_applies(p, nc, c0))
                st = launch_spread_tab(p, in, out, nc, c0, s);
            else
                st = dispatch<GATHER, 8>(p, in, out, nc, c0, scale, ws, s);
            break;
        }
        if (st != NUFFT3D_SUCCESS) return st;
        if (cb > rem) break;
    }
    return NUFFT3D_SUCCESS;
}

int launch_weight_sum(nufft3d_plan *p, cudaStream_t s)
{
    if (p->n_blocks == 0) return NUFFT3D_SUCCESS;
    const size_t smem = smem_interp_bytes(p->geom, 1) / 2 + cand_smem_bytes(p->n_cand);
    if (p->geom.radial)
        k_weight_sum<true><<<(unsigned)p->n_blocks, kInterpThreads, smem, s>>>(p->samples, p->blocks, p->geom,
                                                                            p->kb, cand_of(p));
    else
        k_weight_sum<false><<<(unsigned)p->n_blocks, kInterpThreads, smem, s>>>(p->samples, p->blocks, p->geom,
                                                                             p->kb, cand_of(p));
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

int launch_tap_count(nufft3d_plan *p, uint32_t *rows, cudaStream_t s)
{
    if (p->nnz == 0) return NUFFT3D_SUCCESS;
    const size_t smem = cand_smem_bytes(p->n_cand);
    const unsigned nb = (unsigned)std::min<int64_t>((p->nnz + 7) / 8, (int64_t)p->sm_count * 8);
    if (p->geom.radial)
        k_tap_count<true><<<nb, 256, smem, s>>>(p->samples, p->nnz, p->geom, p->kb, cand_of(p), rows);
    else
        k_tap_count<false><<<nb, 256, smem, s>>>(p->samples, p->nnz, p->geom, p->kb, cand_of(p), rows);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

int launch_tap_fill(nufft3d_plan *p, const uint32_t *rows, int2 *taps, cudaStream_t s)
{
    if (p->nnz == 0) return NUFFT3D_SUCCESS;
    int *err = p->work + kWorkTapFill;  // the plan's own flag (plans may be built concurrently)
    NUFFT_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    int cap = 0;
    for (int q = 0; q < 8; ++q) cap = std::max(cap, p->cand_desc.cnt[q]);
    const size_t smem = cand_smem_bytes(p->n_cand) + (size_t)8 * 2 * cap * sizeof(int2);
    if (smem > 200 * 1024) return fail(NUFFT3D_ERR_UNSUPPORTED, "candidate lists too long for the stored H");
    const unsigned nb = (unsigned)std::min<int64_t>((p->nnz + 7) / 8, (int64_t)p->sm_count * 8);
    if (p->geom.radial)
        k_tap_fill<true><<<nb, 256, smem, s>>>(p->samples, p->nnz, p->geom, p->kb, cand_of(p), rows, taps, cap, err);
    else
        k_tap_fill<false><<<nb, 256, smem, s>>>(p->samples, p->nnz, p->geom, p->kb, cand_of(p), rows, taps, cap, err);
    NUFFT_CUDA_TRY(cudaGetLastError());
    int herr = 0;
    NUFFT_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr) return fail(NUFFT3D_ERR_CUDA, "stored H: fill pass disagrees with the count pass");
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


template <int CB, bool RADIAL, int R>
static int interp_batch_t(bool gather, const BatchInterp *vols, const int4 *table, int nblocks, size_t smem,
                          const KBParams &kb, int *work, int nsm, cudaStream_t s)
{
    NUFFT_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(int), s));
    const int grid = nblocks < nsm ? nblocks : nsm;
    if (gather)
        k_gather_batch<CB, RADIAL, R><<<grid, kInterpThreads, smem, s>>>(vols, table, nblocks, work, kb);
    else
        k_spread_batch<CB, RADIAL, R><<<grid, kInterpThreads, smem, s>>>(vols, table, nblocks, work, kb);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

template <int CB, bool RADIAL>
static int interp_batch_r(bool gather, int R, const BatchInterp *vols, const int4 *table, int nblocks, size_t smem,
                          const KBParams &kb, int *work, int nsm, cudaStream_t s)
{
    switch (R) {
    case 1: return interp_batch_t<CB, RADIAL, 1>(gather, vols, table, nblocks, smem, kb, work, nsm, s);
    case 2: return interp_batch_t<CB, RADIAL, 2>(gather, vols, table, nblocks, smem, kb, work, nsm, s);
    case 3: return interp_batch_t<CB, RADIAL, 3>(gather, vols, table, nblocks, smem, kb, work, nsm, s);
    default: return interp_batch_t<(CB < 8 ? CB : 4), RADIAL, 4>(gather, vols, table, nblocks, smem, kb, work, nsm, s);
    }
}

int launch_interp_batch(bool gather, int cb, int R, bool radial, const BatchInterp *vols, const int4 *table,
                        int nblocks, size_t smem, const KBParams &kb, int *work, int nsm, cudaStream_t s,
                        bool stored_h)
{
    if (nblocks <= 0) return NUFFT3D_SUCCESS;
    if (gather && cb >= 8 && stored_h && R <= 3) {
        NUFFT_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(int), s));
        const int grid = nblocks < nsm ? nblocks : nsm;
        const size_t sm = smem_plane_bytes(R, 8) + 128;
        switch (R) {
        case 1: k_gather_batch_tab<1><<<grid, kInterpThreads, sm, s>>>(vols, table, nblocks, work); break;
        case 2: k_gather_batch_tab<2><<<grid, kInterpThreads, sm, s>>>(vols, table, nblocks, work); break;
        default: k_gather_batch_tab<3><<<grid, kInterpThreads, sm, s>>>(vols, table, nblocks, work); break;
        }
        NUFFT_CUDA_TRY(cudaGetLastError());
        return NUFFT3D_SUCCESS;
    }
    if (cb >= 8) return radial ? interp_batch_r<8, true>(gather, R, vols, table, nblocks, smem, kb, work, nsm, s)
                               : interp_batch_r<8, false>(gather, R, vols, table, nblocks, smem, kb, work, nsm, s);
    if (cb >= 4) return radial ? interp_batch_r<4, true>(gather, R, vols, table, nblocks, smem, kb, work, nsm, s)
                               : interp_batch_r<4, false>(gather, R, vols, table, nblocks, smem, kb, work, nsm, s);
    if (cb >= 2) return radial ? interp_batch_r<2, true>(gather, R, vols, table, nblocks, smem, kb, work, nsm, s)
                               : interp_batch_r<2, false>(gather, R, vols, table, nblocks, smem, kb, work, nsm, s);
    return radial ? interp_batch_r<1, true>(gather, R, vols, table, nblocks, smem, kb, work, nsm, s)
                  : interp_batch_r<1, false>(gather, R, vols, table, nblocks, smem, kb, work, nsm, s);
}

int launch_perm_batch(bool out, const BatchPerm *vols, const int4 *table, int nblocks, cudaStream_t s)
{
    if (nblocks <= 0) return NUFFT3D_SUCCESS;
    k_perm_batch<<<nblocks, 256, 0, s>>>(vols, table, out ? 1 : 0);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

// Allow each kernel all the shared memory a block can have, less its static part.
template <typename K>
static int allow_smem(K kernel)
{
    cudaFuncAttributes fa;
    NUFFT_CUDA_TRY(cudaFuncGetAttributes(&fa, kernel));
    const int mx = 227 * 1024 - (int)fa.sharedSizeBytes;
    NUFFT_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    return NUFFT3D_SUCCESS;
}

template <int CB, bool RADIAL, int R>
static int cfg_one()
{
    NUFFT_TRY(allow_smem(k_gather<CB, RADIAL, R>));
    NUFFT_TRY(allow_smem(k_spread<CB, RADIAL, R>));
    NUFFT_TRY(allow_smem(k_gather_batch<CB, RADIAL, R>));
    NUFFT_TRY(allow_smem(k_spread_batch<CB, RADIAL, R>));
    return NUFFT3D_SUCCESS;
}

template <int CB, bool RADIAL>
static int cfg_r()
{
    NUFFT_TRY((cfg_one<CB, RADIAL, 1>()));
    NUFFT_TRY((cfg_one<CB, RADIAL, 2>()));
    NUFFT_TRY((cfg_one<CB, RADIAL, 3>()));
    NUFFT_TRY((cfg_one<(CB < 8 ? CB : 4), RADIAL, 4>()));
    return NUFFT3D_SUCCESS;
}

template <int CB>
static int cfg_cb()
{
    NUFFT_TRY((cfg_r<CB, true>()));
    NUFFT_TRY((cfg_r<CB, false>()));
    return NUFFT3D_SUCCESS;
}

int configure_interp_kernels()
{
    NUFFT_TRY(allow_smem(k_weight_sum<true>));
    NUFFT_TRY(allow_smem(k_weight_sum<false>));
    NUFFT_TRY(allow_smem(k_tap_count<true>));
    NUFFT_TRY(allow_smem(k_tap_count<false>));
    NUFFT_TRY(allow_smem(k_tap_fill<true>));
    NUFFT_TRY(allow_smem(k_tap_fill<false>));
    NUFFT_TRY(allow_smem(k_gather_batch_tab<1>));
    NUFFT_TRY(allow_smem(k_gather_batch_tab<2>));
    NUFFT_TRY(allow_smem(k_gather_batch_tab<3>));
    NUFFT_TRY(allow_smem(k_gather_tab<1>));
    NUFFT_TRY(allow_smem(k_gather_tab<2>));
    NUFFT_TRY(allow_smem(k_gather_tab<3>));
    NUFFT_TRY(cfg_cb<1>());
    NUFFT_TRY(cfg_cb<2>());
    NUFFT_TRY(cfg_cb<4>());
    NUFFT_TRY(cfg_cb<8>());
    return NUFFT3D_SUCCESS;
}

} // namespace nufft3d
