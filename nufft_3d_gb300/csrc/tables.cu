// Spread (aNUFT's H' product, spmv_t of nufft_3d.m:274-282) from a stored
// transpose of H, for 8-coil passes.
//
// The reference multiplies by the transpose of its sparse H through cuSPARSE
// (and on its CPU path keeps HT = H' as a matrix of its own, nufft_3d.m:218-219,
// so that the product reads a matrix laid out for it; this is that table for
// the GPU).  The on-the-fly spread (interp.cu) scatters each sample's taps into a tile
// with shared-memory integer reductions, which bounds it by instruction issue
// and the reduction pipe.  This form turns the product around: the samples of
// a tile piece are staged in shared memory, and each grid point of the
// piece's padded tile (tile plus halo) owns a row of (sample, weight) entries
// -- H' restricted to the piece.  Two lanes (four coils each) walk a row,
// accumulate the grid point's 8 coils in registers with FP32 FMAs, and add
// the finished point to the grid with two 16-byte vector atomics each
// (neighbouring pieces' halos overlap).  No shared-memory atomics, no kernel
// evaluation, and FP32 accumulation throughout.
//
// Stored H' layout, per spread piece (at most kSpreadCap samples of one
// tile, so that their 8 coils fit in shared memory):
//   * the piece's non-empty rows are sorted by length (longest first, ties
//     by grid point) and taken 16 at a time into bundles; a bundle is a run
//     of 256-byte lines, one 16-byte unit per row slot (row slot r = lanes
//     2r, 2r+1 of a warp), so a warp walks 16 rows in lockstep and every
//     branch on the bundle structure is warp-uniform;
//   * line 0 of a bundle is its header: per row slot int4 (B, y, 0, 0) with
//     B the bundle's body lines and y = -1 - (grid point index), or 0 for a
//     slot without a row (the last bundle of a piece);
//   * each body line holds two entries per row slot, int2 (weight bits,
//     byte offset of the sample's 64-byte slot in the staged samples: local
//     index + 2; slots 0 and 1 stay zero and serve as padding);
//   * inside a row, even-slot and odd-slot samples alternate, starting with
//     the parity of the row slot, so neighbouring rows of a quarter-warp
//     (4 rows) read samples in different halves of the shared-memory banks;
//     leftovers of the larger parity and padding (weight 0) follow;
//   * the piece's lines are laid out in 32 runs of equal length, one per
//     warp (a bundle that does not fit in what is left of a run is cut, its
//     rest continuing in the next run behind a header of its own):
//     wstart[33 * piece + w] is warp w's first line.
// Inside a row each parity's samples keep their sorted order, interleaved by
// a fixed rule (the fill is deterministic), so a row's FP32 sum does not
// depend on scheduling.
//
// The table is built from the stored H (same weights, same support test)
// once per plan: a count pass gives each piece's lines, the host scans them,
// and a fill pass writes the bundles.
#include <cub/block/block_radix_sort.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "internal.h"

namespace nufft3d {

// Bundles: kRows rows walked by one warp in lockstep, lane (r, h) =
// (lane / 2, lane % 2) owning row slot r and coils 4h..4h+3.  Rows are stored
// as runs of lines, one 16-byte unit per row slot: a header line
// int4 (B, y, 0, 0) per slot (B body lines follow; y = -1 - the row's grid
// point, 0 for an empty slot), then B body lines holding two entries
// int2 (weight bits, byte offset into the staged samples) per slot.  Each
// warp streams a run of whole lines; runs hold a whole number of pipeline
// steps (empty headers, B = 0, fill the rest) and the stream ends with
// kBundleDepth spare empty lines, so the line loop needs no bounds test.
constexpr int kBundleWarps = 32;   // warps per block of the spread (1024 threads)
constexpr int kRows = 16;          // row slots of a bundle: two lanes per row, four coils per lane
constexpr int kLineInt4 = kRows;   // 16-byte units of a line
constexpr int kLineBytes = 16 * kRows;
constexpr int kBundleDepth = 4;    // lines each lane keeps in flight
// Lines of a warp's run that lane 0 asks L2 to fetch ahead of the register
// loads (kPrefetchAhead lines ahead, kPrefetchLines at a time), so that the
// loads wait on L2 rather than on DRAM.
constexpr int kPrefetchLines = 8;
constexpr int kPrefetchAhead = 24;

__device__ __forceinline__ void prefetch_l2(const int4 *lines, uint32_t l, uint32_t l_hi)
{
    if (l >= l_hi) return;
    const uint32_t n = min((uint32_t)kPrefetchLines, l_hi - l);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lines + (size_t)l * kLineInt4),
                 "r"(n * (uint32_t)kLineBytes)
                 : "memory");
}

// Streaming 16-byte load of table entries (read once: no L1 allocation).
__device__ __forceinline__ int4 ld_ent4(const int4 *p)
{
    int4 v;
    asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

// acc0, acc1 (a coil pair) += w * the 16 bytes at byte offset y of base
// (a 16-byte shared load, two packed FP32x2 FMAs)
__device__ __forceinline__ void bundle_apply(const char *base_q, int wbits, int y, float2 &acc0, float2 &acc1)
{
    const float4 v = *reinterpret_cast<const float4 *>(base_q + y);
    const float2 ww = make_float2(__int_as_float(wbits), __int_as_float(wbits));
    acc0 = __ffma2_rn(ww, make_float2(v.x, v.y), acc0);
    acc1 = __ffma2_rn(ww, make_float2(v.z, v.w), acc1);
}

constexpr int kTabBuildThreads = 256;
constexpr int kTabBuildWarps = kTabBuildThreads / 32;
constexpr int kTabSortItems = 11;  // 256 x 11 >= 14^3 padded-tile points
constexpr int kSpreadThreads = 1024;
constexpr int kSpreadWarps = kBundleWarps;
constexpr int kSpreadDepth = kBundleDepth;
constexpr int kMaxBundles = (kTabBuildThreads * kTabSortItems + kRows - 1) / kRows;

// Origin of the padded tile of tile index tid (may be negative or past the
// grid edge: the grid wraps around).
__device__ __forceinline__ void tab_tile_origin(const Geom &g, int tid, int &ox, int &oy, int &oz)
{
    const int tx = tid % g.nt[0];
    const int ty = (tid / g.nt[0]) % g.nt[1];
    const int tz = tid / (g.nt[0] * g.nt[1]);
    ox = tx * g.T[0] - g.Ra[0];
    oy = ty * g.T[1] - g.Ra[1];
    oz = tz * g.T[2] - g.Ra[2];
}

__device__ __forceinline__ int tab_wrap(int x, int K)
{
    x %= K;
    return x < 0 ? x + K : x;
}

// Warp runs of a piece's bundles, of equal capacity (a whole number of
// pipeline steps): the bundles are laid out one after the other; a bundle
// that does not fit in what is left of a run is cut, and its rest continues
// in the next run behind a header of its own (both parts add their partial
// sums to the output), so every warp streams about as many lines as the
// others.  Space left at the end of a run holds empty headers (B = 0).
template <int MAXB>
struct RunLayout {
    uint32_t bl[MAXB];                       // body lines of each bundle
    uint16_t fs[MAXB + 1];                   // first segment of each bundle
    uint16_t seg_i0[MAXB + 2 * kBundleWarps];  // a segment: body lines [i0, i0 + n) of its bundle
    uint16_t seg_n[MAXB + 2 * kBundleWarps];
    uint32_t seg_line[MAXB + 2 * kBundleWarps];  // the segment's header line (piece-relative)
    uint32_t wbase[kBundleWarps + 1];        // first line of each warp's run
    uint32_t wused[kBundleWarps];            // lines of each run before its padding
};

// Lays out nb bundles (bl set); one thread.
template <int MAXB>
__device__ void layout_runs(RunLayout<MAXB> &L, int nb)
{
    uint32_t T = 0;
    for (int k = 0; k < nb; ++k) T += 1u + L.bl[k];
    const uint32_t C =
        (T + kBundleWarps + kBundleWarps * kBundleDepth - 1) / (kBundleWarps * kBundleDepth) * kBundleDepth;
    int w = 0, ns = 0;
    uint32_t used = 0;
    for (int k = 0; k < nb; ++k) {
        L.fs[k] = (uint16_t)ns;
        uint32_t rem = L.bl[k], i0 = 0;
        while (rem > 0) {
            const uint32_t space = w < kBundleWarps - 1 ? C - used : 0xFFFFFFFFu;  // the last run grows
            if (space < 2u) {
                L.wused[w] = used;
                ++w;
                used = 0;
                continue;
            }
            const uint32_t n = min(rem, space - 1u);
            L.seg_i0[ns] = (uint16_t)i0;
            L.seg_n[ns] = (uint16_t)n;
            L.seg_line[ns] = (uint32_t)w * C + used;
            ++ns;
            used += 1u + n;
            rem -= n;
            i0 += n;
        }
    }
    L.fs[nb] = (uint16_t)ns;
    for (; w < kBundleWarps; ++w) {
        L.wused[w] = used;
        used = 0;
    }
    for (int v = 0; v < kBundleWarps; ++v) L.wbase[v] = (uint32_t)v * C;
    const uint32_t last = L.wused[kBundleWarps - 1];
    L.wbase[kBundleWarps] =
        (uint32_t)(kBundleWarps - 1) * C + max(C, (last + kBundleDepth - 1) / kBundleDepth * kBundleDepth);
}

// Piece-relative line of body line i of bundle k.
template <int MAXB>
__device__ __forceinline__ uint32_t body_line(const RunLayout<MAXB> &L, int k, uint32_t i)
{
    int sg = L.fs[k];
    while (sg + 1 < (int)L.fs[k + 1] && i >= (uint32_t)L.seg_i0[sg] + L.seg_n[sg]) ++sg;
    return L.seg_line[sg] + 1u + (i - L.seg_i0[sg]);
}

// Empty headers after each run's bundles.
template <int MAXB>
__device__ void pad_runs(const RunLayout<MAXB> &L, uint32_t base, int4 *ent4)
{
    for (int w = 0; w < kBundleWarps; ++w) {
        const uint32_t l0 = L.wbase[w] + L.wused[w], l1 = L.wbase[w + 1];
        for (uint32_t i = threadIdx.x; i < (l1 - l0) * (uint32_t)kLineInt4; i += blockDim.x)
            ent4[((size_t)base + l0) * kLineInt4 + i] = make_int4(0, 0, 0, 0);
    }
}

using TabSort = cub::BlockRadixSort<uint32_t, kTabBuildThreads, kTabSortItems>;

struct TabBuildSmem {
    typename TabSort::TempStorage sort;
    RunLayout<kMaxBundles> L;
    uint16_t srow[kTabBuildThreads * kTabSortItems];  // point of each sorted row
    int nrows;
};

// Plan time, one block per spread piece.  FILL = false: writes the piece's
// line count to lines_out[b].  FILL = true: writes the piece's bundles from
// line pieces[b].w on and the warps' first lines to wstart[33 b ..].
// Dynamic shared memory: per-warp packed counts [warps][P] (even-slot count
// | odd-slot count << 16), the row totals [P] and each point's row rank [P].
// Warp w takes a contiguous run of the piece's samples, one sample at a time
// (a sample's taps are distinct points, so its lanes never update the same
// counter), which makes each row's entries come out in sample order.
template <bool FILL>
__global__ void __launch_bounds__(kTabBuildThreads)
k_spread_tab_build(const int4 *__restrict__ pieces, const uint32_t *__restrict__ rows,
                   const int2 *__restrict__ taps, Geom g, uint32_t *__restrict__ lines_out,
                   uint32_t *__restrict__ wstart, int2 *__restrict__ ent)
{
    extern __shared__ uint32_t sm[];
    __shared__ TabBuildSmem ss;
    const int P = g.P[0] * g.P[1] * g.P[2];
    uint32_t *hist = sm;
    uint32_t *tot = sm + kTabBuildWarps * P;
    uint32_t *rank = tot + P;  // row rank of point p (sorted order), or ~0u
    const int4 pc = pieces[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < kTabBuildWarps * P; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const int s_lo = pc.y + (int)(((long long)pc.z * warp) / kTabBuildWarps);
    const int s_hi = pc.y + (int)(((long long)pc.z * (warp + 1)) / kTabBuildWarps);
    uint32_t *h = hist + (size_t)warp * P;
    for (int s = s_lo; s < s_hi; ++s) {
        const size_t r0 = (size_t)__ldg(&rows[s]) * 8, r1 = (size_t)__ldg(&rows[s + 1]) * 8;
        const uint32_t inc = ((s - pc.y) & 1) ? 0x10000u : 1u;
        for (size_t e = r0 + lane; e < r1; e += 32) {
            const int2 t = __ldg(&taps[e]);
            if (t.x != 0) h[t.y] += inc;  // padding entries have weight 0
        }
        __syncwarp();
    }
    __syncthreads();
    // per point: exclusive prefix over the warps and the row's total
    for (int p = tid; p < P; p += blockDim.x) {
        uint32_t acc = 0;
        for (int w = 0; w < kTabBuildWarps; ++w) {
            const uint32_t v = hist[(size_t)w * P + p];
            hist[(size_t)w * P + p] = acc;
            acc += v;
        }
        tot[p] = acc;
    }
    __syncthreads();
    // rows by length, longest first, ties by point: key (4095 - L) << 12 | p
    uint32_t key[kTabSortItems];
#pragma unroll
    for (int i = 0; i < kTabSortItems; ++i) {
        const int p = tid * kTabSortItems + i;
        uint32_t k = 0xFFFFFFFFu;
        if (p < P) {
            const uint32_t a = tot[p], L = (a & 0xFFFFu) + (a >> 16);
            k = ((4095u - L) << 12) | (uint32_t)p;
        }
        key[i] = k;
    }
    if (tid == 0) ss.nrows = 0;
    __syncthreads();  // (tot is read above; nrows is counted below)
    TabSort(ss.sort).Sort(key, 0, 24);
    // blocked arrangement: thread t holds sorted positions t*items + i; the
    // rows (points with entries) come first
#pragma unroll
    for (int i = 0; i < kTabSortItems; ++i) {
        const uint32_t k = key[i];
        if (k == 0xFFFFFFFFu) continue;
        const bool row = (k >> 12) != 4095u;
        rank[k & 0xFFFu] = row ? (uint32_t)(tid * kTabSortItems + i) : 0xFFFFFFFFu;
        if (row) {
            ss.srow[tid * kTabSortItems + i] = (uint16_t)(k & 0xFFFu);
            atomicAdd(&ss.nrows, 1);
        }
    }
    __syncthreads();
    const int nr = ss.nrows, nb = (nr + kRows - 1) / kRows;
    // bundle lengths: a bundle's first row is its longest
    for (int p = tid; p < P; p += blockDim.x) {
        const uint32_t r = rank[p];
        if (r != 0xFFFFFFFFu && r % kRows == 0) {
            const uint32_t a = tot[p], L = (a & 0xFFFFu) + (a >> 16);
            ss.L.bl[r / kRows] = (L + 1u) / 2u;  // body lines
        }
    }
    __syncthreads();
    if (tid == 0) layout_runs(ss.L, nb);
    __syncthreads();
    const uint32_t nlines = ss.L.wbase[kSpreadWarps];
    if (!FILL) {
        if (tid == 0) lines_out[blockIdx.x] = nlines;
        return;
    }
    const uint32_t base = (uint32_t)pc.w;
    if (tid <= kSpreadWarps) wstart[(size_t)blockIdx.x * (kSpreadWarps + 1) + tid] = base + ss.L.wbase[tid];
    int4 *ent4 = reinterpret_cast<int4 *>(ent);
    pad_runs(ss.L, base, ent4);
    // entry j of row slot r of bundle k: its body line j/2 lies in one of the
    // bundle's segments, behind that segment's header
    auto at = [&](int k, int r, uint32_t j) -> size_t {
        return (((size_t)base + body_line(ss.L, k, j / 2u)) * kLineInt4 + (size_t)r) * 2u + (j & 1u);
    };
    // headers of every segment (grid point of each row slot, or 0 for a slot
    // without a row in the last bundle)
    int ox, oy, oz;
    tab_tile_origin(g, pc.x, ox, oy, oz);
    for (int i = tid; i < nb * kRows; i += blockDim.x) {
        const int k = i / kRows, r = i % kRows;
        int y = 0;
        if (i < nr) {
            const int p = ss.srow[i];
            const int lx = p % g.P[0], ly = (p / g.P[0]) % g.P[1], lz = p / (g.P[0] * g.P[1]);
            const long long gi = ((long long)tab_wrap(oz + lz, g.K[2]) * g.K[1] + tab_wrap(oy + ly, g.K[1])) *
                                     g.K[0] + tab_wrap(ox + lx, g.K[0]);
            y = (int)(-1 - gi);
        }
        for (int sg = ss.L.fs[k]; sg < (int)ss.L.fs[k + 1]; ++sg)
            ent4[((size_t)base + ss.L.seg_line[sg]) * kLineInt4 + r] = make_int4((int)ss.L.seg_n[sg], y, 0, 0);
        // padding of the row (weight 0, alternating zero slots) up to the bundle's length
        uint32_t L = 0;
        if (i < nr) {
            const uint32_t a = tot[ss.srow[i]];
            L = (a & 0xFFFFu) + (a >> 16);
        }
        for (uint32_t j = L; j < 2u * ss.L.bl[k]; ++j) ent[at(k, r, j)] = make_int2(0, 64 * (int)((j + r) & 1u));
    }
    // the entries: row slot r starts with parity r & 1, then alternates while
    // both parities last; leftovers follow in sample order
    for (int s = s_lo; s < s_hi; ++s) {
        const int sl = s - pc.y, par = sl & 1;
        const uint32_t inc = par ? 0x10000u : 1u;
        const size_t r0 = (size_t)__ldg(&rows[s]) * 8, r1 = (size_t)__ldg(&rows[s + 1]) * 8;
        for (size_t e = r0 + lane; e < r1; e += 32) {
            const int2 t = __ldg(&taps[e]);
            if (t.x == 0) continue;
            const int p = t.y;
            const uint32_t hv = h[p];
            h[p] = hv + inc;
            const uint32_t rk = par ? hv >> 16 : hv & 0xFFFFu;
            const uint32_t a = tot[p], m = min(a & 0xFFFFu, a >> 16);
            const uint32_t rr = rank[p];
            const int k = (int)(rr / kRows), r = (int)(rr % kRows);
            const uint32_t j = rk < m ? 2u * rk + (uint32_t)(par != (r & 1)) : 2u * m + (rk - m);
            ent[at(k, r, j)] = make_int2(t.x, (sl + 2) * 64);
        }
        __syncwarp();
    }
}

// Stage the samples of a piece into one of the two sample buffers (slot
// 2 + i holds sorted sample first + i) with asynchronous copies; the caller
// waits for them (cp.async.wait_all) and synchronises before reading.
__device__ __forceinline__ void stage_samples(const float2 *__restrict__ ks, int nc, int c0, int first, int n,
                                              unsigned buf_sa)
{
    for (int i = threadIdx.x; i < n * 4; i += blockDim.x) {
        const int sl = i >> 2, pr = i & 3;
        const float2 *src = ks + (size_t)(first + sl) * nc + c0 + 2 * pr;
        const unsigned dst = buf_sa + (unsigned)((sl + 2) * 64 + pr * 16);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// The spread.  Persistent blocks (one per SM) take spread pieces from a work
// counter, one piece ahead: while a piece is applied from one sample buffer,
// the next piece's samples land in the other (64-byte slots of 8 coils), and
// each warp's first lines of the next piece are loaded into its pipeline
// before the piece barrier.  Warp w streams its run of bundle lines: lane
// (r, h) reads row slot r's 16-byte unit of each line and applies its two
// entries to coils 4h..4h+3 (two 16-byte shared loads and four packed FP32x2
// FMAs each); after a bundle's last line every lane adds its four coils of
// its row's grid point to the grid.  Runs hold a whole number of pipeline
// steps and the stream ends with spare empty lines, so the loads need no
// bounds test.  Requires nc even and a full pass of 8 coils (c0 + 8 <= nc).
__global__ void __launch_bounds__(kSpreadThreads)
k_spread_tab(const float2 *__restrict__ ks, float2 *__restrict__ G, int nc, int c0,
             const int4 *__restrict__ pieces, int npieces, int *__restrict__ work,
             const uint32_t *__restrict__ wstart, const int4 *__restrict__ lines)
{
    extern __shared__ float4 ys[];  // two buffers of kSpreadCap + 2 slots; slots 0 and 1 stay zero
    __shared__ int next;
    constexpr int kBufF4 = (kSpreadCap + 2) * 4;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // lane (r, h): row slot r, coils 4h..4h+3 as two 16-byte halves; rows 2
    // and 3 of every 4 take their halves in the other order, so the 8 lanes
    // of a quarter-warp (4 rows, alternate sample parities) read 8 distinct
    // 16-byte bank groups in each load
    const int r = lane >> 1, h = lane & 1;
    const int o1 = 16 * ((r >> 1) & 1), o2 = 16 - o1;  // byte offsets of this lane's first and second load
    if (tid < 8) {
        ys[tid] = make_float4(0.f, 0.f, 0.f, 0.f);
        ys[kBufF4 + tid] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const unsigned ys_sa = (unsigned)__cvta_generic_to_shared(ys);
    float2 *G1 = G + c0 + 4 * h + o1 / 8, *G2 = G + c0 + 4 * h + o2 / 8;  // coil pairs of the two loads
    const int4 *lr = lines + r;  // this lane's row slot of every line
    if (tid == 0) next = atomicAdd(work, 1);
    __syncthreads();
    int b = next;
    int4 e[kSpreadDepth];
    uint32_t l_lo = 0, l_hi = 0;
    if (b < npieces) {
        const int4 pc = pieces[b];
        stage_samples(ks, nc, c0, pc.y, pc.z, ys_sa);
        l_lo = __ldg(&wstart[(size_t)b * (kSpreadWarps + 1) + warp]);
        l_hi = __ldg(&wstart[(size_t)b * (kSpreadWarps + 1) + warp + 1]);
#pragma unroll
        for (int k = 0; k < kSpreadDepth; ++k) e[k] = ld_ent4(lr + (size_t)(l_lo + k) * kLineInt4);
    }
    int buf = 0;
    while (b < npieces) {
        __syncthreads();  // every thread has read `next`
        if (tid == 0) next = atomicAdd(work, 1);
        if (lane == 0)
            for (int k = 0; k < kPrefetchAhead + kPrefetchLines; k += kPrefetchLines)
                prefetch_l2(lines, l_lo + kSpreadDepth + k, l_hi);
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();  // this piece's samples are in, `next` is set
        const int bn = next;
        if (bn < npieces) {
            const int4 pn = pieces[bn];
            stage_samples(ks, nc, c0, pn.y, pn.z, ys_sa + (unsigned)((buf ^ 1) * kBufF4 * 16));
        }
        const char *ys1 = reinterpret_cast<const char *>(ys + buf * kBufF4) + 32 * h + o1;  // first half
        const char *ys2 = ys1 + (o2 - o1);                                                  // second half
        float2 acc0 = make_float2(0.f, 0.f), acc1 = make_float2(0.f, 0.f);
        float2 acc2 = make_float2(0.f, 0.f), acc3 = make_float2(0.f, 0.f);
        int rem = 0, gy = 0;  // body lines left in the bundle, its row's grid point
        auto apply = [&](int wbits, int y) {
            bundle_apply(ys1, wbits, y, acc0, acc1);
            bundle_apply(ys2, wbits, y, acc2, acc3);
        };
        auto line = [&](const int4 u) {
            if (rem == 0) {  // a header (warp-uniform: the rows of a bundle move together)
                rem = u.x;
                gy = u.y;
                return;
            }
            apply(u.x, u.y);
            apply(u.z, u.w);
            if (--rem == 0) {
                if (gy < 0) {
                    const size_t gp = (size_t)(-1 - gy) * nc;
                    atomicAdd(reinterpret_cast<float4 *>(G1 + gp), make_float4(acc0.x, acc0.y, acc1.x, acc1.y));
                    atomicAdd(reinterpret_cast<float4 *>(G2 + gp), make_float4(acc2.x, acc2.y, acc3.x, acc3.y));
                }
                acc0 = make_float2(0.f, 0.f);
                acc1 = make_float2(0.f, 0.f);
                acc2 = make_float2(0.f, 0.f);
                acc3 = make_float2(0.f, 0.f);
            }
        };
        uint32_t pf = l_lo + kSpreadDepth + kPrefetchAhead + kPrefetchLines;  // next line to prefetch
        for (uint32_t l = l_lo; l < l_hi; l += kSpreadDepth) {
            if (lane == 0 && l + kSpreadDepth + kPrefetchAhead >= pf) {
                prefetch_l2(lines, pf, l_hi);
                pf += kPrefetchLines;
            }
#pragma unroll
            for (int k = 0; k < kSpreadDepth; ++k) {
                const int4 u = e[k];
                e[k] = ld_ent4(lr + (size_t)(l + k + kSpreadDepth) * kLineInt4);
                line(u);
            }
        }
        // the next piece's first lines, while the others finish this piece
        if (bn < npieces) {
            l_lo = __ldg(&wstart[(size_t)bn * (kSpreadWarps + 1) + warp]);
            l_hi = __ldg(&wstart[(size_t)bn * (kSpreadWarps + 1) + warp + 1]);
#pragma unroll
            for (int k = 0; k < kSpreadDepth; ++k) e[k] = ld_ent4(lr + (size_t)(l_lo + k) * kLineInt4);
        }
        __syncthreads();  // this buffer is free: the piece after next lands in it
        buf ^= 1;
        b = bn;
    }
}

// ---------------------------------------------------------------- host

bool spread_tab_applies(const nufft3d_plan *p, int nc, int c0)
{
    return p->spread_ent != nullptr && nc % 2 == 0 && c0 + 8 <= nc;
}

size_t spread_tab_smem() { return (size_t)2 * (kSpreadCap + 2) * 64; }

int launch_spread_tab(nufft3d_plan *p, const float2 *ks, float2 *G, int nc, int c0, cudaStream_t s)
{
    if (p->n_spread_pieces == 0) return NUFFT3D_SUCCESS;
    NUFFT_CUDA_TRY(cudaMemsetAsync(p->work + kWorkSpread, 0, sizeof(int), s));
    const int64_t grid = std::min<int64_t>(p->n_spread_pieces, interp_grid_sms(p));
    k_spread_tab<<<(unsigned)grid, kSpreadThreads, spread_tab_smem(), s>>>(
        ks, G, nc, c0, p->spread_pieces, (int)p->n_spread_pieces, p->work + kWorkSpread, p->spread_wstart,
        reinterpret_cast<const int4 *>(p->spread_ent));
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

static size_t build_smem(const Geom &g)
{
    return (size_t)(kTabBuildWarps + 2) * g.P[0] * g.P[1] * g.P[2] * sizeof(uint32_t);
}

int configure_spread_tab_kernels()
{
    NUFFT_CUDA_TRY(cudaFuncSetAttribute(k_spread_tab, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)spread_tab_smem()));
    for (auto k : {k_spread_tab_build<false>, k_spread_tab_build<true>}) {
        cudaFuncAttributes fa;
        NUFFT_CUDA_TRY(cudaFuncGetAttributes(&fa, k));
        NUFFT_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            227 * 1024 - (int)fa.sharedSizeBytes));
    }
    return NUFFT3D_SUCCESS;
}

// The stored H' (needs the stored H).  mode 0 = none, 1 = always, -1 = when
// it takes at most half of the free device memory.
int build_spread_table(nufft3d_plan *p, int mode, cudaStream_t s)
{
    if (mode == 0 || p->tap_ent == nullptr || p->nnz == 0) return NUFFT3D_SUCCESS;
    const Geom &g = p->geom;
    const int P = g.P[0] * g.P[1] * g.P[2];
    if (P > kTabBuildThreads * kTabSortItems || P > 4096 || build_smem(g) > 160 * 1024) {
        if (mode < 0) return NUFFT3D_SUCCESS;
        return fail(NUFFT3D_ERR_UNSUPPORTED, "padded tile too large for the stored H'");
    }
    std::vector<int4> pcs = make_pieces(p->tile_counts, kSpreadCap);
    const int64_t np = (int64_t)pcs.size();
    pcs.push_back(make_int4(0, 0, 0, 0));
    struct Tmp {
        std::vector<void *> ptrs;
        ~Tmp()
        {
            NUFFT_DEVICE_LOCK;
            for (void *q : ptrs) cudaFree(q);
        }
    } tmp;
    int4 *dp = nullptr;
    uint32_t *dl = nullptr;
    {
        NUFFT_DEVICE_LOCK;
        NUFFT_CUDA_TRY(cudaMalloc(&dp, sizeof(int4) * pcs.size()));
        tmp.ptrs.push_back(dp);
        NUFFT_CUDA_TRY(cudaMalloc(&dl, sizeof(uint32_t) * pcs.size()));
        tmp.ptrs.push_back(dl);
    }
    NUFFT_CUDA_TRY(cudaMemcpyAsync(dp, pcs.data(), sizeof(int4) * pcs.size(), cudaMemcpyHostToDevice, s));
    const size_t smem = build_smem(g);
    k_spread_tab_build<false><<<(unsigned)np, kTabBuildThreads, smem, s>>>(dp, p->tap_rows, p->tap_ent, g, dl,
                                                                         nullptr, nullptr);
    NUFFT_CUDA_TRY(cudaGetLastError());
    std::vector<uint32_t> nl((size_t)np);
    NUFFT_CUDA_TRY(cudaMemcpyAsync(nl.data(), dl, sizeof(uint32_t) * np, cudaMemcpyDeviceToHost, s));
    NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    uint64_t total = 0;  // lines
    for (int64_t b = 0; b < np; ++b) {
        pcs[(size_t)b].w = (int)(uint32_t)total;
        total += nl[(size_t)b];
        if (total >= 0xffffffffull) {  // line indices are 32-bit
            if (mode < 0) return NUFFT3D_SUCCESS;
            return fail(NUFFT3D_ERR_SIZE, "too many entries for the stored H'");
        }
    }
    const size_t bytes = ((size_t)total + kSpreadDepth) * kLineBytes;  // spare empty lines for the pipeline's overrun
    const size_t wbytes = sizeof(uint32_t) * (size_t)np * (kSpreadWarps + 1);
    if (mode < 0) {
        size_t fr = 0, to = 0;
        if (cudaMemGetInfo(&fr, &to) != cudaSuccess || bytes + wbytes > fr / 2) {
            cudaGetLastError();
            return NUFFT3D_SUCCESS;  // the spread evaluates the kernel instead
        }
    }
    int2 *ent = nullptr;
    int4 *pieces = nullptr;
    uint32_t *wst = nullptr;
    {
        NUFFT_DEVICE_LOCK;
        cudaError_t e = cudaMalloc(&ent, bytes);
        if (e == cudaSuccess) e = cudaMalloc(&pieces, sizeof(int4) * pcs.size());
        if (e == cudaSuccess) e = cudaMalloc(&wst, wbytes ? wbytes : 4);
        if (e != cudaSuccess) {
            if (ent) cudaFree(ent);
            if (pieces) cudaFree(pieces);
            cudaGetLastError();
            if (mode < 0) return NUFFT3D_SUCCESS;
            return fail(NUFFT3D_ERR_NOMEM, std::string("stored H': ") + cudaGetErrorString(e));
        }
    }
    NUFFT_CUDA_TRY(cudaMemsetAsync(reinterpret_cast<char *>(ent) + (size_t)total * kLineBytes, 0,
                                   (size_t)kSpreadDepth * kLineBytes, s));
    p->spread_ent = ent;
    p->spread_pieces = pieces;
    p->spread_wstart = wst;
    p->n_spread_pieces = np;
    p->spread_bytes = (int64_t)(bytes + wbytes + sizeof(int4) * pcs.size());
    p->table_bytes += p->spread_bytes;
    NUFFT_CUDA_TRY(cudaMemcpyAsync(pieces, pcs.data(), sizeof(int4) * pcs.size(), cudaMemcpyHostToDevice, s));
    k_spread_tab_build<true><<<(unsigned)np, kTabBuildThreads, smem, s>>>(pieces, p->tap_rows, p->tap_ent, g,
                                                                        nullptr, wst, ent);
    NUFFT_CUDA_TRY(cudaGetLastError());
    NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    return NUFFT3D_SUCCESS;
}

}  // namespace nufft3d
