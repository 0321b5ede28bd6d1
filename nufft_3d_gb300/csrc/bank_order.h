// Host-side ordering of the candidate taps for shared-memory bank spread.
//
// The interpolation kernels read (gather) or add to (spread) the staged tile
// at offsets base + off(candidate, octant).  In the gather a chunk of 8
// consecutive candidates is read by 8 lanes in rotated coil-pair order (lanes
// l and l+4 share the rotation), which is conflict-free when those two taps
// have tile offsets of different parity.  In the spread 8 consecutive entries
// of the hit queue (the hits of a block of 64 candidates, in list order) are
// added by one instruction, conflict-free when their offsets differ modulo 8
// (the integer planes are shifted by 8 banks per coil pair).  The
// distance-sorted candidate list is therefore re-partitioned by a seeded local
// search: swaps between nearby chunks (keeping the near-to-far order that
// lets whole chunks of far taps go idle) are kept by simulated annealing on
// the expected number of wavefronts, estimated over a fixed set of sample
// positions in all 8 octants.  Deterministic: same inputs, same order.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace nufft3d {

struct BankOrderStats {
    double gather_before, gather_after;  // expected wavefronts per sample and coil pair
    double spread_before, spread_after;
};

// lo/hi: the box of reflected offsets |f| the list serves (per axis).
// The first `ncore` entries (the taps inside the support for every f of the
// box) stay the first ncore entries: swaps never cross that boundary.
inline void bank_order(std::vector<int> &code, int Px, int PxPy, double J, int radial, int is2d,
                       const double lo[3], const double hi[3], int ncore = 0, BankOrderStats *stats = nullptr,
                       int n_samples = 160, int sweeps = 24)
{
    const int n = (int)code.size();
    if (n <= 8) return;
    const double h2 = (J / 2) * (J / 2);
    uint64_t st = 0x2545f4914f6cdd1dull;
    auto uni = [&st]() {
        st ^= st >> 12;
        st ^= st << 25;
        st ^= st >> 27;
        return (double)((st * 0x2545f4914f6cdd1dull) >> 11) * (1.0 / 9007199254740992.0);
    };
    const int S = n_samples;
    // per sample: slot (0..7) or 8 when the candidate misses the support
    std::vector<uint8_t> slot((size_t)S * n);
    for (int s = 0; s < S; ++s) {
        double f[3];
        int sg[3];
        for (int a = 0; a < 3; ++a) {
            sg[a] = uni() < 0.5 ? -1 : 1;
            f[a] = lo[a] + (hi[a] - lo[a]) * uni();
        }
        if (is2d) {
            f[2] = 0;
            sg[2] = 1;
        }
        for (int i = 0; i < n; ++i) {
            const int d[3] = {(code[i] & 15) - 8, ((code[i] >> 4) & 15) - 8, ((code[i] >> 8) & 15) - 8};
            double e2[3];
            for (int a = 0; a < 3; ++a) e2[a] = (d[a] - f[a]) * (d[a] - f[a]);
            const bool hit = radial ? (e2[0] + e2[1] + e2[2] <= h2) : (e2[0] <= h2 && e2[1] <= h2 && e2[2] <= h2);
            const int off = sg[2] * d[2] * PxPy + sg[1] * d[1] * Px + sg[0] * d[0];
            slot[(size_t)s * n + i] = hit ? (uint8_t)(((off % 8) + 8) % 8) : 8;
        }
    }
    std::vector<int> pos(n);  // position -> candidate
    for (int i = 0; i < n; ++i) pos[i] = i;
    constexpr int kQ = 64;  // candidates evaluated per spread queue fill
    const int nchunk = (n + 7) / 8, nblock = (n + kQ - 1) / kQ;
    // gather: lanes l and l+4 of a chunk read the same rotated coil pair of
    // their taps, so a load takes a second wavefront when two such taps are
    // both hit and have tile offsets of equal parity
    auto chunk_cost = [&](int c) {
        long t = 0;
        const int b = 8 * c;
        for (int s = 0; s < S; ++s) {
            const uint8_t *sl = &slot[(size_t)s * n];
            bool any = false, coll = false;
            for (int l = 0; l < 8 && b + l < n; ++l) any |= sl[pos[b + l]] < 8;
            for (int l = 0; l < 4 && b + l + 4 < n; ++l) {
                const int u = sl[pos[b + l]], v = sl[pos[b + l + 4]];
                coll |= u < 8 && v < 8 && ((u ^ v) & 1) == 0;
            }
            t += any ? 1 + (coll ? 1 : 0) : 0;
        }
        return t;
    };
    auto block_cost = [&](int blk) {
        long t = 0;
        const int b = kQ * blk, e = b + kQ < n ? b + kQ : n;
        for (int s = 0; s < S; ++s) {
            const uint8_t *sl = &slot[(size_t)s * n];
            int cnt[9] = {0}, mx = 0, q = 0;
            for (int p = b; p < e; ++p) {
                const int k = sl[pos[p]];
                if (k == 8) continue;
                if (++cnt[k] > mx) mx = cnt[k];
                if (++q == 8) {
                    t += mx;
                    q = mx = 0;
                    for (int z = 0; z < 8; ++z) cnt[z] = 0;
                }
            }
            t += mx;
        }
        return t;
    };
    std::vector<long> cc(nchunk), bc(nblock);
    long g0 = 0, s0 = 0;
    for (int c = 0; c < nchunk; ++c) g0 += cc[c] = chunk_cost(c);
    for (int b = 0; b < nblock; ++b) s0 += bc[b] = block_cost(b);
    long gsum = g0, ssum = s0;
    const long trials = (long)sweeps * n;
    for (long t = 0; t < trials; ++t) {
        const int p1 = (int)(uni() * n);
        int c2 = p1 / 8 + (int)(uni() * 5) - 2;
        if (c2 < 0 || c2 >= nchunk || c2 == p1 / 8) continue;
        const int lo = 8 * c2, hi = lo + 8 < n ? lo + 8 : n;
        const int p2 = lo + (int)(uni() * (hi - lo));
        if ((p1 < ncore) != (p2 < ncore)) continue;
        const int ca = p1 / 8, cb = p2 / 8, ba = p1 / kQ, bb = p2 / kQ;
        std::swap(pos[p1], pos[p2]);
        const long na = chunk_cost(ca), nb = chunk_cost(cb);
        const long nba = block_cost(ba), nbb = ba != bb ? block_cost(bb) : 0;
        const long delta = (na + nb - cc[ca] - cc[cb]) + (nba - bc[ba]) + (ba != bb ? nbb - bc[bb] : 0);
        // annealed acceptance: early on, small increases are taken to leave
        // local minima; the temperature falls linearly to zero
        const double T = 0.02 * S * (1.0 - (double)t / (double)trials);
        if (delta <= 0 || (T > 0 && uni() < std::exp(-(double)delta / T))) {
            gsum += na + nb - cc[ca] - cc[cb];
            ssum += (nba - bc[ba]) + (ba != bb ? nbb - bc[bb] : 0);
            cc[ca] = na;
            cc[cb] = nb;
            bc[ba] = nba;
            if (ba != bb) bc[bb] = nbb;
        } else {
            std::swap(pos[p1], pos[p2]);
        }
    }
    std::vector<int> out(n);
    for (int p = 0; p < n; ++p) out[p] = code[pos[p]];
    code.swap(out);
    if (stats) {
        stats->gather_before = (double)g0 / S;
        stats->gather_after = (double)gsum / S;
        stats->spread_before = (double)s0 / S;
        stats->spread_after = (double)ssum / S;
    }
}

} // namespace nufft3d
