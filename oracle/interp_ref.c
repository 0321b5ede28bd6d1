/*
 * Matrix-free FP64 restatement of the interpolation matrix H of
 * marcsous/nufft_3d (TEST INFRASTRUCTURE ONLY -- the oracle, never shipped).
 *
 * It applies y = H*g and g += H'*y without storing H, so configurations whose
 * H has billions of nonzeros (N=128..192, M=8..23 M) can be checked.  The
 * arithmetic follows the reference line by line:
 *
 *   @nufft_3d/nufft_3d.m:154      offsets -ceil(J/2):ceil(J/2)
 *   @nufft_3d/nufft_3d.m:168-175  x = round(om)+dx (half away from zero),
 *                                 squared distances in double
 *   @nufft_3d/nufft_3d.m:178-180  mod-K wrap
 *   @nufft_3d/nufft_3d.m:183-192  radial (4*dist2 <= J^2) or separable test,
 *                                 column-major index x + K1*y + K1*K2*z
 *   @nufft_3d/nufft_3d.m:160,195  weights stored as single: (double)(float)w
 *   @nufft_3d/kernel.m:2-30       KB kernel with the Numerical Recipes I0
 *                                 polynomial (real branch: 4*dist2 <= J^2
 *                                 keeps the argument real)
 *
 * Data: om_g is the scaled trajectory u*om, [3 x M] column-major doubles;
 * ok is the in-bounds mask (nufft_3d.m:123-125); complex arrays are
 * interleaved (re, im) doubles; grids are K1*K2*K3 per coil, coil planes
 * contiguous; sample data is M per coil.
 *
 * Parallelism: forward is a parallel loop over samples.  The adjoint splits
 * the grid into an even number of z-slabs of height >= 2R+1 and runs the even
 * slabs, then the odd ones, so two threads never write the same grid plane;
 * the result does not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static double bessi0_nr(double ax)
{
    if (fabs(ax) < 3.75) {
        double y = ax / 3.75;
        y = y * y;
        return 1.0 + y * (3.5156229 + y * (3.0899424 + y * (1.2067492 +
               y * (0.2659732 + y * (0.360768e-1 + y * 0.45813e-2)))));
    }
    double y = 3.75 / ax;
    return (exp(ax) / sqrt(ax)) * (0.39894228 + y * (0.1328592e-1 +
           y * (0.225319e-2 + y * (-0.157565e-2 + y * (0.916281e-2 + y * (-0.2057706e-1 +
           y * (0.2635537e-1 + y * (-0.1647633e-1 + y * 0.392377e-2))))))));
}

typedef struct {
    int64_t K[3];
    double J, alpha, i0a;
    int radial, is2d, R;
} params_t;

static double kb(const params_t *p, double dist2)
{
    double half = p->J / 2;
    double arg = p->alpha * sqrt(1 - dist2 / (half * half));
    return bessi0_nr(arg) / p->i0a;
}

static int64_t wrap(int64_t x, int64_t K)
{
    int64_t r = x % K;
    return r < 0 ? r + K : r;
}

/* Visit every (grid index, single-rounded weight) of row m of H. */
#define FOR_TAPS(p, og, BODY)                                                   \
    do {                                                                        \
        double bx = round(og[0]), by = round(og[1]), bz = round(og[2]);         \
        int rz_lo = (p)->is2d ? 0 : -(p)->R, rz_hi = (p)->is2d ? 0 : (p)->R;    \
        double J2 = (p)->J * (p)->J;                                            \
        for (int dx = -(p)->R; dx <= (p)->R; ++dx)                              \
            for (int dy = -(p)->R; dy <= (p)->R; ++dy)                          \
                for (int dz = rz_lo; dz <= rz_hi; ++dz) {                       \
                    double tx_ = bx + dx, ty_ = by + dy, tz_ = bz + dz;         \
                    double dx2 = (tx_ - og[0]) * (tx_ - og[0]);                 \
                    double dy2 = (ty_ - og[1]) * (ty_ - og[1]);                 \
                    double dz2 = (tz_ - og[2]) * (tz_ - og[2]);                 \
                    double w;                                                   \
                    if ((p)->radial) {                                          \
                        double dist2 = dx2 + dy2 + dz2;                         \
                        if (!(4 * dist2 <= J2)) continue;                       \
                        w = kb((p), dist2);                                     \
                    } else {                                                    \
                        if (!(4 * dx2 <= J2 && 4 * dy2 <= J2 && 4 * dz2 <= J2)) \
                            continue;                                           \
                        w = kb((p), dx2) * kb((p), dy2) * kb((p), dz2);         \
                    }                                                           \
                    w = (double)(float)w;                                       \
                    int64_t col = wrap((int64_t)tx_, (p)->K[0]) +               \
                        (p)->K[0] * (wrap((int64_t)ty_, (p)->K[1]) +            \
                        (p)->K[1] * wrap((int64_t)tz_, (p)->K[2]));             \
                    BODY                                                        \
                }                                                               \
    } while (0)

static void init_params(params_t *p, const int64_t K[3], double J, double alpha,
                        int radial, int is2d)
{
    p->K[0] = K[0]; p->K[1] = K[1]; p->K[2] = K[2];
    p->J = J; p->alpha = alpha; p->radial = radial; p->is2d = is2d;
    p->R = (int)ceil(J / 2);
    p->i0a = bessi0_nr(alpha);
}

/* out[m + M*c] = sum_taps w * grid[col + G*c]  (out of bounds rows -> 0) */
void oracle_interp_forward(const double *om_g, const uint8_t *ok, int64_t M,
                           const int64_t *K, double J, double alpha, int radial,
                           int is2d, const double *grid, int nc, double *out)
{
    params_t p;
    init_params(&p, K, J, alpha, radial, is2d);
    const int64_t G = K[0] * K[1] * K[2];
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t m = 0; m < M; ++m) {
        double acc[2 * 64];
        int ncc = nc < 64 ? nc : 64;
        for (int c0 = 0; c0 < nc; c0 += ncc) {
            int cn = nc - c0 < ncc ? nc - c0 : ncc;
            memset(acc, 0, sizeof(double) * 2 * cn);
            if (ok[m]) {
                const double *og = om_g + 3 * m;
                FOR_TAPS(&p, og, {
                    for (int c = 0; c < cn; ++c) {
                        const double *gv = grid + 2 * (col + G * (c0 + c));
                        acc[2 * c] += w * gv[0];
                        acc[2 * c + 1] += w * gv[1];
                    }
                });
            }
            for (int c = 0; c < cn; ++c) {
                out[2 * (m + M * (int64_t)(c0 + c))] = acc[2 * c];
                out[2 * (m + M * (int64_t)(c0 + c)) + 1] = acc[2 * c + 1];
            }
        }
    }
}

static void spread_one(const params_t *p, const double *om_g, int64_t m, int64_t M,
                       int64_t G, const double *y, int nc, double *grid)
{
    const double *og = om_g + 3 * m;
    FOR_TAPS(p, og, {
        for (int c = 0; c < nc; ++c) {
            const double *yv = y + 2 * (m + M * (int64_t)c);
            double *gv = grid + 2 * (col + G * (int64_t)c);
            gv[0] += w * yv[0];
            gv[1] += w * yv[1];
        }
    });
}

/* grid[col + G*c] += sum_m w * y[m + M*c]  (grid accumulates; caller zeroes) */
void oracle_interp_adjoint(const double *om_g, const uint8_t *ok, int64_t M,
                           const int64_t *K, double J, double alpha, int radial,
                           int is2d, const double *y, int nc, double *grid)
{
    params_t p;
    init_params(&p, K, J, alpha, radial, is2d);
    const int64_t G = K[0] * K[1] * K[2];
    /* n slabs (n even) of height >= 2R+1: slabs s and s+2 are separated by a
       whole slab, so one colour never writes the same grid plane twice, even
       across the periodic wrap (slab n-1 separates slab n-2 from slab 0). */
    int64_t n = is2d ? 0 : K[2] / (2 * p.R + 1);
    if (n & 1) n -= 1;
    if (n < 4) {
        for (int64_t m = 0; m < M; ++m)
            if (ok[m]) spread_one(&p, om_g, m, M, G, y, nc, grid);
        return;
    }
    const int64_t nslab = n;
    int64_t *cnt = (int64_t *)calloc((size_t)nslab + 1, sizeof(int64_t));
    int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(M > 0 ? M : 1));
    int64_t *slab = (int64_t *)malloc(sizeof(int64_t) * (size_t)(M > 0 ? M : 1));
    for (int64_t m = 0; m < M; ++m) {
        slab[m] = -1;
        if (!ok[m]) continue;
        int64_t z = wrap((int64_t)round(om_g[3 * m + 2]), K[2]);
        int64_t s = (z * nslab) / K[2];               /* floor(s*K/n) <= z */
        while (s + 1 < nslab && ((s + 1) * K[2]) / nslab <= z) ++s;
        while (s > 0 && (s * K[2]) / nslab > z) --s;
        slab[m] = s;
        cnt[s + 1]++;
    }
    for (int64_t s = 0; s < nslab; ++s) cnt[s + 1] += cnt[s];
    int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (size_t)nslab);
    memcpy(pos, cnt, sizeof(int64_t) * (size_t)nslab);
    for (int64_t m = 0; m < M; ++m)
        if (slab[m] >= 0) idx[pos[slab[m]]++] = m;
    for (int phase = 0; phase < 2; ++phase) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t s = phase; s < nslab; s += 2)
            for (int64_t q = cnt[s]; q < cnt[s + 1]; ++q)
                spread_one(&p, om_g, idx[q], M, G, y, nc, grid);
    }
    free(pos); free(slab); free(idx); free(cnt);
}
