/*
 * nufft3d_harness.c -- a plain C host for libnufft3d.so (no MATLAB, no CUDA
 * headers): the sequence a MATLAB session runs on @nufft_3d,
 *
 *   obj = nufft_3d(om, N, 'J', 6);       (nufft_3d.m:54-251)
 *   k   = obj.fNUFT(x);                   (fNUFT.m:2-9)
 *   a   = obj.aNUFT(y);                   (aNUFT.m:2-9)
 *   im  = obj.iNUFT(k, 20, 0.01);         (iNUFT.m:2-138, CG here)
 *
 * through the host-pointer entry points of include/nufft3d.h, and checks
 *   1. the adjoint identity <y, A x> = <A' y, x> (relative error < 1e-5),
 *   2. that the reconstruction lowers the weighted least-squares objective
 *      ||d^(1/2) (A im - k)||^2 + damp^2 ||im||^2 of iNUFT below half its
 *      value at im = 0 (CG decreases it monotonically from x0 = 0).
 *
 * Trajectory: golden-angle koosh ball, N = 32, 32 points x 600 spokes.
 * Exit status: 0 pass, 1 check failed, 2 no usable CUDA device, 3 API error.
 * Usage: nufft3d_harness [N] [spokes]
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "nufft3d.h"

#define CHECK(call)                                                                  \
    do {                                                                             \
        int st_ = (call);                                                            \
        if (st_ != NUFFT3D_SUCCESS) {                                                \
            fprintf(stderr, "%s failed (%d): %s\n", #call, st_, nufft3d_last_error()); \
            return 3;                                                                \
        }                                                                            \
    } while (0)

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;

/* xorshift64*: uniform in [-1, 1) */
static float urand(void)
{
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    const uint64_t r = rng_state * 0x2545f4914f6cdd1dull;
    return (float)((double)(r >> 11) * (2.0 / 9007199254740992.0) - 1.0);
}

/* Koosh ball: spokes through the centre, directions on a golden-angle
 * spiral over the sphere, nr points per spoke in cycles/FOV. */
static void koosh_ball(double *om, int N, int nr, int ns)
{
    const double ga = M_PI * (3.0 - sqrt(5.0));
    for (int s = 0; s < ns; ++s) {
        const double z = 1.0 - 2.0 * (s + 0.5) / ns;
        const double r = sqrt(1.0 - z * z), ph = ga * s;
        const double dir[3] = {r * cos(ph), r * sin(ph), z};
        for (int i = 0; i < nr; ++i) {
            const double rad = (i - nr / 2) * ((double)N / nr);
            for (int a = 0; a < 3; ++a) om[3 * ((int64_t)s * nr + i) + a] = rad * dir[a];
        }
    }
}

/* sum conj(a) b over n complex values, in double */
static void cdot(const float *a, const float *b, int64_t n, double *re, double *im)
{
    double sr = 0, si = 0;
    for (int64_t i = 0; i < n; ++i) {
        const double ar = a[2 * i], ai = a[2 * i + 1], br = b[2 * i], bi = b[2 * i + 1];
        sr += ar * br + ai * bi;
        si += ar * bi - ai * br;
    }
    *re = sr;
    *im = si;
}

int main(int argc, char **argv)
{
    const int N = argc > 1 ? atoi(argv[1]) : 32;
    const int ns = argc > 2 ? atoi(argv[2]) : 600;
    const int nr = N;
    const int64_t M = (int64_t)nr * ns, nvox = (int64_t)N * N * N;
    const int32_t Nv[1] = {N};

    double *om = malloc(sizeof(double) * 3 * M);
    float *x = malloc(sizeof(float) * 2 * nvox), *a = malloc(sizeof(float) * 2 * nvox);
    float *im = malloc(sizeof(float) * 2 * nvox);
    float *k = malloc(sizeof(float) * 2 * M), *y = malloc(sizeof(float) * 2 * M);
    float *r = malloc(sizeof(float) * 2 * M), *d = malloc(sizeof(float) * M);
    if (!om || !x || !a || !im || !k || !y || !r || !d) {
        fprintf(stderr, "host allocation failed\n");
        return 3;
    }
    koosh_ball(om, N, nr, ns);

    nufft3d_opts o;
    CHECK(nufft3d_opts_default(&o));
    o.J = 6;
    nufft3d_plan *plan = NULL;
    const int st = nufft3d_plan_create(om, M, Nv, 1, &o, &plan);
    if (st == NUFFT3D_ERR_CUDA) {
        printf("no CUDA device: %s\n", nufft3d_last_error());
        return 2;
    }
    if (st != NUFFT3D_SUCCESS) {
        fprintf(stderr, "nufft3d_plan_create failed (%d): %s\n", st, nufft3d_last_error());
        return 3;
    }
    nufft3d_info info;
    CHECK(nufft3d_plan_info(plan, &info));
    printf("%s: N=[%d %d %d] K=[%d %d %d] M=%lld nnz=%lld J=%g u=%g alpha=%.6f taps/sample=%.1f\n",
           nufft3d_version(), info.N[0], info.N[1], info.N[2], info.K[0], info.K[1], info.K[2],
           (long long)info.M, (long long)info.nnz, info.J, info.u, info.alpha, info.taps_per_sample);

    /* 1. adjoint identity */
    for (int64_t i = 0; i < 2 * nvox; ++i) x[i] = urand();
    for (int64_t i = 0; i < 2 * M; ++i) y[i] = urand();
    CHECK(nufft3d_forward_host(plan, x, k, 1));
    CHECK(nufft3d_adjoint_host(plan, y, a, 1));
    double lr, li, rr, ri;
    cdot(y, k, M, &lr, &li);
    cdot(a, x, nvox, &rr, &ri);
    const double adj_err = hypot(lr - rr, li - ri) / hypot(lr, li);
    printf("adjoint identity: <y,Ax> = %.6e%+.6ei  <A'y,x> = %.6e%+.6ei  rel err %.2e\n", lr, li, rr, ri,
           adj_err);

    /* 2. iNUFT on the samples of a smooth image (a centred ball) */
    for (int64_t v = 0; v < nvox; ++v) {
        const int i = (int)(v % N), j = (int)((v / N) % N), l = (int)(v / ((int64_t)N * N));
        const double rx = i - N / 2, ry = j - N / 2, rz = l - N / 2;
        x[2 * v] = (rx * rx + ry * ry + rz * rz < (N / 3.0) * (N / 3.0)) ? 1.f : 0.f;
        x[2 * v + 1] = 0.f;
    }
    CHECK(nufft3d_forward_host(plan, x, k, 1));
    const double damp = 0.01;
    int iters = 0;
    CHECK(nufft3d_inverse_host(plan, k, im, 1, 20, damp, NULL, NUFFT3D_SOLVER_CG, 0.0, &iters));
    CHECK(nufft3d_get_density(plan, d));
    CHECK(nufft3d_forward_host(plan, im, r, 1));
    double f0 = 0, f1 = 0, xn = 0;
    for (int64_t i = 0; i < M; ++i) {
        const double er = r[2 * i] - k[2 * i], ei = r[2 * i + 1] - k[2 * i + 1];
        f0 += d[i] * ((double)k[2 * i] * k[2 * i] + (double)k[2 * i + 1] * k[2 * i + 1]);
        f1 += d[i] * (er * er + ei * ei);
    }
    for (int64_t v = 0; v < 2 * nvox; ++v) xn += (double)im[v] * im[v];
    f1 += damp * damp * xn;
    printf("iNUFT (CG, %d iterations): objective %.6e at im=0 -> %.6e (ratio %.3e)\n", iters, f0, f1, f1 / f0);

    CHECK(nufft3d_plan_destroy(plan));
    free(om); free(x); free(a); free(im); free(k); free(y); free(r); free(d);
    const int ok = adj_err < 1e-5 && iters == 20 && isfinite(f1) && f1 < 0.5 * f0;
    printf("%s\n", ok ? "PASS" : "FAIL");
    return ok ? 0 : 1;
}
