/*
 * Runs the MATLAB gateway (nufft_3d_gb300/matlab/nufft3d_mex.c) through the
 * mock MEX runtime (mex_mock.c), the way @nufft_3d calls it: create, info,
 * forward, adjoint, inverse (CG and MINRES, with and without W),
 * inverse_x0, inverse_phase, deap, getd, density and destroy, plus error
 * paths.  Each result is compared bit for bit with the same C-ABI call made
 * directly.  Exit 0 and "PASS" on success, 2 if there is no CUDA device,
 * 1 on a mismatch.  Test infrastructure only.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex_mock.h"
#include "nufft3d.h"

static unsigned long long g_seed = 12345;
static double urand(void)
{
    g_seed = g_seed * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(g_seed >> 11) * (1.0 / 9007199254740992.0);
}

#define CHECK(cond, what)                                          \
    do {                                                           \
        if (!(cond)) {                                             \
            printf("FAIL %s (%s)\n", what, mock_last_error());     \
            return 1;                                              \
        }                                                          \
    } while (0)

static int same(const void *a, const void *b, size_t n) { return memcmp(a, b, n) == 0; }

int main(void)
{
    const int N = 24, nc = 2;
    const int64_t M = 4000;
    const size_t nimg = (size_t)N * N * N;
    mxArray *om = mxCreateNumericMatrix(3, (mwSize)M, mxDOUBLE_CLASS, mxREAL);
    for (int64_t i = 0; i < 3 * M; ++i) mxGetDoubles(om)[i] = urand() * (N - 1) - N / 2;
    const char *fields[] = {"J"};
    mxArray *opts = mxCreateStructMatrix(1, 1, 1, fields);
    mxSetField(opts, 0, "J", mxCreateDoubleScalar(6));
    mxArray *Nmx = mxCreateDoubleScalar(N);
    mxArray *out[2] = {NULL, NULL};
    const mxArray *in[9];

    in[0] = mock_string("create"); in[1] = om; in[2] = Nmx; in[3] = opts;
    if (mock_call(1, out, 4, in)) {
        printf("create: %s\n", mock_last_error());
        return strstr(mock_last_error(), "no CUDA device") ? 2 : 1;
    }
    mxArray *h = out[0];
    nufft3d_plan *p = (nufft3d_plan *)(uintptr_t)mxGetUint64s(h)[0];

    in[0] = mock_string("info"); in[1] = h;
    CHECK(!mock_call(1, out, 2, in), "info");
    CHECK(mxGetDoubles(mxGetField(out[0], 0, "N"))[2] == N && mxGetScalar(mxGetField(out[0], 0, "M")) == M, "info N/M");

    mwSize dims[4] = {(mwSize)N, (mwSize)N, (mwSize)N, (mwSize)nc};
    mxArray *x = mxCreateNumericArray(4, dims, mxSINGLE_CLASS, mxCOMPLEX);
    float *xf = (float *)mxGetComplexSingles(x);
    for (size_t i = 0; i < 2 * nimg * nc; ++i) xf[i] = (float)(urand() - 0.5);

    in[0] = mock_string("forward"); in[1] = h; in[2] = x;
    CHECK(!mock_call(1, out, 3, in), "forward");
    mxArray *k = out[0];
    float *kref = (float *)malloc(sizeof(float) * 2 * M * nc);
    CHECK(nufft3d_forward_host(p, xf, kref, nc) == 0, "direct forward");
    CHECK(same(mxGetComplexSingles(k), kref, sizeof(float) * 2 * M * nc), "forward equals the C ABI");

    in[0] = mock_string("adjoint"); in[1] = h; in[2] = k;
    CHECK(!mock_call(1, out, 3, in), "adjoint");
    float *aref = (float *)malloc(sizeof(float) * 2 * nimg * nc);
    CHECK(nufft3d_adjoint_host(p, kref, aref, nc) == 0, "direct adjoint");
    CHECK(same(mxGetComplexSingles(out[0]), aref, sizeof(float) * 2 * nimg * nc), "adjoint equals the C ABI");

    mxArray *empty = mxCreateDoubleMatrix(0, 0, mxREAL);
    mxArray *W = mxCreateNumericMatrix((mwSize)M, 1, mxSINGLE_CLASS, mxREAL);
    for (int64_t i = 0; i < M; ++i) mxGetSingles(W)[i] = (float)(0.5 + urand());
    float *iref = (float *)malloc(sizeof(float) * 2 * nimg * nc);
    int its[2], its_ref[2];
    const char *solvers[2] = {"cg", "minres"};
    for (int sv = 0; sv < 2; ++sv)
        for (int wi = 0; wi < 2; ++wi) {
            in[0] = mock_string("inverse"); in[1] = h; in[2] = k; in[3] = mxCreateDoubleScalar(5);
            in[4] = mxCreateDoubleScalar(0.1); in[5] = wi ? W : empty; in[6] = mock_string(solvers[sv]);
            in[7] = mxCreateDoubleScalar(0);
            CHECK(!mock_call(2, out, 8, in), "inverse");
            memcpy(its, mxGetInt32s(out[1]), sizeof its);
            CHECK(nufft3d_inverse_host(p, kref, iref, nc, 5, 0.1, wi ? mxGetSingles(W) : NULL,
                                       sv ? NUFFT3D_SOLVER_MINRES : NUFFT3D_SOLVER_CG, 0.0, its_ref) == 0,
                  "direct inverse");
            CHECK(same(mxGetComplexSingles(out[0]), iref, sizeof(float) * 2 * nimg * nc), "inverse equals the C ABI");
            CHECK(its[0] == 5 && its[1] == 5 && its_ref[0] == 5, "iteration counts");
        }
    mxArray *x0 = out[0];   /* the last (MINRES, weighted) image starts the warm solve */

    in[0] = mock_string("inverse_x0"); in[1] = h; in[2] = k; in[3] = x0; in[4] = mxCreateDoubleScalar(3);
    in[5] = mxCreateDoubleScalar(0.1); in[6] = empty; in[7] = mock_string("minres"); in[8] = mxCreateDoubleScalar(0);
    CHECK(!mock_call(2, out, 9, in), "inverse_x0");
    memcpy(iref, mxGetComplexSingles(x0), sizeof(float) * 2 * nimg * nc);
    CHECK(nufft3d_inverse_x0_host(p, kref, iref, nc, 3, 0.1, NULL, NUFFT3D_SOLVER_MINRES, 0.0, its_ref) == 0,
          "direct inverse_x0");
    CHECK(same(mxGetComplexSingles(out[0]), iref, sizeof(float) * 2 * nimg * nc), "inverse_x0 equals the C ABI");

    in[0] = mock_string("inverse_phase"); in[1] = h; in[2] = k; in[3] = mxCreateDoubleScalar(4);
    in[4] = mxCreateDoubleScalar(0.1); in[5] = mxCreateDoubleScalar(0.5); in[6] = empty; in[7] = mxCreateDoubleScalar(0);
    CHECK(!mock_call(2, out, 8, in), "inverse_phase");
    CHECK(nufft3d_inverse_phase_host(p, kref, iref, nc, 4, 0.1, 0.5, NULL, 0.0, its_ref) == 0, "direct inverse_phase");
    CHECK(same(mxGetComplexSingles(out[0]), iref, sizeof(float) * 2 * nimg * nc), "inverse_phase equals the C ABI");

    in[0] = mock_string("deap"); in[1] = h;
    CHECK(!mock_call(1, out, 2, in), "deap");
    float *U = (float *)malloc(sizeof(float) * nimg);
    CHECK(nufft3d_get_deap(p, U) == 0 && same(mxGetSingles(out[0]), U, sizeof(float) * nimg), "deap");
    in[0] = mock_string("getd");
    CHECK(!mock_call(1, out, 2, in), "getd");
    float *d = (float *)malloc(sizeof(float) * M);
    CHECK(nufft3d_get_density(p, d) == 0 && same(mxGetSingles(out[0]), d, sizeof(float) * M), "getd");
    in[0] = mock_string("density"); in[2] = mxCreateDoubleScalar(5);
    CHECK(!mock_call(0, out, 3, in), "density");

    /* errors come back as MATLAB errors with the library's or the gateway's text */
    in[0] = mock_string("inverse"); in[1] = h; in[2] = k; in[3] = mxCreateDoubleScalar(5);
    in[4] = mxCreateDoubleScalar(0.1); in[5] = empty; in[6] = mock_string("bicg"); in[7] = mxCreateDoubleScalar(0);
    CHECK(mock_call(1, out, 8, in) && strstr(mock_last_error(), "solver"), "bad solver is refused");
    in[0] = mock_string("nosuchcmd");
    CHECK(mock_call(1, out, 2, in) && strstr(mock_last_error(), "unknown command"), "unknown command is refused");
    mwSize bad[2] = {7, 1};
    mxArray *xbad = mxCreateNumericArray(2, bad, mxSINGLE_CLASS, mxCOMPLEX);
    in[0] = mock_string("forward"); in[2] = xbad;
    CHECK(mock_call(1, out, 3, in) && strstr(mock_last_error(), "multiple of"), "wrong image size is refused");
    in[0] = mock_string("inverse_phase"); in[2] = k;
    CHECK(mock_call(1, out, 3, in), "missing arguments are refused");

    in[0] = mock_string("destroy"); in[1] = h;
    CHECK(!mock_call(0, out, 2, in), "destroy");
    printf("PASS: gateway commands equal the C ABI calls\n");
    return 0;
}
