/*
 * nufft3d_mex.c -- MATLAB gateway to libnufft3d.so (interleaved complex API,
 * build with `mex -R2018a`).  The class in @nufft_3d/ calls it; each command
 * maps to one C-ABI entry point of include/nufft3d.h:
 *
 *   h        = nufft3d_mex('create', om, N, opts)   nufft3d_plan_create
 *              om [3 x M] double, N 1 or 3 values, opts a struct with any of
 *              J u alpha radial gpu density_iters d (single [M])
 *   k        = nufft3d_mex('forward', h, x)         nufft3d_forward_host
 *              x complex single [N1 N2 N3 nc] -> k complex single [M nc]
 *   x        = nufft3d_mex('adjoint', h, k)         nufft3d_adjoint_host
 *   [x, it]  = nufft3d_mex('inverse', h, raw, maxit, damp, W, solver, tol)
 *              nufft3d_inverse_host; W [] or single [M]; solver 'minres'|'cg'
 *              it = iterations per coil
 *   [x, it]  = nufft3d_mex('inverse_x0', h, raw, x0, maxit, damp, W, solver, tol)
 *              nufft3d_inverse_x0_host: the same solve started from x0
 *              (complex single [N1 N2 N3 nc]), as discrep.m warm-starts it
 *   [x, it]  = nufft3d_mex('inverse_phase', h, raw, maxit, damp, lambda, W, tol)
 *              nufft3d_inverse_phase_host: iNUFT with 'phase-constraint'
 *              (iNUFT.m:140-168); it = iterations of the constrained solve
 *              nufft3d_mex('density', h, maxit)     nufft3d_density
 *   s        = nufft3d_mex('info', h)               nufft3d_plan_info
 *   U        = nufft3d_mex('deap', h)               nufft3d_get_deap
 *   d        = nufft3d_mex('getd', h)               nufft3d_get_density
 *              nufft3d_mex('destroy', h)            nufft3d_plan_destroy
 *
 * The handle is the plan pointer stored in a uint64 scalar.  Every failure
 * (a negative status) becomes a MATLAB error with the library's message.
 */
#include <stdint.h>
#include <string.h>

#include "mex.h"
#include "nufft3d.h"

static void fail_status(int st)
{
    mexErrMsgIdAndTxt("nufft3d:status", "libnufft3d status %d: %s", st, nufft3d_last_error());
}

#define CALL(expr)                          \
    do {                                    \
        int st_ = (expr);                   \
        if (st_ != NUFFT3D_SUCCESS) fail_status(st_); \
    } while (0)

static nufft3d_plan *get_plan(const mxArray *a)
{
    if (!mxIsUint64(a) || mxGetNumberOfElements(a) != 1)
        mexErrMsgIdAndTxt("nufft3d:handle", "plan handle must be a uint64 scalar");
    nufft3d_plan *p = (nufft3d_plan *)(uintptr_t)(*mxGetUint64s(a));
    if (!p) mexErrMsgIdAndTxt("nufft3d:handle", "plan handle is empty (destroyed?)");
    return p;
}

static const mxComplexSingle *complex_single(const mxArray *a, const char *what)
{
    if (!mxIsSingle(a) || !mxIsComplex(a))
        mexErrMsgIdAndTxt("nufft3d:type", "%s must be complex single", what);
    return mxGetComplexSingles(a);
}

static double field_or(const mxArray *s, const char *name, double dflt)
{
    const mxArray *f = s ? mxGetField(s, 0, name) : NULL;
    return (f && !mxIsEmpty(f)) ? mxGetScalar(f) : dflt;
}

static nufft3d_info plan_info(nufft3d_plan *p)
{
    nufft3d_info info;
    CALL(nufft3d_plan_info(p, &info));
    return info;
}

static void cmd_create(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs)
{
    if (nrhs < 3) mexErrMsgIdAndTxt("nufft3d:args", "create needs om and N");
    const mxArray *om = prhs[1];
    if (!mxIsDouble(om) || mxIsComplex(om) || mxGetM(om) != 3 || mxIsEmpty(om))
        mexErrMsgIdAndTxt("nufft3d:args", "om must be a real double array with leading dimension of 3");
    const int64_t M = (int64_t)(mxGetNumberOfElements(om) / 3);
    const size_t nN = mxGetNumberOfElements(prhs[2]);
    if (!mxIsDouble(prhs[2]) || (nN != 1 && nN != 3))
        mexErrMsgIdAndTxt("nufft3d:args", "N must be a double scalar or 3-vector");
    int32_t N[3];
    const double *Nd = mxGetDoubles(prhs[2]);
    for (size_t i = 0; i < nN; ++i) N[i] = (int32_t)Nd[i];
    const mxArray *s = (nrhs > 3 && mxIsStruct(prhs[3])) ? prhs[3] : NULL;

    nufft3d_opts o;
    CALL(nufft3d_opts_default(&o));
    o.J = field_or(s, "J", o.J);
    o.u = field_or(s, "u", o.u);
    o.alpha = field_or(s, "alpha", o.alpha);
    o.radial = (int)field_or(s, "radial", o.radial);
    o.gpu = (int)field_or(s, "gpu", o.gpu);
    o.density_iters = (int)field_or(s, "density_iters", o.density_iters);
    const mxArray *d = s ? mxGetField(s, 0, "d") : NULL;
    if (d && !mxIsEmpty(d)) {
        if (!mxIsSingle(d) || mxIsComplex(d) || (int64_t)mxGetNumberOfElements(d) != M)
            mexErrMsgIdAndTxt("nufft3d:args", "d must be real single with %lld elements", (long long)M);
        o.d = mxGetSingles(d);
    }
    nufft3d_plan *p = NULL;
    CALL(nufft3d_plan_create(mxGetDoubles(om), M, N, (int)nN, &o, &p));
    plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
    *mxGetUint64s(plhs[0]) = (uint64_t)(uintptr_t)p;
    (void)nlhs;
}

/* number of coils of an array whose leading elements form one coil */
static int coils_of(const mxArray *a, int64_t per_coil, const char *what)
{
    const int64_t n = (int64_t)mxGetNumberOfElements(a);
    if (per_coil <= 0 || n % per_coil || n == 0)
        mexErrMsgIdAndTxt("nufft3d:size", "%s must have a multiple of %lld elements (has %lld)", what,
                          (long long)per_coil, (long long)n);
    return (int)(n / per_coil);
}

static mxArray *complex_out(int64_t rows, int64_t cols, const int32_t *N3)
{
    if (N3) {
        mwSize dims[4] = {(mwSize)N3[0], (mwSize)N3[1], (mwSize)N3[2], (mwSize)cols};
        return mxCreateNumericArray(cols > 1 ? 4 : 3, dims, mxSINGLE_CLASS, mxCOMPLEX);
    }
    return mxCreateNumericMatrix((mwSize)rows, (mwSize)cols, mxSINGLE_CLASS, mxCOMPLEX);
}

static void cmd_forward(mxArray **plhs, const mxArray **prhs)
{
    nufft3d_plan *p = get_plan(prhs[1]);
    const nufft3d_info in = plan_info(p);
    const int64_t nvox = (int64_t)in.N[0] * in.N[1] * in.N[2];
    const int nc = coils_of(prhs[2], nvox, "x");
    const mxComplexSingle *x = complex_single(prhs[2], "x");
    plhs[0] = complex_out(in.M, nc, NULL);
    CALL(nufft3d_forward_host(p, (const float *)x, (float *)mxGetComplexSingles(plhs[0]), nc));
}

static void cmd_adjoint(mxArray **plhs, const mxArray **prhs)
{
    nufft3d_plan *p = get_plan(prhs[1]);
    const nufft3d_info in = plan_info(p);
    const int nc = coils_of(prhs[2], in.M, "k");
    const mxComplexSingle *k = complex_single(prhs[2], "k");
    plhs[0] = complex_out(0, nc, in.N);
    CALL(nufft3d_adjoint_host(p, (const float *)k, (float *)mxGetComplexSingles(plhs[0]), nc));
}

static const float *weights_or_null(const mxArray *a, int64_t M)
{
    if (mxIsEmpty(a)) return NULL;
    if (!mxIsSingle(a) || mxIsComplex(a) || (int64_t)mxGetNumberOfElements(a) != M)
        mexErrMsgIdAndTxt("nufft3d:args", "W must be [] or real single with %lld elements", (long long)M);
    return mxGetSingles(a);
}

static int solver_of(const mxArray *a)
{
    char solver[16] = {0};
    if (mxGetString(a, solver, sizeof solver) != 0)
        mexErrMsgIdAndTxt("nufft3d:args", "solver must be 'minres' or 'cg'");
    const int sol = strcmp(solver, "cg") == 0 ? NUFFT3D_SOLVER_CG : NUFFT3D_SOLVER_MINRES;
    if (sol == NUFFT3D_SOLVER_MINRES && strcmp(solver, "minres") != 0)
        mexErrMsgIdAndTxt("nufft3d:args", "solver must be 'minres' or 'cg'");
    return sol;
}

static void iters_out(int nlhs, mxArray **plhs, mxArray *it)
{
    if (nlhs > 1)
        plhs[1] = it;
    else
        mxDestroyArray(it);
}

/* [x, it] = inverse(h, raw, maxit, damp, W, solver, tol) and, with warm = 1,
 * inverse_x0(h, raw, x0, maxit, damp, W, solver, tol) */
static void cmd_inverse(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs, int warm)
{
    const int a = warm ? 1 : 0;  /* x0 shifts the later arguments by one */
    if (nrhs < 8 + a)
        mexErrMsgIdAndTxt("nufft3d:args", warm ? "inverse_x0 needs h, raw, x0, maxit, damp, W, solver, tol"
                                               : "inverse needs h, raw, maxit, damp, W, solver, tol");
    nufft3d_plan *p = get_plan(prhs[1]);
    const nufft3d_info in = plan_info(p);
    const int nc = coils_of(prhs[2], in.M, "raw");
    const mxComplexSingle *raw = complex_single(prhs[2], "raw");
    const int maxit = (int)mxGetScalar(prhs[3 + a]);
    const double damp = mxGetScalar(prhs[4 + a]);
    const float *W = weights_or_null(prhs[5 + a], in.M);
    const int sol = solver_of(prhs[6 + a]);
    const double tol = mxGetScalar(prhs[7 + a]);
    plhs[0] = complex_out(0, nc, in.N);
    float *x = (float *)mxGetComplexSingles(plhs[0]);
    mxArray *it = mxCreateNumericMatrix(1, (mwSize)nc, mxINT32_CLASS, mxREAL);
    if (warm) {
        const int64_t nvox = (int64_t)in.N[0] * in.N[1] * in.N[2];
        if (coils_of(prhs[3], nvox, "x0") != nc)
            mexErrMsgIdAndTxt("nufft3d:size", "x0 must have as many coils as raw");
        memcpy(x, complex_single(prhs[3], "x0"), sizeof(mxComplexSingle) * (size_t)(nvox * nc));
        CALL(nufft3d_inverse_x0_host(p, (const float *)raw, x, nc, maxit, damp, W, sol, tol, mxGetInt32s(it)));
    } else {
        CALL(nufft3d_inverse_host(p, (const float *)raw, x, nc, maxit, damp, W, sol, tol, mxGetInt32s(it)));
    }
    iters_out(nlhs, plhs, it);
}

/* [x, it] = inverse_phase(h, raw, maxit, damp, lambda, W, tol) */
static void cmd_inverse_phase(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs)
{
    if (nrhs < 8) mexErrMsgIdAndTxt("nufft3d:args", "inverse_phase needs h, raw, maxit, damp, lambda, W, tol");
    nufft3d_plan *p = get_plan(prhs[1]);
    const nufft3d_info in = plan_info(p);
    const int nc = coils_of(prhs[2], in.M, "raw");
    const mxComplexSingle *raw = complex_single(prhs[2], "raw");
    const int maxit = (int)mxGetScalar(prhs[3]);
    const double damp = mxGetScalar(prhs[4]);
    const double lambda = mxGetScalar(prhs[5]);
    const float *W = weights_or_null(prhs[6], in.M);
    const double tol = mxGetScalar(prhs[7]);
    plhs[0] = complex_out(0, nc, in.N);
    mxArray *it = mxCreateNumericMatrix(1, (mwSize)nc, mxINT32_CLASS, mxREAL);
    CALL(nufft3d_inverse_phase_host(p, (const float *)raw, (float *)mxGetComplexSingles(plhs[0]), nc, maxit, damp,
                                    lambda, W, tol, mxGetInt32s(it)));
    iters_out(nlhs, plhs, it);
}

static void cmd_info(mxArray **plhs, const mxArray **prhs)
{
    const nufft3d_info in = plan_info(get_plan(prhs[1]));
    static const char *names[] = {"N", "K", "M", "nnz", "J", "u", "alpha", "radial", "taps_per_sample",
                                  "device_bytes"};
    mxArray *s = mxCreateStructMatrix(1, 1, 10, names);
    mxArray *N = mxCreateDoubleMatrix(1, 3, mxREAL), *K = mxCreateDoubleMatrix(1, 3, mxREAL);
    for (int a = 0; a < 3; ++a) {
        mxGetDoubles(N)[a] = in.N[a];
        mxGetDoubles(K)[a] = in.K[a];
    }
    mxSetField(s, 0, "N", N);
    mxSetField(s, 0, "K", K);
    mxSetField(s, 0, "M", mxCreateDoubleScalar((double)in.M));
    mxSetField(s, 0, "nnz", mxCreateDoubleScalar((double)in.nnz));
    mxSetField(s, 0, "J", mxCreateDoubleScalar(in.J));
    mxSetField(s, 0, "u", mxCreateDoubleScalar(in.u));
    mxSetField(s, 0, "alpha", mxCreateDoubleScalar(in.alpha));
    mxSetField(s, 0, "radial", mxCreateDoubleScalar(in.radial));
    mxSetField(s, 0, "taps_per_sample", mxCreateDoubleScalar(in.taps_per_sample));
    mxSetField(s, 0, "device_bytes", mxCreateDoubleScalar((double)in.device_bytes));
    plhs[0] = s;
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    char cmd[16] = {0};
    if (nrhs < 1 || mxGetString(prhs[0], cmd, sizeof cmd) != 0)
        mexErrMsgIdAndTxt("nufft3d:args", "first argument must be a command string");
    if (strcmp(cmd, "create") == 0) {
        cmd_create(nlhs, plhs, nrhs, prhs);
        return;
    }
    if (nrhs < 2) mexErrMsgIdAndTxt("nufft3d:args", "'%s' needs a plan handle", cmd);
    if (strcmp(cmd, "forward") == 0 && nrhs >= 3) {
        cmd_forward(plhs, prhs);
    } else if (strcmp(cmd, "adjoint") == 0 && nrhs >= 3) {
        cmd_adjoint(plhs, prhs);
    } else if (strcmp(cmd, "inverse") == 0) {
        cmd_inverse(nlhs, plhs, nrhs, prhs, 0);
    } else if (strcmp(cmd, "inverse_x0") == 0) {
        cmd_inverse(nlhs, plhs, nrhs, prhs, 1);
    } else if (strcmp(cmd, "inverse_phase") == 0) {
        cmd_inverse_phase(nlhs, plhs, nrhs, prhs);
    } else if (strcmp(cmd, "density") == 0 && nrhs >= 3) {
        CALL(nufft3d_density(get_plan(prhs[1]), (int)mxGetScalar(prhs[2])));
    } else if (strcmp(cmd, "info") == 0) {
        cmd_info(plhs, prhs);
    } else if (strcmp(cmd, "deap") == 0) {
        nufft3d_plan *p = get_plan(prhs[1]);
        const nufft3d_info in = plan_info(p);
        mwSize dims[3] = {(mwSize)in.N[0], (mwSize)in.N[1], (mwSize)in.N[2]};
        plhs[0] = mxCreateNumericArray(3, dims, mxSINGLE_CLASS, mxREAL);
        CALL(nufft3d_get_deap(p, mxGetSingles(plhs[0])));
    } else if (strcmp(cmd, "getd") == 0) {
        nufft3d_plan *p = get_plan(prhs[1]);
        const nufft3d_info in = plan_info(p);
        plhs[0] = mxCreateNumericMatrix((mwSize)in.M, 1, mxSINGLE_CLASS, mxREAL);
        CALL(nufft3d_get_density(p, mxGetSingles(plhs[0])));
    } else if (strcmp(cmd, "destroy") == 0) {
        CALL(nufft3d_plan_destroy(get_plan(prhs[1])));
    } else {
        mexErrMsgIdAndTxt("nufft3d:args", "unknown command '%s' or missing arguments", cmd);
    }
}
