// iNUFT: regridding and the iterative solve of iNUFT.m:119-136.
//
// The reference calls MATLAB's minres on (A'WA + damp^2 I) x = A'W raw with
// tol 1e-4 (iNUFT.m:114-136).  Here each coil is its own Hermitian system
// (the operator is block-diagonal per coil, nufft_3d.m:313) and the Krylov
// recurrences run on the device: vector updates in FP32, every dot product,
// norm and recurrence scalar in FP64, convergence flags per coil on the
// device.  One iteration is captured as a CUDA graph and replayed, so the
// host never synchronises inside the solve.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <string>

#include "internal.h"

namespace nufft3d {

constexpr int kVecThreads = 256;
constexpr int kChunks = 304; // partial sums per coil (2 x 152 SMs)

// per-coil scalar state (doubles)
enum {
    S_RR, S_BN2, S_ALPHA, S_BETA, S_DONE, S_ITERS, S_ACTIVE, S_BETA1, S_CS, S_SN, S_DBAR, S_EPS,
    S_PHIBAR, S_OLDEPS, S_DELTA, S_GAMMA, S_PHI, S_BNEXT, S_TOL, kS = 20
};

__device__ __forceinline__ void reduce_store(double acc, double *out)
{
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[kVecThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < kVecThreads / 32; ++i) s += ws[i];
        *out = s;
    }
}

__device__ __forceinline__ double sum_parts(const double *parts, int c)
{
    double s = 0;
    for (int k = 0; k < kChunks; ++k) s += parts[c * kChunks + k];
    return s;
}

#define VEC_LOOP(i, n) \
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (size_t)gridDim.x * blockDim.x)

__device__ __forceinline__ double rdot(float2 a, float2 b) { return (double)fmaf(a.x, b.x, a.y * b.y); }

// partial[c][chunk] = Re <a, b> over coil c
__global__ void __launch_bounds__(kVecThreads)
k_dot(const float2 *__restrict__ a, const float2 *__restrict__ b, size_t n, double *__restrict__ part)
{
    const int c = blockIdx.y;
    const float2 *A = a + c * n, *B = b + c * n;
    double acc = 0;
    VEC_LOOP(i, n) acc += rdot(A[i], B[i]);
    reduce_store(acc, &part[c * kChunks + blockIdx.x]);
}

__global__ void k_copy_scaled(float2 *__restrict__ dst, const float2 *__restrict__ src, size_t n,
                              const double *__restrict__ scal, int which_inv)
{
    const int c = blockIdx.y;
    double f = 1.0;
    if (which_inv >= 0) {
        const double v = scal[c * kS + which_inv];
        f = v > 0 ? 1.0 / v : 0.0;
    }
    const float ff = (float)f;
    VEC_LOOP(i, n)
    {
        const float2 v = src[c * n + i];
        dst[c * n + i] = make_float2(v.x * ff, v.y * ff);
    }
}

// ------------------------------------------------------------------ CG
__global__ void k_cg_init(const double *__restrict__ part, double *__restrict__ scal, int nc, double tol)
{
    const int c = threadIdx.x;
    if (c >= nc) return;
    double *S = scal + c * kS;
    const double rr = sum_parts(part, c);
    for (int i = 0; i < kS; ++i) S[i] = 0;
    S[S_RR] = rr;
    S[S_BN2] = rr;
    S[S_DONE] = rr == 0 ? 1 : 0;
    S[S_TOL] = tol;
}

__global__ void k_cg_alpha(const double *__restrict__ part, double *__restrict__ scal, int nc)
{
    const int c = threadIdx.x;
    if (c >= nc) return;
    double *S = scal + c * kS;
    const double pq = sum_parts(part, c);
    if (S[S_DONE] != 0 || !(pq > 0)) {
        S[S_DONE] = 1;
        S[S_ALPHA] = 0;
    } else {
        S[S_ALPHA] = S[S_RR] / pq;
    }
}

// x += alpha p; r -= alpha q; partial |r|^2
__global__ void __launch_bounds__(kVecThreads)
k_cg_xr(float2 *__restrict__ x, float2 *__restrict__ r, const float2 *__restrict__ p,
        const float2 *__restrict__ q, size_t n, const double *__restrict__ scal, double *__restrict__ part)
{
    const int c = blockIdx.y;
    const float a = (float)scal[c * kS + S_ALPHA];
    float2 *X = x + c * n, *Rr = r + c * n;
    const float2 *P = p + c * n, *Q = q + c * n;
    double acc = 0;
    VEC_LOOP(i, n)
    {
        float2 xv = X[i], rv = Rr[i];
        const float2 pv = P[i], qv = Q[i];
        if (a != 0.f) {
            xv.x = fmaf(a, pv.x, xv.x);
            xv.y = fmaf(a, pv.y, xv.y);
            rv.x = fmaf(-a, qv.x, rv.x);
            rv.y = fmaf(-a, qv.y, rv.y);
            X[i] = xv;
            Rr[i] = rv;
        }
        acc += rdot(rv, rv);
    }
    reduce_store(acc, &part[c * kChunks + blockIdx.x]);
}

__global__ void k_cg_beta(const double *__restrict__ part, double *__restrict__ scal, int nc)
{
    const int c = threadIdx.x;
    if (c >= nc) return;
    double *S = scal + c * kS;
    const double rr_new = sum_parts(part, c);
    if (S[S_DONE] != 0) {
        S[S_BETA] = 0;
        return;
    }
    S[S_ITERS] += 1;
    const double tol = S[S_TOL];
    if ((tol > 0 && std::sqrt(rr_new) <= tol * std::sqrt(S[S_BN2])) || rr_new == 0) S[S_DONE] = 1;
    S[S_BETA] = rr_new / S[S_RR];
    S[S_RR] = rr_new;
}

// p = r + beta p
__global__ void __launch_bounds__(kVecThreads)
k_cg_p(float2 *__restrict__ p, const float2 *__restrict__ r, size_t n, const double *__restrict__ scal)
{
    const int c = blockIdx.y;
    if (scal[c * kS + S_DONE] != 0) return;
    const float b = (float)scal[c * kS + S_BETA];
    float2 *P = p + c * n;
    const float2 *Rr = r + c * n;
    VEC_LOOP(i, n)
    {
        const float2 rv = Rr[i], pv = P[i];
        P[i] = make_float2(fmaf(b, pv.x, rv.x), fmaf(b, pv.y, rv.y));
    }
}

// -------------------------------------------------------------- MINRES
__global__ void k_mr_init(const double *__restrict__ part, double *__restrict__ scal, int nc, double tol)
{
    const int c = threadIdx.x;
    if (c >= nc) return;
    double *S = scal + c * kS;
    const double b2 = sum_parts(part, c);
    for (int i = 0; i < kS; ++i) S[i] = 0;
    const double beta1 = std::sqrt(b2);
    S[S_BETA1] = beta1;
    S[S_BETA] = beta1;
    S[S_CS] = -1;
    S[S_SN] = 0;
    S[S_PHIBAR] = beta1;
    S[S_DONE] = beta1 == 0 ? 1 : 0;
    S[S_TOL] = tol;
}

// q -= beta * vprev; partial <v, q>
__global__ void __launch_bounds__(kVecThreads)
k_mr_sub1(float2 *__restrict__ q, const float2 *__restrict__ vprev, const float2 *__restrict__ v, size_t n,
          const double *__restrict__ scal, double *__restrict__ part)
{
    const int c = blockIdx.y;
    const float b = (float)scal[c * kS + S_BETA];
    float2 *Q = q + c * n;
    const float2 *VP = vprev + c * n, *V = v + c * n;
    double acc = 0;
    VEC_LOOP(i, n)
    {
        float2 qv = Q[i];
        const float2 vp = VP[i];
        qv.x = fmaf(-b, vp.x, qv.x);
        qv.y = fmaf(-b, vp.y, qv.y);
        Q[i] = qv;
        acc += rdot(V[i], qv);
    }
    reduce_store(acc, &part[c * kChunks + blockIdx.x]);
}

__global__ void k_mr_alpha(const double *__restrict__ part, double *__restrict__ scal, int nc)
{
    const int c = threadIdx.x;
    if (c < nc) scal[c * kS + S_ALPHA] = sum_parts(part, c);
}

// q -= alpha v; partial |q|^2
__global__ void __launch_bounds__(kVecThreads)
k_mr_sub2(float2 *__restrict__ q, const float2 *__restrict__ v, size_t n, const double *__restrict__ scal,
          double *__restrict__ part)
{
    const int c = blockIdx.y;
    const float a = (float)scal[c * kS + S_ALPHA];
    float2 *Q = q + c * n;
    const float2 *V = v + c * n;
    double acc = 0;
    VEC_LOOP(i, n)
    {
        float2 qv = Q[i];
        const float2 vv = V[i];
        qv.x = fmaf(-a, vv.x, qv.x);
        qv.y = fmaf(-a, vv.y, qv.y);
        Q[i] = qv;
        acc += rdot(qv, qv);
    }
    reduce_store(acc, &part[c * kChunks + blockIdx.x]);
}

// Givens rotation of the Lanczos tridiagonal (Paige & Saunders).
__global__ void k_mr_rot(const double *__restrict__ part, double *__restrict__ scal, int nc)
{
    const int c = threadIdx.x;
    if (c >= nc) return;
    double *S = scal + c * kS;
    const double bn = std::sqrt(fmax(sum_parts(part, c), 0.0));
    const bool active = S[S_DONE] == 0;
    S[S_ACTIVE] = active ? 1 : 0;
    if (!active) return;
    const double alpha = S[S_ALPHA], cs = S[S_CS], sn = S[S_SN], dbar = S[S_DBAR];
    S[S_OLDEPS] = S[S_EPS];
    const double delta = cs * dbar + sn * alpha;
    const double gbar = sn * dbar - cs * alpha;
    S[S_EPS] = sn * bn;
    S[S_DBAR] = -cs * bn;
    const double gamma = fmax(hypot(gbar, bn), DBL_EPSILON);
    S[S_CS] = gbar / gamma;
    S[S_SN] = bn / gamma;
    S[S_DELTA] = delta;
    S[S_GAMMA] = gamma;
    S[S_PHI] = S[S_CS] * S[S_PHIBAR];
    S[S_PHIBAR] = S[S_SN] * S[S_PHIBAR];
    S[S_BNEXT] = bn;
    S[S_BETA] = bn;
    S[S_ITERS] += 1;
    const double tol = S[S_TOL];
    if ((tol > 0 && S[S_PHIBAR] <= tol * S[S_BETA1]) || bn == 0) S[S_DONE] = 1;
}

// w = (v - oldeps w1 - delta w2)/gamma; x += phi w; w1 = w2; w2 = w;
// vprev = v; v = q / beta_next
__global__ void __launch_bounds__(kVecThreads)
k_mr_update(float2 *__restrict__ x, float2 *__restrict__ v, float2 *__restrict__ vprev,
            float2 *__restrict__ w1, float2 *__restrict__ w2, const float2 *__restrict__ q, size_t n,
            const double *__restrict__ scal)
{
    const int c = blockIdx.y;
    const double *S = scal + c * kS;
    if (S[S_ACTIVE] == 0) return;
    const float oe = (float)S[S_OLDEPS], de = (float)S[S_DELTA];
    const float ig = (float)(1.0 / S[S_GAMMA]), ph = (float)S[S_PHI];
    const float ib = S[S_BNEXT] > 0 ? (float)(1.0 / S[S_BNEXT]) : 0.f;
    const size_t o = c * n;
    VEC_LOOP(i, n)
    {
        const float2 vv = v[o + i], a1 = w1[o + i], a2 = w2[o + i], qv = q[o + i];
        float2 w;
        w.x = (vv.x - oe * a1.x - de * a2.x) * ig;
        w.y = (vv.y - oe * a1.y - de * a2.y) * ig;
        float2 xv = x[o + i];
        xv.x = fmaf(ph, w.x, xv.x);
        xv.y = fmaf(ph, w.y, xv.y);
        x[o + i] = xv;
        w1[o + i] = a2;
        w2[o + i] = w;
        vprev[o + i] = vv;
        v[o + i] = make_float2(qv.x * ib, qv.y * ib);
    }
}

// Warm start (x0 given): dst = b - A x0, in place over b.
__global__ void __launch_bounds__(kVecThreads)
k_sub_inplace(float2 *__restrict__ b, const float2 *__restrict__ ax, size_t n)
{
    const int c = blockIdx.y;
    VEC_LOOP(i, n)
    {
        const float2 u = b[c * n + i], v = ax[c * n + i];
        b[c * n + i] = make_float2(u.x - v.x, u.y - v.y);
    }
}

// Warm start: stop tests stay relative to |b| (MATLAB minres/pcg with x0):
// CG compares |r| with tol*|b| through S_BN2; MINRES compares its residual
// estimate (which starts at |r0|) with tol*S_BETA1, so the tolerance is
// rescaled by |b|/|r0|.
__global__ void k_warm_ref(const double *__restrict__ part_b, double *__restrict__ scal, int nc, int minres)
{
    const int c = threadIdx.x;
    if (c >= nc) return;
    double *S = scal + c * kS;
    const double b2 = sum_parts(part_b, c);
    if (minres) {
        if (S[S_BETA1] > 0) S[S_TOL] *= std::sqrt(b2) / S[S_BETA1];
    } else {
        S[S_BN2] = b2;
    }
}

__global__ void k_weights(const float *__restrict__ W, const int32_t *__restrict__ perm,
                          const float *__restrict__ d, int64_t nnz, float *__restrict__ ws)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nnz) ws[s] = W[perm[s]] * d[s];
}

__global__ void k_iters_out(const double *__restrict__ scal, int nc, int *__restrict__ out)
{
    const int c = threadIdx.x;
    if (c < nc) out[c] = (int)scal[c * kS + S_ITERS];
}

// ------------------------------------------------------ phase constraint
// iNUFT.m:147-150: P = exp(i angle(convn(x, ones(3), 'same'))).  ones(3) is
// a 3x3 matrix, so the box sum runs over x and y only, slice by slice, with
// zeros outside the image; angle(0) = 0 gives P = 1.
__global__ void k_box_phase(const float2 *__restrict__ x, float2 *__restrict__ P, int N1, int N2, size_t nimg)
{
    const int c = blockIdx.y;
    const float2 *X = x + c * nimg;
    VEC_LOOP(i, nimg)
    {
        const int ix = (int)(i % N1), iy = (int)((i / N1) % N2);
        const size_t slice = i - (size_t)ix - (size_t)iy * N1;
        float sr = 0.f, si = 0.f;
        for (int dy = -1; dy <= 1; ++dy) {
            const int yy = iy + dy;
            if (yy < 0 || yy >= N2) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int xx = ix + dx;
                if (xx < 0 || xx >= N1) continue;
                const float2 v = X[slice + (size_t)yy * N1 + xx];
                sr += v.x;
                si += v.y;
            }
        }
        const float m = sqrtf(sr * sr + si * si);
        P[c * nimg + i] = m > 0.f ? make_float2(sr / m, si / m) : make_float2(1.f, 0.f);
    }
}

// y = P .* x (conj_p = 0) or conj(P) .* x (conj_p = 1), in place allowed
__global__ void k_phase_mul(float2 *__restrict__ y, const float2 *__restrict__ x, const float2 *__restrict__ P,
                            size_t n, int conj_p)
{
    const int c = blockIdx.y;
    VEC_LOOP(i, n)
    {
        const float2 a = x[c * n + i], q = P[c * n + i];
        const float qi = conj_p ? -q.y : q.y;
        y[c * n + i] = make_float2(a.x * q.x - a.y * qi, a.x * qi + a.y * q.x);
    }
}

// nufft_3d.m:333: y = conj(P) .* y + i lambda^2 imag(x)
__global__ void k_phase_finish(float2 *__restrict__ y, const float2 *__restrict__ x, const float2 *__restrict__ P,
                               size_t n, float lam2)
{
    const int c = blockIdx.y;
    VEC_LOOP(i, n)
    {
        const float2 a = y[c * n + i], q = P[c * n + i];
        const float xi = x[c * n + i].y;
        y[c * n + i] = make_float2(a.x * q.x + a.y * q.y, a.y * q.x - a.x * q.y + lam2 * xi);
    }
}

// The phase-constrained normal operator (pprojection, nufft_3d.m:325-334):
// y = P' A'WA (P x) + damp^2 x + i lambda^2 imag(x), real-linear in x.
struct PhaseOp {
    const float2 *P;
    float2 *tmp;
    float lam2;
};

static int apply_normal(nufft3d_plan *p, const float2 *x, float2 *y, int nc, double damp, const float *ws,
                        const PhaseOp *ph, cudaStream_t s)
{
    if (!ph) return op_normal(p, x, y, nc, damp, ws, s);
    const size_t n = p->solver.nimg;
    const dim3 grid(kChunks, nc);
    k_phase_mul<<<grid, kVecThreads, 0, s>>>(ph->tmp, x, ph->P, n, 0);
    NUFFT_TRY(op_normal(p, ph->tmp, y, nc, damp, ws, s));
    k_phase_finish<<<grid, kVecThreads, 0, s>>>(y, x, ph->P, n, ph->lam2);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

// ---------------------------------------------------------------- host
// iNUFT.m:55-74: W = W .* d in sorted order (W = d when none is given).
int prepare_weights(nufft3d_plan *p, const float *W_orig, const float **wsorted, cudaStream_t s)
{
    if (!W_orig) {
        *wsorted = p->d;
        return NUFFT3D_SUCCESS;
    }
    if (!p->wbuf) {
        NUFFT_DEVICE_LOCK;
        NUFFT_CUDA_TRY(cudaMalloc(&p->wbuf, sizeof(float) * (p->nnz > 0 ? p->nnz : 1)));
    }
    if (p->nnz > 0) {
        k_weights<<<(unsigned)((p->nnz + 255) / 256), 256, 0, s>>>(W_orig, p->perm, p->d, p->nnz, p->wbuf);
        NUFFT_CUDA_TRY(cudaGetLastError());
    }
    *wsorted = p->wbuf;
    return NUFFT3D_SUCCESS;
}

int ensure_solver(nufft3d_plan *p, int nc)
{
    SolverWork &w = p->solver;
    const size_t nimg = (size_t)p->N[0] * p->N[1] * p->N[2];
    if (w.nc >= nc && w.nimg == nimg) return NUFFT3D_SUCCESS;
    NUFFT_DEVICE_LOCK;
    float2 **vecs[] = {&w.r, &w.p, &w.q, &w.v, &w.vprev, &w.w1, &w.w2};
    for (auto pp : vecs)
        if (*pp) {
            cudaFree(*pp);
            *pp = nullptr;
        }
    if (w.partial) cudaFree(w.partial);
    if (w.bpart) cudaFree(w.bpart);
    if (w.scal) cudaFree(w.scal);
    if (w.iters) cudaFree(w.iters);
    w = SolverWork();
    for (auto pp : vecs) NUFFT_CUDA_TRY(cudaMalloc((void **)pp, nimg * nc * sizeof(float2)));
    NUFFT_CUDA_TRY(cudaMalloc(&w.partial, sizeof(double) * kChunks * nc));
    NUFFT_CUDA_TRY(cudaMalloc(&w.bpart, sizeof(double) * kChunks * nc));
    NUFFT_CUDA_TRY(cudaMalloc(&w.scal, sizeof(double) * kS * nc));
    NUFFT_CUDA_TRY(cudaMalloc(&w.iters, sizeof(int) * nc));
    w.nc = nc;
    w.nimg = nimg;
    w.nchunk = kChunks;
    return NUFFT3D_SUCCESS;
}

static int cg_iteration(nufft3d_plan *p, float2 *x, int nc, double damp, const float *ws, cudaStream_t s,
                        const PhaseOp *ph = nullptr)
{
    SolverWork &w = p->solver;
    const size_t n = w.nimg;
    const dim3 grid(kChunks, nc);
    NUFFT_TRY(apply_normal(p, w.p, w.q, nc, damp, ws, ph, s));
    k_dot<<<grid, kVecThreads, 0, s>>>(w.p, w.q, n, w.partial);
    k_cg_alpha<<<1, 32 * ((nc + 31) / 32), 0, s>>>(w.partial, w.scal, nc);
    k_cg_xr<<<grid, kVecThreads, 0, s>>>(x, w.r, w.p, w.q, n, w.scal, w.partial);
    k_cg_beta<<<1, 32 * ((nc + 31) / 32), 0, s>>>(w.partial, w.scal, nc);
    k_cg_p<<<grid, kVecThreads, 0, s>>>(w.p, w.r, n, w.scal);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

static int minres_iteration(nufft3d_plan *p, float2 *x, int nc, double damp, const float *ws, cudaStream_t s)
{
    SolverWork &w = p->solver;
    const size_t n = w.nimg;
    const dim3 grid(kChunks, nc);
    const int th1 = 32 * ((nc + 31) / 32);
    NUFFT_TRY(op_normal(p, w.v, w.q, nc, damp, ws, s));
    k_mr_sub1<<<grid, kVecThreads, 0, s>>>(w.q, w.vprev, w.v, n, w.scal, w.partial);
    k_mr_alpha<<<1, th1, 0, s>>>(w.partial, w.scal, nc);
    k_mr_sub2<<<grid, kVecThreads, 0, s>>>(w.q, w.v, n, w.scal, w.partial);
    k_mr_rot<<<1, th1, 0, s>>>(w.partial, w.scal, nc);
    k_mr_update<<<grid, kVecThreads, 0, s>>>(x, w.v, w.vprev, w.w1, w.w2, w.q, n, w.scal);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

// Captures one solver iteration (the operator and the vector kernels) as a
// CUDA graph and replays it maxit times on `own`.
template <typename Body>
static int replay_iterations(cudaStream_t own, int maxit, Body &&body)
{
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int st;
    cudaError_t ce;
    {
        NUFFT_DEVICE_LOCK;
        NUFFT_CUDA_TRY(cudaStreamBeginCapture(own, cudaStreamCaptureModeThreadLocal));
        st = body(own);
        ce = cudaStreamEndCapture(own, &graph);
        if (st == NUFFT3D_SUCCESS && ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
    }
    if (st != NUFFT3D_SUCCESS) {
        if (exec) cudaGraphExecDestroy(exec);
        return st;
    }
    if (ce != cudaSuccess) return fail(NUFFT3D_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    for (int it = 0; it < maxit && ce == cudaSuccess; ++it) ce = cudaGraphLaunch(exec, own);
    cudaGraphExecDestroy(exec);
    if (ce != cudaSuccess) return fail(NUFFT3D_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(ce));
    return NUFFT3D_SUCCESS;
}

int run_inverse(nufft3d_plan *p, const float2 *raw, float2 *x, int nc, int maxit, double damp,
                const float *W_orig, int solver, double tol, int *iters_host, cudaStream_t s, bool warm)
{
    cudaStream_t own = p->own_stream;
    cudaEvent_t ev = nullptr;
    NUFFT_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    struct EvGuard {
        cudaEvent_t e;
        ~EvGuard() { cudaEventDestroy(e); }
    } eg{ev};
    if (s != own) {
        NUFFT_CUDA_TRY(cudaEventRecord(ev, s));
        NUFFT_CUDA_TRY(cudaStreamWaitEvent(own, ev, 0));
    }
    const float *ws = nullptr;
    NUFFT_TRY(prepare_weights(p, W_orig, &ws, own));
    NUFFT_TRY(ensure_scratch(p, nc));
    if (maxit == 0) { // iNUFT.m:119-122 regridding
        NUFFT_TRY(op_adjoint_weighted(p, raw, x, nc, ws, own));
        if (iters_host)
            for (int c = 0; c < nc; ++c) iters_host[c] = 0;
    } else {
        NUFFT_TRY(ensure_solver(p, nc));
        SolverWork &w = p->solver;
        const size_t n = w.nimg;
        const size_t vb = n * nc * sizeof(float2);
        const dim3 grid(kChunks, nc);
        const int th1 = 32 * ((nc + 31) / 32);
        if (!warm) NUFFT_CUDA_TRY(cudaMemsetAsync(x, 0, vb, own));
        // right-hand side b = A'W raw (into r for CG, q for MINRES); with a
        // warm start the partial sums of |b|^2 go to w.bpart and the Krylov
        // start vector becomes b - A x0
        float2 *bvec = solver == NUFFT3D_SOLVER_CG ? w.r : w.q;
        NUFFT_TRY(op_adjoint_weighted(p, raw, bvec, nc, ws, own));
        if (warm) {
            k_dot<<<grid, kVecThreads, 0, own>>>(bvec, bvec, n, w.bpart);
            NUFFT_TRY(op_normal(p, x, w.v, nc, damp, ws, own));         // A x0 (v is reset below)
            k_sub_inplace<<<grid, kVecThreads, 0, own>>>(bvec, w.v, n);
        }
        if (solver == NUFFT3D_SOLVER_CG) {
            NUFFT_CUDA_TRY(cudaMemcpyAsync(w.p, w.r, vb, cudaMemcpyDeviceToDevice, own));
            k_dot<<<grid, kVecThreads, 0, own>>>(w.r, w.r, n, w.partial);
            k_cg_init<<<1, th1, 0, own>>>(w.partial, w.scal, nc, tol);
            if (warm) k_warm_ref<<<1, th1, 0, own>>>(w.bpart, w.scal, nc, 0);
        } else {
            k_dot<<<grid, kVecThreads, 0, own>>>(w.q, w.q, n, w.partial);
            k_mr_init<<<1, th1, 0, own>>>(w.partial, w.scal, nc, tol);
            if (warm) k_warm_ref<<<1, th1, 0, own>>>(w.bpart, w.scal, nc, 1);
            k_copy_scaled<<<grid, kVecThreads, 0, own>>>(w.v, w.q, n, w.scal, S_BETA1);
            NUFFT_CUDA_TRY(cudaMemsetAsync(w.vprev, 0, vb, own));
            NUFFT_CUDA_TRY(cudaMemsetAsync(w.w1, 0, vb, own));
            NUFFT_CUDA_TRY(cudaMemsetAsync(w.w2, 0, vb, own));
        }
        NUFFT_CUDA_TRY(cudaGetLastError());
        NUFFT_TRY(replay_iterations(own, maxit, [&](cudaStream_t cs) {
            return solver == NUFFT3D_SOLVER_CG ? cg_iteration(p, x, nc, damp, ws, cs)
                                               : minres_iteration(p, x, nc, damp, ws, cs);
        }));
        if (iters_host) {
            k_iters_out<<<1, th1, 0, own>>>(w.scal, nc, w.iters);
            NUFFT_CUDA_TRY(cudaGetLastError());
            NUFFT_CUDA_TRY(cudaMemcpyAsync(iters_host, w.iters, sizeof(int) * nc, cudaMemcpyDeviceToHost, own));
            NUFFT_CUDA_TRY(cudaStreamSynchronize(own));
        }
    }
    if (s != own) {
        NUFFT_CUDA_TRY(cudaEventRecord(ev, own));
        NUFFT_CUDA_TRY(cudaStreamWaitEvent(s, ev, 0));
    }
    return NUFFT3D_SUCCESS;
}

// iNUFT.m:140-168, 'phase-constraint': the MINRES image x gives the smooth
// phase P; then (P'A'WAP + damp^2 + lambda^2 imag) y = P'A'W raw is solved
// from y = 0 and the image is P y.  The reference's solver for this
// real-linear system, pcgpc, lives in an external package; here it is
// conjugate gradients with real inner products Re<a, b> (the operator is
// self-adjoint and positive definite for that inner product), FP64 scalars,
// stop on |r| <= tol |b|.
int run_inverse_phase(nufft3d_plan *p, const float2 *raw, float2 *x, int nc, int maxit, double damp, double lambda,
                      const float *W_orig, double tol, int *iters_host, cudaStream_t s)
{
    NUFFT_TRY(run_inverse(p, raw, x, nc, maxit, damp, W_orig, NUFFT3D_SOLVER_MINRES, tol, iters_host, s, false));
    if (maxit <= 1) return NUFFT3D_SUCCESS;  // iNUFT.m:77-78: no effect with maxit <= 1
    cudaStream_t own = p->own_stream;
    cudaEvent_t ev = nullptr;
    NUFFT_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    struct EvGuard {
        cudaEvent_t e;
        ~EvGuard() { cudaEventDestroy(e); }
    } eg{ev};
    if (s != own) {
        NUFFT_CUDA_TRY(cudaEventRecord(ev, s));
        NUFFT_CUDA_TRY(cudaStreamWaitEvent(own, ev, 0));
    }
    const float *ws = nullptr;
    NUFFT_TRY(prepare_weights(p, W_orig, &ws, own));
    NUFFT_TRY(ensure_solver(p, nc));
    SolverWork &w = p->solver;
    const size_t n = w.nimg;
    const size_t vb = n * nc * sizeof(float2);
    const dim3 grid(kChunks, nc);
    const int th1 = 32 * ((nc + 31) / 32);
    PhaseOp ph{w.w1, w.w2, (float)(lambda * lambda)};
    k_box_phase<<<grid, kVecThreads, 0, own>>>(x, w.w1, p->N[0], p->N[1], n);
    NUFFT_TRY(op_adjoint_weighted(p, raw, w.r, nc, ws, own));   // A'W raw
    k_phase_mul<<<grid, kVecThreads, 0, own>>>(w.r, w.r, w.w1, n, 1);  // b = P' A'W raw
    NUFFT_CUDA_TRY(cudaMemsetAsync(x, 0, vb, own));
    NUFFT_CUDA_TRY(cudaMemcpyAsync(w.p, w.r, vb, cudaMemcpyDeviceToDevice, own));
    k_dot<<<grid, kVecThreads, 0, own>>>(w.r, w.r, n, w.partial);
    k_cg_init<<<1, th1, 0, own>>>(w.partial, w.scal, nc, tol);
    NUFFT_CUDA_TRY(cudaGetLastError());
    NUFFT_TRY(replay_iterations(own, maxit, [&](cudaStream_t cs) {
        return cg_iteration(p, x, nc, damp, ws, cs, &ph);
    }));
    k_phase_mul<<<grid, kVecThreads, 0, own>>>(x, x, w.w1, n, 0);  // x = P y
    NUFFT_CUDA_TRY(cudaGetLastError());
    if (iters_host) {
        k_iters_out<<<1, th1, 0, own>>>(w.scal, nc, w.iters);
        NUFFT_CUDA_TRY(cudaGetLastError());
        NUFFT_CUDA_TRY(cudaMemcpyAsync(iters_host, w.iters, sizeof(int) * nc, cudaMemcpyDeviceToHost, own));
        NUFFT_CUDA_TRY(cudaStreamSynchronize(own));
    }
    if (s != own) {
        NUFFT_CUDA_TRY(cudaEventRecord(ev, own));
        NUFFT_CUDA_TRY(cudaStreamWaitEvent(s, ev, 0));
    }
    return NUFFT3D_SUCCESS;
}

} // namespace nufft3d

using namespace nufft3d;

namespace {
struct DevGuardS {
    int prev = -1;
    explicit DevGuardS(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DevGuardS()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int check_inverse(nufft3d_plan *p, const void *raw, const void *x, int nc, int maxit, double damp, int solver)
{
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    if (!raw || !x) return fail(NUFFT3D_ERR_ARG, "NULL data pointer");
    if (nc < 1) return fail(NUFFT3D_ERR_ARG, "number of coils must be >= 1");
    if (maxit < 0) return fail(NUFFT3D_ERR_ARG, "maxit must be a nonnegative integer"); // iNUFT.m:48
    if (!std::isfinite(damp) || damp < 0) return fail(NUFFT3D_ERR_ARG, "damp must be finite and nonnegative"); // iNUFT.m:53
    if (solver != NUFFT3D_SOLVER_MINRES && solver != NUFFT3D_SOLVER_CG)
        return fail(NUFFT3D_ERR_ARG, "unknown solver");
    return NUFFT3D_SUCCESS;
}
} // namespace

extern "C" int nufft3d_inverse(nufft3d_plan *p, const float *raw, float *x, int nc, int maxit, double damp,
                               const float *W, int solver, double tol, int *iters_host, void *stream)
{
    clear_error();
    NUFFT_TRY(check_inverse(p, raw, x, nc, maxit, damp, solver));
    DevGuardS g(p->device);
    return run_inverse(p, (const float2 *)raw, (float2 *)x, nc, maxit, damp, W, solver, tol, iters_host,
                       (cudaStream_t)stream, false);
}

extern "C" int nufft3d_inverse_x0(nufft3d_plan *p, const float *raw, float *x, int nc, int maxit, double damp,
                                  const float *W, int solver, double tol, int *iters_host, void *stream)
{
    clear_error();
    NUFFT_TRY(check_inverse(p, raw, x, nc, maxit, damp, solver));
    DevGuardS g(p->device);
    return run_inverse(p, (const float2 *)raw, (float2 *)x, nc, maxit, damp, W, solver, tol, iters_host,
                       (cudaStream_t)stream, maxit > 0);
}

// lambda >= 0 selects the phase-constrained solve (solver ignored)
static int inverse_host(nufft3d_plan *p, const float *raw, float *x, int nc, int maxit, double damp,
                        const float *W, int solver, double tol, int *iters_host, bool warm, double lambda = -1)
{
    clear_error();
    NUFFT_TRY(check_inverse(p, raw, x, nc, maxit, damp, solver));
    DevGuardS g(p->device);
    if (W) {
        for (int64_t m = 0; m < p->M; ++m)
            if (!std::isfinite(W[m]) || W[m] < 0) return fail(NUFFT3D_ERR_ARG, "W must be finite and nonnegative");
    }
    const size_t braw = (size_t)p->M * nc * sizeof(float2);
    const size_t bW = W ? (size_t)p->M * sizeof(float) : 0;
    const size_t bx = (size_t)p->N[0] * p->N[1] * p->N[2] * nc * sizeof(float2);
    HostStage &h = p->stage;
    if (h.bytes_in < braw + bW + 256 || h.bytes_out < bx) {
        NUFFT_DEVICE_LOCK;
    if (h.bytes_in < braw + bW + 256) {
        if (h.in) cudaFree(h.in);
        h.in = nullptr;
        h.bytes_in = 0;
        NUFFT_CUDA_TRY(cudaMalloc(&h.in, braw + bW + 256));
        h.bytes_in = braw + bW + 256;
    }
    if (h.bytes_out < bx) {
        if (h.out) cudaFree(h.out);
        h.out = nullptr;
        h.bytes_out = 0;
        NUFFT_CUDA_TRY(cudaMalloc(&h.out, bx));
        h.bytes_out = bx;
    }
    }
    cudaStream_t s = p->own_stream;
    char *base = (char *)h.in;
    float *Wd = W ? (float *)(base + ((braw + 255) / 256) * 256) : nullptr;
    NUFFT_CUDA_TRY(cudaMemcpyAsync(base, raw, braw, cudaMemcpyHostToDevice, s));
    if (W) NUFFT_CUDA_TRY(cudaMemcpyAsync(Wd, W, bW, cudaMemcpyHostToDevice, s));
    if (warm) NUFFT_CUDA_TRY(cudaMemcpyAsync(h.out, x, bx, cudaMemcpyHostToDevice, s));
    if (lambda >= 0)
        NUFFT_TRY(run_inverse_phase(p, (const float2 *)base, (float2 *)h.out, nc, maxit, damp, lambda, Wd, tol,
                                    iters_host, s));
    else
        NUFFT_TRY(run_inverse(p, (const float2 *)base, (float2 *)h.out, nc, maxit, damp, Wd, solver, tol,
                              iters_host, s, warm));
    NUFFT_CUDA_TRY(cudaMemcpyAsync(x, h.out, bx, cudaMemcpyDeviceToHost, s));
    NUFFT_TRY(plan_check_status(p, s));
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_inverse_host(nufft3d_plan *p, const float *raw, float *x, int nc, int maxit,
                                    double damp, const float *W, int solver, double tol, int *iters_host)
{
    return inverse_host(p, raw, x, nc, maxit, damp, W, solver, tol, iters_host, false);
}

extern "C" int nufft3d_inverse_x0_host(nufft3d_plan *p, const float *raw, float *x, int nc, int maxit,
                                       double damp, const float *W, int solver, double tol, int *iters_host)
{
    return inverse_host(p, raw, x, nc, maxit, damp, W, solver, tol, iters_host, maxit > 0);
}

extern "C" int nufft3d_inverse_phase(nufft3d_plan *p, const float *raw, float *x, int nc, int maxit, double damp,
                                     double lambda, const float *W, double tol, int *iters_host, void *stream)
{
    clear_error();
    NUFFT_TRY(check_inverse(p, raw, x, nc, maxit, damp, NUFFT3D_SOLVER_MINRES));
    if (!std::isfinite(lambda) || lambda < 0) return fail(NUFFT3D_ERR_ARG, "lambda must be finite and nonnegative");
    DevGuardS g(p->device);
    return run_inverse_phase(p, (const float2 *)raw, (float2 *)x, nc, maxit, damp, lambda, W, tol, iters_host,
                             (cudaStream_t)stream);
}

extern "C" int nufft3d_inverse_phase_host(nufft3d_plan *p, const float *raw, float *x, int nc, int maxit,
                                          double damp, double lambda, const float *W, double tol, int *iters_host)
{
    if (!std::isfinite(lambda) || lambda < 0) {
        clear_error();
        return fail(NUFFT3D_ERR_ARG, "lambda must be finite and nonnegative");
    }
    return inverse_host(p, raw, x, nc, maxit, damp, W, NUFFT3D_SOLVER_MINRES, tol, iters_host, false, lambda);
}
