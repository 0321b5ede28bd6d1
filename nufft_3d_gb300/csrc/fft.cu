// Oversampled 3-D FFT of fNUFT / aNUFT as three pruned line passes.
//
// Replaces fft3_pad / ifft3_crop of @nufft_3d/nufft_3d.m:285-302 (cuFFT via
// gpuArray in the reference).  Per axis j the reference zero-pads (K-N)/2 on
// both sides, fftshifts and takes a length-K FFT; the inverse takes an
// unnormalised inverse FFT (ifft * K), ifftshifts and crops the central N.
// Both shifts reduce to a slot map: image index n (0..N-1) <-> FFT slot
// (n - N/2) mod K, so no padded array is ever materialised.
//
// Layouts (complex64, coil fastest inside the library):
//   image  [nc][N3][N2][N1]   (MATLAB [N1 N2 N3 nc])
//   B1     [N3][N2][K1][nc]   after the x pass
//   B2     [N3][K2][K1][nc]   after the y pass
//   G      [K3][K2][K1][nc]   oversampled grid
// Forward: FX (image*U -> B1), FY (B1 -> B2), FZ (B2 -> G).
// Adjoint: IZ (G -> B2), IY (B2 -> B1), IX (B1 -> image, *U*scale).
//
// Each block runs a mixed-radix Stockham FFT (radix 2,3,4,5,7,8,11,13) on a
// batch of lines held in shared memory; the inverse is conj(FFT(conj(x))).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "internal.h"

namespace nufft3d {

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// multiply by -i
__device__ __forceinline__ float2 cmi(float2 a) { return make_float2(a.y, -a.x); }

template <int R>
__device__ __forceinline__ void dft(float2 (&u)[R], const float2 *__restrict__ tw, int n)
{
    // generic small prime: y_q = sum_t u_t W_R^{qt}, W from the length-n table
    float2 y[R];
    const int step = n / R;
#pragma unroll
    for (int q = 0; q < R; ++q) {
        float2 acc = u[0];
#pragma unroll
        for (int t = 1; t < R; ++t) acc = cadd(acc, cmul(u[t], __ldg(&tw[((q * t) % R) * step])));
        y[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) u[q] = y[q];
}

template <>
__device__ __forceinline__ void dft<2>(float2 (&u)[2], const float2 *__restrict__, int)
{
    float2 a = u[0], b = u[1];
    u[0] = cadd(a, b);
    u[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft<3>(float2 (&u)[3], const float2 *__restrict__, int)
{
    const float s3 = 0.86602540378443864676f; // sin(2 pi / 3)
    float2 t = cadd(u[1], u[2]);
    float2 d = csub(u[1], u[2]);
    float2 y0 = cadd(u[0], t);
    float2 m = make_float2(u[0].x - 0.5f * t.x, u[0].y - 0.5f * t.y);
    float2 s = make_float2(s3 * d.y, -s3 * d.x); // -i * s3 * d
    u[0] = y0;
    u[1] = cadd(m, s);
    u[2] = csub(m, s);
}

template <>
__device__ __forceinline__ void dft<4>(float2 (&u)[4], const float2 *__restrict__, int)
{
    float2 t0 = cadd(u[0], u[2]), t1 = csub(u[0], u[2]);
    float2 t2 = cadd(u[1], u[3]), t3 = cmi(csub(u[1], u[3]));
    u[0] = cadd(t0, t2);
    u[2] = csub(t0, t2);
    u[1] = cadd(t1, t3);
    u[3] = csub(t1, t3);
}

template <>
__device__ __forceinline__ void dft<5>(float2 (&u)[5], const float2 *__restrict__, int)
{
    const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
    const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
    float2 t1 = cadd(u[1], u[4]), t2 = cadd(u[2], u[3]);
    float2 t3 = csub(u[1], u[4]), t4 = csub(u[2], u[3]);
    float2 y0 = cadd(u[0], cadd(t1, t2));
    float2 b1 = make_float2(u[0].x + c1 * t1.x + c2 * t2.x, u[0].y + c1 * t1.y + c2 * t2.y);
    float2 b2 = make_float2(u[0].x + c2 * t1.x + c1 * t2.x, u[0].y + c2 * t1.y + c1 * t2.y);
    float2 e1 = make_float2(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    float2 e2 = make_float2(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
    float2 d1 = cmi(e1), d2 = cmi(e2);
    u[0] = y0;
    u[1] = cadd(b1, d1);
    u[4] = csub(b1, d1);
    u[2] = cadd(b2, d2);
    u[3] = csub(b2, d2);
}

template <>
__device__ __forceinline__ void dft<8>(float2 (&u)[8], const float2 *__restrict__ tw, int n)
{
    // radix-2 split: evens and odds through radix-4, combined with W8^k
    float2 e[4] = {u[0], u[2], u[4], u[6]};
    float2 o[4] = {u[1], u[3], u[5], u[7]};
    dft<4>(e, tw, n);
    dft<4>(o, tw, n);
    const float h = 0.70710678118654752440f;
    float2 o1 = make_float2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x)); // * (1-i)/sqrt2
    float2 o2 = cmi(o[2]);                                                   // * -i
    float2 o3 = make_float2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y)); // * (-1-i)/sqrt2
    u[0] = cadd(e[0], o[0]);
    u[4] = csub(e[0], o[0]);
    u[1] = cadd(e[1], o1);
    u[5] = csub(e[1], o1);
    u[2] = cadd(e[2], o2);
    u[6] = csub(e[2], o2);
    u[3] = cadd(e[3], o3);
    u[7] = csub(e[3], o3);
}

// One Stockham stage: lines of length n, stride LS; p = product of the
// radices already applied.  Output position j + q*p with j = (i-k)*R + k.
template <int R>
__device__ __forceinline__ void fft_stage(const float2 *__restrict__ a, float2 *__restrict__ b,
                                          int nlines, int LS, int n, int p,
                                          const float2 *__restrict__ tw)
{
    const int m = n / R;
    const int total = nlines * m;
    const int twstep = n / (p * R);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int line = t / m;
        const int i = t - line * m;
        const int k = i % p;
        const float2 *src = a + line * LS;
        float2 *dst = b + line * LS;
        float2 u[R];
#pragma unroll
        for (int q = 0; q < R; ++q) u[q] = src[i + q * m];
        if (k) {
#pragma unroll
            for (int q = 1; q < R; ++q) u[q] = cmul(u[q], __ldg(&tw[q * k * twstep]));
        }
        dft<R>(u, tw, n);
        const int j = (i - k) * R + k;
#pragma unroll
        for (int q = 0; q < R; ++q) dst[j + q * p] = u[q];
    }
}

// Forward FFT of `nlines` lines held in a (stride LS); b is the ping-pong
// buffer.  Returns the buffer holding the result.  RARE enables the radix
// 7/11/13 stages (only sizes with such factors pay their register cost).
template <bool RARE>
__device__ float2 *block_fft(float2 *a, float2 *b, int nlines, int LS, const FFTDesc &f)
{
    int p = 1;
    for (int s = 0; s < f.nst; ++s) {
        const int r = f.rad[s];
        switch (r) {
        case 2: fft_stage<2>(a, b, nlines, LS, f.n, p, f.tw); break;
        case 3: fft_stage<3>(a, b, nlines, LS, f.n, p, f.tw); break;
        case 4: fft_stage<4>(a, b, nlines, LS, f.n, p, f.tw); break;
        case 5: fft_stage<5>(a, b, nlines, LS, f.n, p, f.tw); break;
        case 8: fft_stage<8>(a, b, nlines, LS, f.n, p, f.tw); break;
        default:
            if (RARE) {
                if (r == 7) fft_stage<7>(a, b, nlines, LS, f.n, p, f.tw);
                else if (r == 11) fft_stage<11>(a, b, nlines, LS, f.n, p, f.tw);
                else if (r == 13) fft_stage<13>(a, b, nlines, LS, f.n, p, f.tw);
            }
            break;
        }
        __syncthreads();
        float2 *t = a;
        a = b;
        b = t;
        p *= r;
    }
    return a;
}

bool needs_rare(const FFTDesc &f)
{
    for (int s = 0; s < f.nst; ++s)
        if (f.rad[s] == 7 || f.rad[s] == 11 || f.rad[s] == 13) return true;
    return false;
}

__device__ __forceinline__ int slot_of(int n, int N, int K)
{
    int s = n - N / 2;
    return s < 0 ? s + K : s;
}

// ------------------------------------------------ four-step line passes
// In-register DFTs of 12, 16, 20 and 24 points built from the radix 3/4/5/8
// butterflies (n = B*a + b, k = ka + A*kb), with the W_AB twiddles read from
// constant memory at compile-time indices (tables filled once per device from
// FP64 values).
__constant__ float2 c_w12[12];
__constant__ float2 c_w16[16];
__constant__ float2 c_w20[20];
__constant__ float2 c_w24[24];

template <int N>
__device__ __forceinline__ float2 wconst(int j);
template <> __device__ __forceinline__ float2 wconst<12>(int j) { return c_w12[j]; }
template <> __device__ __forceinline__ float2 wconst<16>(int j) { return c_w16[j]; }
template <> __device__ __forceinline__ float2 wconst<20>(int j) { return c_w20[j]; }
template <> __device__ __forceinline__ float2 wconst<24>(int j) { return c_w24[j]; }

template <int A, int B>
__device__ __forceinline__ void dft_comp(float2 (&u)[A * B])
{
    float2 t[A * B];
#pragma unroll
    for (int b = 0; b < B; ++b) {
        float2 v[A];
#pragma unroll
        for (int a = 0; a < A; ++a) v[a] = u[B * a + b];
        dft<A>(v, nullptr, 0);
#pragma unroll
        for (int ka = 0; ka < A; ++ka) {
            float2 x = v[ka];
            if (b != 0 && ka != 0) x = cmul(x, wconst<A * B>((b * ka) % (A * B)));
            t[b * A + ka] = x;
        }
    }
#pragma unroll
    for (int ka = 0; ka < A; ++ka) {
        float2 v[B];
#pragma unroll
        for (int b = 0; b < B; ++b) v[b] = t[b * A + ka];
        dft<B>(v, nullptr, 0);
#pragma unroll
        for (int kb = 0; kb < B; ++kb) u[ka + A * kb] = v[kb];
    }
}

template <int R>
__device__ __forceinline__ void dft_reg(float2 (&u)[R]);
template <> __device__ __forceinline__ void dft_reg<8>(float2 (&u)[8]) { dft<8>(u, nullptr, 0); }
template <> __device__ __forceinline__ void dft_reg<12>(float2 (&u)[12]) { dft_comp<3, 4>(u); }
template <> __device__ __forceinline__ void dft_reg<16>(float2 (&u)[16]) { dft_comp<4, 4>(u); }
template <> __device__ __forceinline__ void dft_reg<20>(float2 (&u)[20]) { dft_comp<4, 5>(u); }
template <> __device__ __forceinline__ void dft_reg<24>(float2 (&u)[24]) { dft_comp<3, 8>(u); }

// Strided pass (y or z) for K = R1 * 16 over lp.vec = 16 contiguous lines:
// X[k1 + R1 k2] = sum_n2 W16^(n2 k2) W_K^(n2 k1) sum_n1 x[16 n1 + n2] W_R1^(n1 k1).
// Pass 1 (lanes over lines, n2 outer): DFT_R1 in registers, twiddle, store to
// shared memory; pass 2: DFT_16 in registers, store.  Lane -> line mapping
// keeps global accesses coalesced (a line is one complex of a contiguous row)
// and the row stride K+1 keeps shared-memory accesses conflict-free.
template <int R1>
__device__ __forceinline__ void line4_body(const float2 *__restrict__ in, float2 *__restrict__ out,
                                           const LinePass &lp, const float2 *__restrict__ twg, int inv, int blk,
                                           float2 *sm)
{
    constexpr int R2 = 16, K = R1 * R2, L = 16, LS = K + 1;
    float2 *Y = sm;
    float2 *tw = sm + L * LS;
    for (int t = threadIdx.x; t < K; t += blockDim.x) tw[t] = twg[t];
    const int outer = blk / lp.nchunks;
    const int chunk = blk - outer * lp.nchunks;
    const float2 *ib = in + outer * lp.in_outer_stride + (int64_t)chunk * L;
    float2 *ob = out + outer * lp.out_outer_stride + (int64_t)chunk * L;
    const float sg = inv ? -1.f : 1.f;
    // slot map (n - N/2) mod K: slots [0, N - N/2) hold n = slot + N/2,
    // slots [K - N/2, K) hold n = slot - (K - N/2), the rest are zero padding
    const int Nh = lp.Nimg / 2, Nt = lp.Nimg - Nh;
    __syncthreads();
    for (int it = threadIdx.x; it < L * R2; it += blockDim.x) {
        const int line = it % L, n2 = it / L;
        float2 u[R1];
#pragma unroll
        for (int n1 = 0; n1 < R1; ++n1) {
            const int pos = n2 + R2 * n1;
            int src = pos;
            if (lp.pad_in) src = pos < Nt ? pos + Nh : (pos >= K - Nh ? pos - (K - Nh) : -1);
            float2 v = make_float2(0.f, 0.f);
            if (src >= 0) {
                v = ib[(int64_t)src * lp.in_axis_stride + line];
                v.y *= sg;
            }
            u[n1] = v;
        }
        dft_reg<R1>(u);
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) {
            float2 x = u[k1];
            if (k1) x = cmul(x, tw[n2 * k1]);
            Y[line * LS + k1 * R2 + n2] = x;
        }
    }
    __syncthreads();
    for (int it = threadIdx.x; it < L * R1; it += blockDim.x) {
        const int line = it % L, k1 = it / L;
        float2 u[R2];
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) u[n2] = Y[line * LS + k1 * R2 + n2];
        dft_reg<R2>(u);
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) {
            const int k = k1 + R1 * k2;
            int dst = k;
            if (lp.crop_out) dst = k < Nt ? k + Nh : (k >= K - Nh ? k - (K - Nh) : -1);
            if (dst >= 0) {
                const float2 r = u[k2];
                ob[(int64_t)dst * lp.out_axis_stride + line] = make_float2(r.x, sg * r.y);
            }
        }
    }
}

template <int R1>
__global__ void __launch_bounds__(384)
k_line4(const float2 *__restrict__ in, float2 *__restrict__ out, LinePass lp, const float2 *__restrict__ twg,
        int inv)
{
    extern __shared__ float2 sm[];
    line4_body<R1>(in, out, lp, twg, inv, blockIdx.x, sm);
}

// x passes as register four-step FFTs (K = 16*R1).  A block takes 16 lines,
// a line being one (row yz, coil c) pair with the coil fastest, so any coil
// count fills the blocks.  Forward (fNUFT.m:5 + nufft_3d.m:287-289, j=1):
// image rows are contiguous, so the first phase reads with the point index
// fastest (pad, shift and *U on the way in), and the coil-interleaved B1 is
// written with the line index fastest.  Inverse (nufft_3d.m:296-298, j=1 +
// aNUFT.m:8-9): B1 is read with the line index fastest and the rows go out
// through shared memory in a third phase, contiguous, with the crop, *U*scale
// and the optional addend; conj(FFT(conj x)) as in the other passes.
template <int R1, bool INV>
__global__ void __launch_bounds__(384)
k_xline4(const float2 *__restrict__ in, float2 *__restrict__ out, const float *__restrict__ U,
         const float2 *__restrict__ twg, int N1, int64_t N23, int nc, int64_t nlines, float scale,
         const float2 *__restrict__ addend, float add_coef)
{
    constexpr int R2 = 16, K = R1 * R2, L = 16, LS = K + 1;
    extern __shared__ float2 sm[];
    float2 *Y = sm;
    float2 *tw = sm + L * LS;
    __shared__ int64_t rowb[L], intl[L];  // per line: image row start (c*N23 + yz)*N1, interleaved start yz*K*nc + c
    __shared__ int64_t ub[L];             // U row start yz*N1, or -1 past the last line
    for (int t = threadIdx.x; t < K; t += blockDim.x) tw[t] = twg[t];
    if (threadIdx.x < L) {
        const int64_t g = (int64_t)blockIdx.x * L + threadIdx.x;
        if (g < nlines) {
            const int64_t yz = g / nc;
            const int c = (int)(g - yz * nc);
            rowb[threadIdx.x] = ((int64_t)c * N23 + yz) * N1;
            intl[threadIdx.x] = yz * K * nc + c;
            ub[threadIdx.x] = yz * N1;
        } else {
            rowb[threadIdx.x] = intl[threadIdx.x] = 0;
            ub[threadIdx.x] = -1;
        }
    }
    const int Nh = N1 / 2, Nt = N1 - Nh;
    __syncthreads();
    // phase 1: DFT_R1 of the points n2 + 16*n1 of each column n2
    for (int it = threadIdx.x; it < L * R2; it += blockDim.x) {
        const int line = INV ? it % L : it / R2, n2 = INV ? it / L : it % R2;
        const bool live = ub[line] >= 0;
        float2 u[R1];
#pragma unroll
        for (int n1 = 0; n1 < R1; ++n1) {
            const int pos = n2 + R2 * n1;
            float2 v = make_float2(0.f, 0.f);
            if (live) {
                if (INV) {
                    v = in[intl[line] + (int64_t)pos * nc];
                    v.y = -v.y;
                } else {
                    // slot map (n - N1/2) mod K: slots [0, Nt) hold n = slot + N1/2,
                    // slots [K - N1/2, K) hold n = slot - (K - N1/2), the rest zero padding
                    const int src = pos < Nt ? pos + Nh : (pos >= K - Nh ? pos - (K - Nh) : -1);
                    if (src >= 0) {
                        const float2 x = in[rowb[line] + src];
                        const float w = __ldg(&U[ub[line] + src]);
                        v = make_float2(x.x * w, x.y * w);
                    }
                }
            }
            u[n1] = v;
        }
        dft_reg<R1>(u);
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) {
            float2 x = u[k1];
            if (k1) x = cmul(x, tw[n2 * k1]);
            Y[line * LS + k1 * R2 + n2] = x;
        }
    }
    __syncthreads();
    // phase 2: DFT_16 along each row of the exchange (one item per thread:
    // blockDim >= 16*R1)
    const bool act = threadIdx.x < L * R1;
    const int line = threadIdx.x % L, k1 = threadIdx.x / L;
    float2 u[R2];
    if (act) {
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) u[n2] = Y[line * LS + k1 * R2 + n2];
        dft_reg<R2>(u);
    }
    if (!INV) {
        if (act && ub[line] >= 0) {
            float2 *ob = out + intl[line];
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) ob[(int64_t)(k1 + R1 * k2) * nc] = u[k2];
        }
        return;
    }
    __syncthreads();  // every row has been read
    if (act) {
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) Y[line * LS + k1 + R1 * k2] = u[k2];
    }
    __syncthreads();
    // phase 3: contiguous rows out
    for (int it = threadIdx.x; it < L * N1; it += blockDim.x) {
        const int ln = it / N1, n = it - ln * N1;
        if (ub[ln] < 0) continue;
        const float2 r = Y[ln * LS + slot_of(n, N1, K)];
        const float w = __ldg(&U[ub[ln] + n]) * scale;
        const int64_t idx = rowb[ln] + n;
        float2 o = make_float2(r.x * w, -r.y * w);
        if (addend) {
            const float2 a = addend[idx];
            o.x = fmaf(add_coef, a.x, o.x);
            o.y = fmaf(add_coef, a.y, o.y);
        }
        out[idx] = o;
    }
}

template <bool INV>
static int launch_xline4(int r1, const float2 *in, float2 *out, const float *U, const FFTDesc &fd, int N1,
                         int64_t N23, int nc, float scale, const float2 *addend, float add_coef, cudaStream_t s)
{
    const int K = fd.n;
    const int threads = 16 * (r1 > 16 ? r1 : 16);
    const size_t smem = (size_t)(16 * (K + 1) + K) * sizeof(float2);
    const int64_t nlines = N23 * nc;
    const unsigned nblk = (unsigned)((nlines + 15) / 16);
    switch (r1) {
    case 8: k_xline4<8, INV><<<nblk, threads, smem, s>>>(in, out, U, fd.tw, N1, N23, nc, nlines, scale, addend, add_coef); break;
    case 12: k_xline4<12, INV><<<nblk, threads, smem, s>>>(in, out, U, fd.tw, N1, N23, nc, nlines, scale, addend, add_coef); break;
    case 16: k_xline4<16, INV><<<nblk, threads, smem, s>>>(in, out, U, fd.tw, N1, N23, nc, nlines, scale, addend, add_coef); break;
    case 20: k_xline4<20, INV><<<nblk, threads, smem, s>>>(in, out, U, fd.tw, N1, N23, nc, nlines, scale, addend, add_coef); break;
    default: k_xline4<24, INV><<<nblk, threads, smem, s>>>(in, out, U, fd.tw, N1, N23, nc, nlines, scale, addend, add_coef); break;
    }
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

static int four_step_r1(int K, int vec)
{
    if (vec != 16) return 0;
    switch (K) {
    case 128: return 8;
    case 192: return 12;
    case 256: return 16;
    case 320: return 20;
    case 384: return 24;
    default: return 0;
    }
}

static size_t line4_smem(int K) { return (size_t)(16 * (K + 1) + K) * sizeof(float2); }

static int launch_line4(int r1, const float2 *in, float2 *out, const LinePass &lp, const FFTDesc &fd, int inv,
                        int64_t nblk, cudaStream_t s)
{
    const int K = fd.n;
    const int threads = 16 * (r1 > 16 ? r1 : 16);
    const size_t smem = line4_smem(K);
    switch (r1) {
    case 8: k_line4<8><<<(unsigned)nblk, threads, smem, s>>>(in, out, lp, fd.tw, inv); break;
    case 12: k_line4<12><<<(unsigned)nblk, threads, smem, s>>>(in, out, lp, fd.tw, inv); break;
    case 16: k_line4<16><<<(unsigned)nblk, threads, smem, s>>>(in, out, lp, fd.tw, inv); break;
    case 20: k_line4<20><<<(unsigned)nblk, threads, smem, s>>>(in, out, lp, fd.tw, inv); break;
    default: k_line4<24><<<(unsigned)nblk, threads, smem, s>>>(in, out, lp, fd.tw, inv); break;
    }
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

int configure_fft_constants()
{
    auto fill = [](const void *sym, int n) {
        std::vector<float2> w(n);
        for (int j = 0; j < n; ++j) {
            const double a = -2.0 * M_PI * j / n;
            w[j] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        return cudaMemcpyToSymbol(sym, w.data(), n * sizeof(float2));
    };
    NUFFT_CUDA_TRY(fill(c_w12, 12));
    NUFFT_CUDA_TRY(fill(c_w16, 16));
    NUFFT_CUDA_TRY(fill(c_w20, 20));
    NUFFT_CUDA_TRY(fill(c_w24, 24));
    return NUFFT3D_SUCCESS;
}

// ------------------------------------------------------------- kernels
constexpr int kFftThreads = 256;
constexpr int kMaxLineCoils = 16;

// FX: image (user layout) * U -> B1, length-K1 FFT along x for one (y,z) line
// of up to kMaxLineCoils coils.  fNUFT.m:5 + nufft_3d.m:287-289 (j=1).
template <bool RARE>
__device__ __forceinline__ void fx_body(const float2 *__restrict__ img, const float *__restrict__ U,
                                        float2 *__restrict__ B1, int N1, int N23, int nc,
                                        const FFTDesc &fd, int line, int cchunk, float2 *sm)
{
    const int K = fd.n, LS = K + 1;
    const int c0 = cchunk * kMaxLineCoils;
    const int nv = min(kMaxLineCoils, nc - c0);
    float2 *A = sm, *B = sm + nv * LS;
    const int nz = K - N1;
    for (int t = threadIdx.x; t < nz * nv; t += blockDim.x) {
        const int v = t / nz, j = t - v * nz;
        A[v * LS + N1 / 2 + j] = make_float2(0.f, 0.f);
    }
    const float *Ur = U + (size_t)line * N1;
    for (int t = threadIdx.x; t < N1 * nv; t += blockDim.x) {
        const int v = t / N1, n = t - v * N1;
        float2 val = img[((size_t)(c0 + v) * N23 + line) * N1 + n];
        const float w = __ldg(&Ur[n]);
        A[v * LS + slot_of(n, N1, K)] = make_float2(val.x * w, val.y * w);
    }
    __syncthreads();
    const float2 *res = block_fft<RARE>(A, B, nv, LS, fd);
    float2 *ob = B1 + (size_t)line * K * nc + c0;
    for (int t = threadIdx.x; t < K * nv; t += blockDim.x) {
        const int k = t / nv, v = t - k * nv;
        ob[(size_t)k * nc + v] = res[v * LS + k];
    }
}

template <bool RARE>
__global__ void __launch_bounds__(kFftThreads)
k_fx(const float2 *__restrict__ img, const float *__restrict__ U, float2 *__restrict__ B1,
     int N1, int N23, int nc, FFTDesc fd)
{
    extern __shared__ float2 sm[];
    fx_body<RARE>(img, U, B1, N1, N23, nc, fd, blockIdx.x, blockIdx.y, sm);
}

// IX: B1 -> image, unnormalised inverse FFT along x, crop, *U*scale
// (+ add_coef * addend).  nufft_3d.m:296-298 (j=1) + aNUFT.m:8-9.
template <bool RARE>
__device__ __forceinline__ void ix_body(const float2 *__restrict__ B1, const float *__restrict__ U,
                                        float2 *__restrict__ img, int N1, int N23, int nc,
                                        const FFTDesc &fd, float scale, const float2 *__restrict__ addend,
                                        float add_coef, int line, int cchunk, float2 *sm)
{
    const int K = fd.n, LS = K + 1;
    const int c0 = cchunk * kMaxLineCoils;
    const int nv = min(kMaxLineCoils, nc - c0);
    float2 *A = sm, *B = sm + nv * LS;
    const float2 *ib = B1 + (size_t)line * K * nc + c0;
    for (int t = threadIdx.x; t < K * nv; t += blockDim.x) {
        const int k = t / nv, v = t - k * nv;
        float2 val = ib[(size_t)k * nc + v];
        A[v * LS + k] = make_float2(val.x, -val.y);
    }
    __syncthreads();
    const float2 *res = block_fft<RARE>(A, B, nv, LS, fd);
    const float *Ur = U + (size_t)line * N1;
    for (int t = threadIdx.x; t < N1 * nv; t += blockDim.x) {
        const int v = t / N1, n = t - v * N1;
        const float2 r = res[v * LS + slot_of(n, N1, K)];
        const float w = __ldg(&Ur[n]) * scale;
        const size_t idx = ((size_t)(c0 + v) * N23 + line) * N1 + n;
        float2 o = make_float2(r.x * w, -r.y * w);
        if (addend) {
            const float2 a = addend[idx];
            o.x = fmaf(add_coef, a.x, o.x);
            o.y = fmaf(add_coef, a.y, o.y);
        }
        img[idx] = o;
    }
}

template <bool RARE>
__global__ void __launch_bounds__(kFftThreads)
k_ix(const float2 *__restrict__ B1, const float *__restrict__ U, float2 *__restrict__ img,
     int N1, int N23, int nc, FFTDesc fd, float scale, const float2 *__restrict__ addend,
     float add_coef)
{
    extern __shared__ float2 sm[];
    ix_body<RARE>(B1, U, img, N1, N23, nc, fd, scale, addend, add_coef, blockIdx.x, blockIdx.y, sm);
}

// Strided pass along y or z over rows of contiguous complex vectors.
template <bool RARE>
__device__ __forceinline__ void line_body(const float2 *__restrict__ in, float2 *__restrict__ out,
                                          const LinePass &lp, const FFTDesc &fd, int inv, int blk,
                                          float2 *sm)
{
    const int K = fd.n, LS = K + 1, vec = lp.vec;
    float2 *A = sm, *B = sm + vec * LS;
    const int outer = blk / lp.nchunks;
    const int chunk = blk - outer * lp.nchunks;
    const float2 *ib = in + outer * lp.in_outer_stride + (int64_t)chunk * vec;
    float2 *ob = out + outer * lp.out_outer_stride + (int64_t)chunk * vec;
    const float sg = inv ? -1.f : 1.f;
    if (lp.pad_in) {
        const int nz = K - lp.Nimg;
        for (int t = threadIdx.x; t < nz * vec; t += blockDim.x) {
            const int v = t / nz, j = t - v * nz;
            A[v * LS + lp.Nimg / 2 + j] = make_float2(0.f, 0.f);
        }
    }
    for (int t = threadIdx.x; t < lp.n_in * vec; t += blockDim.x) {
        const int i = t / vec, v = t - i * vec;
        const float2 val = ib[(int64_t)i * lp.in_axis_stride + v];
        const int slot = lp.pad_in ? slot_of(i, lp.Nimg, K) : i;
        A[v * LS + slot] = make_float2(val.x, sg * val.y);
    }
    __syncthreads();
    const float2 *res = block_fft<RARE>(A, B, vec, LS, fd);
    for (int t = threadIdx.x; t < lp.n_out * vec; t += blockDim.x) {
        const int o = t / vec, v = t - o * vec;
        const int slot = lp.crop_out ? slot_of(o, lp.Nimg, K) : o;
        const float2 r = res[v * LS + slot];
        ob[(int64_t)o * lp.out_axis_stride + v] = make_float2(r.x, sg * r.y);
    }
}

template <bool RARE>
__global__ void __launch_bounds__(kFftThreads)
k_line(const float2 *__restrict__ in, float2 *__restrict__ out, LinePass lp, FFTDesc fd, int inv)
{
    extern __shared__ float2 sm[];
    line_body<RARE>(in, out, lp, fd, inv, blockIdx.x, sm);
}

// ----------------------------------------------------------------- host
bool fft_factor(int n, FFTDesc &d)
{
    d.n = n;
    d.nst = 0;
    int m = n;
    const int order[] = {8, 4, 2, 3, 5, 7, 11, 13};
    for (int r : order) {
        while (m % r == 0 && d.nst < 16) {
            // a lone factor 2 after 8s is fine; prefer 4 over 2*2
            d.rad[d.nst++] = r;
            m /= r;
        }
    }
    return m == 1;
}

int line_vec(int64_t rowlen)
{
    const int cands[] = {16, 8, 4, 2, 1};
    for (int v : cands)
        if (rowlen % v == 0) return v;
    return 1;
}

size_t line_smem(int vec, int K) { return (size_t)2 * vec * (K + 1) * sizeof(float2); }

LinePass make_linepass(int n_outer, int64_t rowlen, int n_in, int n_out, int Nimg, int pad_in, int crop_out,
                       int64_t in_axis, int64_t out_axis, int64_t in_outer, int64_t out_outer, int64_t *nblk)
{
    LinePass lp;
    lp.vec = line_vec(rowlen);
    lp.nchunks = (int)(rowlen / lp.vec);
    lp.n_in = n_in;
    lp.n_out = n_out;
    lp.Nimg = Nimg;
    lp.pad_in = pad_in;
    lp.crop_out = crop_out;
    lp.in_axis_stride = in_axis;
    lp.out_axis_stride = out_axis;
    lp.in_outer_stride = in_outer;
    lp.out_outer_stride = out_outer;
    *nblk = (int64_t)n_outer * lp.nchunks;
    return lp;
}

static int launch_line(const float2 *in, float2 *out, int n_outer, int64_t rowlen,
                       int n_in, int n_out, int Nimg, int pad_in, int crop_out,
                       int64_t in_axis, int64_t out_axis, int64_t in_outer, int64_t out_outer,
                       const FFTDesc &fd, int inv, cudaStream_t s)
{
    int64_t nblk = 0;
    const LinePass lp = make_linepass(n_outer, rowlen, n_in, n_out, Nimg, pad_in, crop_out, in_axis, out_axis,
                                      in_outer, out_outer, &nblk);
    if (nblk <= 0) return NUFFT3D_SUCCESS;
    if (nblk > 0x7fffffff) return fail(NUFFT3D_ERR_SIZE, "FFT pass grid too large");
    const int r1 = four_step_r1(fd.n, lp.vec);
    if (r1) return launch_line4(r1, in, out, lp, fd, inv, nblk, s);
    if (needs_rare(fd))
        k_line<true><<<(unsigned)nblk, kFftThreads, line_smem(lp.vec, fd.n), s>>>(in, out, lp, fd, inv);
    else
        k_line<false><<<(unsigned)nblk, kFftThreads, line_smem(lp.vec, fd.n), s>>>(in, out, lp, fd, inv);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

__device__ __forceinline__ int batch_volume(const BatchFFTParams &P, int blk)
{
    int lo = 0, hi = P.nvol - 1;  // largest v with first[v] <= blk
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.first[mid] <= blk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <bool RARE>
__global__ void __launch_bounds__(kFftThreads)
k_fft_batch_p(const __grid_constant__ BatchFFTParams P, int kind)
{
    extern __shared__ float2 sm[];
    const int v = batch_volume(P, blockIdx.x);
    const int k = blockIdx.x - P.first[v];
    const BatchFFT &b = P.v[v];
    if (kind == 1) {
        line_body<RARE>(b.in, b.out, b.lp, b.fd, b.inv, k, sm);
    } else {
        const int line = k / P.nch[v], c = k - line * P.nch[v];
        if (kind == 0)
            fx_body<RARE>(b.in, b.U, b.out, b.N1, b.N23, b.nc, b.fd, line, c, sm);
        else
            ix_body<RARE>(b.in, b.U, b.out, b.N1, b.N23, b.nc, b.fd, b.scale, b.addend, b.add_coef, line, c, sm);
    }
}

template <int R1>
__global__ void __launch_bounds__(384)
k_line4_batch_p(const __grid_constant__ BatchFFTParams P)
{
    extern __shared__ float2 sm[];
    const int v = batch_volume(P, blockIdx.x);
    const BatchFFT &b = P.v[v];
    line4_body<R1>(b.in, b.out, b.lp, b.fd.tw, b.inv, blockIdx.x - P.first[v], sm);
}

int launch_fft_batch_p(const BatchFFTParams &P, int kind, size_t smem, bool rare, int r1, cudaStream_t s)
{
    const int nblocks = P.first[P.nvol];
    if (nblocks <= 0) return NUFFT3D_SUCCESS;
    if (kind == 1 && r1) {
        const int threads = 16 * (r1 > 16 ? r1 : 16);
        const size_t sm4 = line4_smem(16 * r1);
        switch (r1) {
        case 8: k_line4_batch_p<8><<<nblocks, threads, sm4, s>>>(P); break;
        case 12: k_line4_batch_p<12><<<nblocks, threads, sm4, s>>>(P); break;
        case 16: k_line4_batch_p<16><<<nblocks, threads, sm4, s>>>(P); break;
        case 20: k_line4_batch_p<20><<<nblocks, threads, sm4, s>>>(P); break;
        default: k_line4_batch_p<24><<<nblocks, threads, sm4, s>>>(P); break;
        }
    } else if (rare) {
        k_fft_batch_p<true><<<nblocks, kFftThreads, smem, s>>>(P, kind);
    } else {
        k_fft_batch_p<false><<<nblocks, kFftThreads, smem, s>>>(P, kind);
    }
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

// Four-step radix R1 (K = 16 R1) of a strided-pass group whose volumes all
// have 16-wide line chunks, else 0.
int batch_four_step(int K, bool all_vec16) { return all_vec16 ? four_step_r1(K, 16) : 0; }

int launch_fx(nufft3d_plan *p, const float2 *img, float2 *B1, int nc, cudaStream_t s)
{
    const int N1 = p->N[0], N23 = p->N[1] * p->N[2];
    const FFTDesc &fd = p->fft[0];
    if (const int r1 = four_step_r1(fd.n, 16))
        return launch_xline4<false>(r1, img, B1, p->U, fd, N1, N23, nc, 1.f, nullptr, 0.f, s);
    const int nv = nc < kMaxLineCoils ? nc : kMaxLineCoils;
    dim3 grid(N23, (nc + kMaxLineCoils - 1) / kMaxLineCoils);
    if (needs_rare(fd))
        k_fx<true><<<grid, kFftThreads, line_smem(nv, fd.n), s>>>(img, p->U, B1, N1, N23, nc, fd);
    else
        k_fx<false><<<grid, kFftThreads, line_smem(nv, fd.n), s>>>(img, p->U, B1, N1, N23, nc, fd);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

int launch_ix(nufft3d_plan *p, const float2 *B1, float2 *img, int nc, float scale,
              const float2 *addend, float add_coef, cudaStream_t s)
{
    const int N1 = p->N[0], N23 = p->N[1] * p->N[2];
    const FFTDesc &fd = p->fft[0];
    if (const int r1 = four_step_r1(fd.n, 16))
        return launch_xline4<true>(r1, B1, img, p->U, fd, N1, N23, nc, scale, addend, add_coef, s);
    const int nv = nc < kMaxLineCoils ? nc : kMaxLineCoils;
    dim3 grid(N23, (nc + kMaxLineCoils - 1) / kMaxLineCoils);
    if (needs_rare(fd))
        k_ix<true><<<grid, kFftThreads, line_smem(nv, fd.n), s>>>(B1, p->U, img, N1, N23, nc, fd, scale,
                                                                addend, add_coef);
    else
        k_ix<false><<<grid, kFftThreads, line_smem(nv, fd.n), s>>>(B1, p->U, img, N1, N23, nc, fd, scale,
                                                                 addend, add_coef);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

int launch_fy(nufft3d_plan *p, const float2 *B1, float2 *B2, int nc, cudaStream_t s)
{
    const int64_t K1 = p->geom.K[0], K2 = p->geom.K[1];
    const int64_t N2 = p->N[1], N3 = p->N[2];
    const int64_t row = K1 * nc;
    return launch_line(B1, B2, (int)N3, row, (int)N2, (int)K2, (int)N2, 1, 0, row, row,
                       N2 * row, K2 * row, p->fft[1], 0, s);
}

int launch_fz(nufft3d_plan *p, const float2 *B2, float2 *G, int nc, cudaStream_t s)
{
    const int64_t K1 = p->geom.K[0], K2 = p->geom.K[1], K3 = p->geom.K[2];
    const int64_t N3 = p->N[2];
    const int64_t row = K1 * nc;
    return launch_line(B2, G, (int)K2, row, (int)N3, (int)K3, (int)N3, 1, 0, K2 * row, K2 * row,
                       row, row, p->fft[2], 0, s);
}

int launch_iz(nufft3d_plan *p, const float2 *G, float2 *B2, int nc, cudaStream_t s)
{
    const int64_t K1 = p->geom.K[0], K2 = p->geom.K[1], K3 = p->geom.K[2];
    const int64_t N3 = p->N[2];
    const int64_t row = K1 * nc;
    return launch_line(G, B2, (int)K2, row, (int)K3, (int)N3, (int)N3, 0, 1, K2 * row, K2 * row,
                       row, row, p->fft[2], 1, s);
}

int launch_iy(nufft3d_plan *p, const float2 *B2, float2 *B1, int nc, cudaStream_t s)
{
    const int64_t K1 = p->geom.K[0], K2 = p->geom.K[1];
    const int64_t N2 = p->N[1], N3 = p->N[2];
    const int64_t row = K1 * nc;
    return launch_line(B2, B1, (int)N3, row, (int)K2, (int)N2, (int)N2, 0, 1, row, row,
                       K2 * row, N2 * row, p->fft[1], 1, s);
}

// Allow each FFT kernel all the shared memory a block can have, less its
// static part.
template <typename Kern>
static int allow_fft_smem(Kern kernel)
{
    cudaFuncAttributes fa;
    NUFFT_CUDA_TRY(cudaFuncGetAttributes(&fa, kernel));
    NUFFT_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        227 * 1024 - (int)fa.sharedSizeBytes));
    return NUFFT3D_SUCCESS;
}

int configure_fft_kernels()
{
    NUFFT_TRY(allow_fft_smem(k_fx<false>));
    NUFFT_TRY(allow_fft_smem(k_ix<false>));
    NUFFT_TRY(allow_fft_smem(k_line<false>));
    NUFFT_TRY(allow_fft_smem(k_fx<true>));
    NUFFT_TRY(allow_fft_smem(k_ix<true>));
    NUFFT_TRY(allow_fft_smem(k_line<true>));
    NUFFT_TRY(allow_fft_smem(k_xline4<8, false>));
    NUFFT_TRY(allow_fft_smem(k_xline4<12, false>));
    NUFFT_TRY(allow_fft_smem(k_xline4<16, false>));
    NUFFT_TRY(allow_fft_smem(k_xline4<20, false>));
    NUFFT_TRY(allow_fft_smem(k_xline4<24, false>));
    NUFFT_TRY(allow_fft_smem(k_xline4<8, true>));
    NUFFT_TRY(allow_fft_smem(k_xline4<12, true>));
    NUFFT_TRY(allow_fft_smem(k_xline4<16, true>));
    NUFFT_TRY(allow_fft_smem(k_xline4<20, true>));
    NUFFT_TRY(allow_fft_smem(k_xline4<24, true>));
    NUFFT_TRY(allow_fft_smem(k_line4<8>));
    NUFFT_TRY(allow_fft_smem(k_line4<12>));
    NUFFT_TRY(allow_fft_smem(k_line4<16>));
    NUFFT_TRY(allow_fft_smem(k_line4<20>));
    NUFFT_TRY(allow_fft_smem(k_line4<24>));
    NUFFT_TRY(allow_fft_smem(k_fft_batch_p<false>));
    NUFFT_TRY(allow_fft_smem(k_fft_batch_p<true>));
    NUFFT_TRY(allow_fft_smem(k_line4_batch_p<8>));
    NUFFT_TRY(allow_fft_smem(k_line4_batch_p<12>));
    NUFFT_TRY(allow_fft_smem(k_line4_batch_p<16>));
    NUFFT_TRY(allow_fft_smem(k_line4_batch_p<20>));
    NUFFT_TRY(allow_fft_smem(k_line4_batch_p<24>));
    return configure_fft_constants();
}

} // namespace nufft3d
