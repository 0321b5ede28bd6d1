// Plan construction: the @nufft_3d constructor (nufft_3d.m:54-251).
//
// Instead of assembling the sparse matrix H (nufft_3d.m:129-212, ~113
// nonzeros per sample for J=6 radial), the plan keeps
//   * the in-bounds samples sorted by oversampled-grid tile (a permutation),
//     each as (frac offset, packed tile-local position);
//   * the tile pieces ("blocks") of at most max_samples_per_block samples;
//   * the deapodization U (deap.m) in FP32, built in FP64 on the host;
//   * the density d (density.m) or the user's d;
//   * FFT twiddle tables built in FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "bank_order.h"
#include "internal.h"

namespace nufft3d {

std::recursive_mutex &device_lock()
{
    static std::recursive_mutex mu;
    return mu;
}

// ------------------------------------------------------------- errors
static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

// -------------------------------------------------- FP64 kernel (host)
// kernel.m:14-34, real or complex argument (complex only for deap.m's
// untruncated samples beyond J/2).
static const double kSmall[7] = {1.0, 3.5156229, 3.0899424, 1.2067492, 0.2659732, 0.360768e-1,
                                 0.45813e-2};
static const double kLarge[9] = {0.39894228, 0.1328592e-1, 0.225319e-2, -0.157565e-2, 0.916281e-2,
                                 -0.2057706e-1, 0.2635537e-1, -0.1647633e-1, 0.392377e-2};

template <typename T>
static T horner(T y, const double *c, int n)
{
    T acc = T(c[n - 1]);
    for (int i = n - 2; i >= 0; --i) acc = T(c[i]) + y * acc;
    return acc;
}

static std::complex<double> bessi0c(std::complex<double> ax)
{
    if (std::abs(ax) < 3.75) {
        std::complex<double> y = ax / 3.75;
        y = y * y;
        return horner(y, kSmall, 7);
    }
    std::complex<double> y = 3.75 / ax;
    std::complex<double> r = (std::exp(ax) / std::sqrt(ax)) * horner(y, kLarge, 9);
    if (ax.real() == 0) r = 2.0 * r; // kernel.m:32-34
    return r;
}

double bessi0_host(double ax) { return bessi0c(std::complex<double>(ax, 0.0)).real(); }

static double kernel_host(double dist2, double alpha, double J)
{
    const double half = J / 2;
    const double t = 1 - dist2 / (half * half);
    const double den = bessi0_host(alpha);
    if (t >= 0) return bessi0_host(alpha * std::sqrt(t)) / den;
    std::complex<double> arg(0.0, alpha * std::sqrt(-t));
    return (bessi0c(arg) / den).real();
}

// Polynomial in t = 1 - dist2/(J/2)^2 for the kernel on its support
// (kernel.m:2-11 with t in [0, 1]): interpolation at the kKBDeg+1 Chebyshev
// nodes of [0, 1], converted to monomial coefficients in t, all in FP64.  The
// FP32 Horner evaluation (as on the device) is then emulated on a fine grid
// against the FP64
// kernel; the fit is used only if its largest error stays below 4e-6 (true
// for the usual alpha; very large alpha keeps the direct evaluation).
static void fit_kb_poly(double alpha, double i0a, KBParams &kb)
{
    constexpr int n = kKBDeg + 1;
    double f[n], c[n];
    for (int j = 0; j < n; ++j) {
        const double x = std::cos(M_PI * (j + 0.5) / n), t = 0.5 * (x + 1);
        f[j] = bessi0_host(alpha * std::sqrt(t)) / i0a;
    }
    for (int k = 0; k < n; ++k) {
        double a = 0;
        for (int j = 0; j < n; ++j) a += f[j] * std::cos(M_PI * k * (j + 0.5) / n);
        c[k] = a * 2.0 / n;
    }
    c[0] *= 0.5;
    // sum_k c_k T_k(2t - 1) in powers of t: T_{k+1} = 2 (2t - 1) T_k - T_{k-1}
    std::vector<double> m(n, 0.0), tkm1(n, 0.0), tk(n, 0.0), tkp1(n, 0.0);
    tkm1[0] = 1;
    tk[0] = -1;
    tk[1] = 2;
    m[0] = c[0];
    for (int i = 0; i < n; ++i) m[i] += c[1] * tk[i];
    for (int k = 1; k + 1 < n; ++k) {
        for (int i = 0; i < n; ++i) tkp1[i] = -2 * tk[i] - tkm1[i] + (i > 0 ? 4 * tk[i - 1] : 0.0);
        for (int i = 0; i < n; ++i) m[i] += c[k + 1] * tkp1[i];
        tkm1.swap(tk);
        tk.swap(tkp1);
    }
    for (int i = 0; i < n; ++i) kb.c[i] = (float)m[i];
    double err = 0;
    for (int i = 0; i <= 8192; ++i) {
        const float t = (float)(i / 8192.0);
        float s = kb.c[kKBDeg];  // the device's Horner steps (kb_weight)
        for (int k = kKBDeg - 1; k >= 0; --k) s = fmaf(s, t, kb.c[k]);
        err = std::max(err, std::fabs((double)s - bessi0_host(alpha * std::sqrt((double)t)) / i0a));
    }
    kb.poly = err < 4e-6 ? 1 : 0;
}

// deap.m:2-36,97-98.  ifft(X*K, 2K, 'symmetric') of the (J+1)-sample kernel
// table is 0.5*T0 + sum_{d>=1} T_d cos(pi d m / K); rows m in [-N/2, N/2) are
// kept and fftshifted, so output index p holds m = p - N/2.  Returns 1/U.
static std::vector<double> deap_host(const int N[3], const int K[3], double J, double alpha,
                                     int radial, int is2d)
{
    const int nJ = (int)std::floor(J) + 1;
    const int nz = is2d ? 1 : nJ;
    std::vector<double> T((size_t)nJ * nJ * nz);
    for (int dz = 0; dz < nz; ++dz)
        for (int dy = 0; dy < nJ; ++dy)
            for (int dx = 0; dx < nJ; ++dx) {
                const double dx2 = (dx / 2.0) * (dx / 2.0), dy2 = (dy / 2.0) * (dy / 2.0),
                             dz2 = (dz / 2.0) * (dz / 2.0);
                double v;
                if (radial)
                    v = kernel_host(dx2 + dy2 + dz2, alpha, J);
                else
                    v = kernel_host(dx2, alpha, J) * kernel_host(dy2, alpha, J) *
                        kernel_host(dz2, alpha, J);
                T[((size_t)dz * nJ + dy) * nJ + dx] = v;
            }
    // per-axis coefficient tables c_a(d, p) = 0.5 (d = 0) or cos(pi d (p - N/2) / K)
    std::vector<double> ctab[3];
    for (int a = 0; a < 3; ++a) {
        ctab[a].resize((size_t)nJ * std::max(N[a], 1));
        for (int d = 0; d < nJ; ++d)
            for (int p = 0; p < N[a]; ++p)
                ctab[a][(size_t)d * N[a] + p] = d == 0 ? 0.5 : std::cos(M_PI * d * (double)(p - N[a] / 2) / K[a]);
    }
    auto coef = [&](int axis, int d, int p) { return ctab[axis][(size_t)d * N[axis] + p]; };
    const int N1 = N[0], N2 = N[1], N3 = N[2];
    // x
    std::vector<double> A((size_t)N1 * nJ * nz, 0.0);
    for (int dz = 0; dz < nz; ++dz)
        for (int dy = 0; dy < nJ; ++dy)
            for (int px = 0; px < N1; ++px) {
                double s = 0;
                for (int dx = 0; dx < nJ; ++dx) s += T[((size_t)dz * nJ + dy) * nJ + dx] * coef(0, dx, px);
                A[((size_t)dz * nJ + dy) * N1 + px] = s;
            }
    // y
    std::vector<double> B((size_t)N1 * N2 * nz, 0.0);
    for (int dz = 0; dz < nz; ++dz)
        for (int py = 0; py < N2; ++py)
            for (int px = 0; px < N1; ++px) {
                double s = 0;
                for (int dy = 0; dy < nJ; ++dy) s += A[((size_t)dz * nJ + dy) * N1 + px] * coef(1, dy, py);
                B[((size_t)dz * N2 + py) * N1 + px] = s;
            }
    std::vector<double> U((size_t)N1 * N2 * N3, 0.0);
    if (is2d) {
        for (size_t i = 0; i < U.size(); ++i) U[i] = 1.0 / B[i];
        return U;
    }
    for (int pz = 0; pz < N3; ++pz)
        for (int py = 0; py < N2; ++py)
            for (int px = 0; px < N1; ++px) {
                double s = 0;
                for (int dz = 0; dz < nz; ++dz) s += B[((size_t)dz * N2 + py) * N1 + px] * coef(2, dz, pz);
                U[((size_t)pz * N2 + py) * N1 + px] = 1.0 / s;
            }
    return U;
}

// Candidate taps for the box lo <= f <= hi (per axis) inside the reflected
// octant [0, 1/2]^3: offsets d' in [-R, R]^3 whose smallest possible distance
// over the box is inside the support, ordered near to far (offsets inside the
// support for every f of the box first; bank_order then re-partitions nearby
// chunks of 8 for shared-memory banks).  A relative slack of 1e-5 keeps every
// tap that the single-precision test in the kernels can accept.
static std::vector<int> make_candidates(int R, int radial, int is2d, double J, const double lo[3],
                                        const double hi[3], int *ncore)
{
    const double h2 = (J / 2) * (J / 2) * (1 + 1e-5);
    auto mn = [&](int d, int a) {
        if (d >= lo[a] && d <= hi[a]) return 0.0;
        const double u = d - lo[a], v = d - hi[a];
        return std::min(u * u, v * v);
    };
    auto mx = [&](int d, int a) {
        const double u = d - lo[a], v = d - hi[a];
        return std::max(u * u, v * v);
    };
    struct C {
        double key, key2;
        int code;
    };
    std::vector<C> v;
    const int rz = is2d ? 0 : R;
    for (int dz = -rz; dz <= rz; ++dz)
        for (int dy = -R; dy <= R; ++dy)
            for (int dx = -R; dx <= R; ++dx) {
                const double n0 = mn(dx, 0), n1 = mn(dy, 1), n2 = mn(dz, 2);
                const double x0 = mx(dx, 0), x1 = mx(dy, 1), x2 = mx(dz, 2);
                const bool keep = radial ? n0 + n1 + n2 <= h2 : (n0 <= h2 && n1 <= h2 && n2 <= h2);
                const double key = radial ? x0 + x1 + x2 : std::max(x0, std::max(x1, x2));
                if (keep) v.push_back({key, n0 + n1 + n2, (dx + 8) | ((dy + 8) << 4) | ((dz + 8) << 8)});
            }
    std::stable_sort(v.begin(), v.end(), [](const C &a, const C &b) {
        return a.key != b.key ? a.key < b.key : a.key2 < b.key2;
    });
    // core: inside the support for every f of the box with a margin far above
    // the single-precision error of the kernels' distance test
    const double h2core = (J / 2) * (J / 2) * (1 - 1e-4);
    *ncore = 0;
    while (*ncore < (int)v.size() && v[*ncore].key <= h2core) ++*ncore;
    std::vector<int> out;
    for (auto &c : v) out.push_back(c.code);
    return out;
}

// The 8 sub-cube lists of the reflected octant (sub-cube q: |f_a| >= 1/4
// iff bit a of q), each ordered by bank_order, back to back.  Cached per
// geometry: the ordering search takes a fraction of a second.
struct CandSet {
    std::vector<int> codes;
    int start[8], cnt[8], core[8];
};

static const CandSet &candidate_set(int R, int radial, int is2d, double J, int Px, int PxPy)
{
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, double, int, int>, CandSet> cache;
    const auto key = std::make_tuple(R, radial, is2d, J, Px, PxPy);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    CandSet cs;
    for (int q = 0; q < 8; ++q) {
        double lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            const bool up = (q >> a) & 1;
            lo[a] = up ? 0.25 : 0.0;
            hi[a] = up ? 0.5 : 0.25;
        }
        if (is2d) lo[2] = hi[2] = 0.0;  // f_z = 0 in 2-D
        int ncore = 0;
        std::vector<int> c = make_candidates(R, radial, is2d, J, lo, hi, &ncore);
        bank_order(c, Px, PxPy, J, radial, is2d, lo, hi, ncore);
        cs.start[q] = (int)cs.codes.size();
        cs.cnt[q] = (int)c.size();
        cs.core[q] = ncore;
        cs.codes.insert(cs.codes.end(), c.begin(), c.end());
    }
    return cache.emplace(key, std::move(cs)).first->second;
}

// ------------------------------------------------------ device kernels
struct KeyParams {
    double u;
    int K[3], T[3], nt[3], Ra[3];
    int is2d;
    uint32_t ntiles;
};

__device__ __forceinline__ int64_t wrap64(int64_t x, int64_t K)
{
    int64_t r = x % K;
    return r < 0 ? r + K : r;
}

// nufft_3d.m:120-125: om scaled by u in double; ok mask; tile key.
__global__ void k_keys(const double *__restrict__ om, int64_t M, KeyParams kp,
                       uint32_t *__restrict__ keys, int32_t *__restrict__ vals)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    double og[3];
    bool ok = true;
    for (int a = 0; a < 3; ++a) {
        og[a] = kp.u * om[3 * m + a];
        ok = ok && og[a] >= -kp.K[a] / 2.0 && og[a] <= kp.K[a] / 2.0 - 1;
    }
    if (kp.is2d) ok = true; // nufft_3d.m:125 ('... & ok | N(3)==1')
    uint32_t key = kp.ntiles;
    if (ok) {
        int t[3];
        for (int a = 0; a < 3; ++a) {
            const int64_t b = wrap64((int64_t)round(og[a]), kp.K[a]);
            t[a] = (int)(b / kp.T[a]);
        }
        key = (uint32_t)(t[0] + kp.nt[0] * (t[1] + kp.nt[1] * t[2]));
    }
    keys[m] = key;
    vals[m] = (int32_t)m;
}

__global__ void k_hist(const uint32_t *__restrict__ keys, int64_t M, uint32_t ntiles,
                       int32_t *__restrict__ counts)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const uint32_t k = keys[m];
    if (k < ntiles) atomicAdd(&counts[k], 1);
}

__global__ void k_records(const double *__restrict__ om, const int32_t *__restrict__ perm,
                          int64_t nnz, KeyParams kp, float4 *__restrict__ samples,
                          int32_t *__restrict__ inv)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nnz) return;
    const int m = perm[s];
    float f[3];
    int l[3];
    for (int a = 0; a < 3; ++a) {
        const double og = kp.u * om[3 * (int64_t)m + a];
        const double r = round(og);
        f[a] = (float)(og - r);
        const int64_t b = wrap64((int64_t)r, kp.K[a]);
        const int64_t t = b / kp.T[a];
        l[a] = (int)(b - t * kp.T[a]) + kp.Ra[a];
    }
    const int packed = l[0] | (l[1] << 8) | (l[2] << 16);
    samples[s] = make_float4(f[0], f[1], f[2], __int_as_float(packed));
    inv[m] = (int32_t)s;
}

__global__ void k_sorted_from_orig(const float *__restrict__ dorig, const int32_t *__restrict__ perm,
                                   int64_t nnz, float *__restrict__ dsorted)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nnz) dsorted[s] = dorig[perm[s]];
}

__global__ void k_orig_from_sorted(const float *__restrict__ dsorted, const int32_t *__restrict__ inv,
                                   int64_t M, float *__restrict__ dorig)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const int s = inv[m];
    dorig[m] = s >= 0 ? dsorted[s] : 0.f;
}

// Count taps (nonzeros of H) per block, for the plan summary.
template <int R>
__global__ void k_count_taps(const float4 *__restrict__ samples, int64_t nnz, float half2, int radial,
                             int rz, unsigned long long *__restrict__ total)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long c = 0;
    if (s < nnz) {
        const float4 r = samples[s];
        for (int dz = -rz; dz <= rz; ++dz)
            for (int dy = -R; dy <= R; ++dy)
                for (int dx = -R; dx <= R; ++dx) {
                    const float ex = dx - r.x, ey = dy - r.y, ez = dz - r.z;
                    if (radial) c += (ez * ez + ey * ey) + ex * ex <= half2;
                    else c += (ex * ex <= half2) && (ey * ey <= half2) && (ez * ez <= half2);
                }
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

// ---------------------------------------------------------------- host
int configure_fft_kernels();
int configure_interp_kernels();

int configure_kernels()
{
    static std::mutex mu;
    static int done_mask = 0; // per device bit (first 32 devices)
    int dev = 0;
    NUFFT_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 32 && (done_mask & (1 << dev))) return NUFFT3D_SUCCESS;
    NUFFT_DEVICE_LOCK; // constant-memory uploads must not overlap a stream capture
    NUFFT_TRY(configure_fft_kernels());
    NUFFT_TRY(configure_interp_kernels());
    NUFFT_TRY(configure_spread_tab_kernels());
    if (dev < 32) done_mask |= 1 << dev;
    return NUFFT3D_SUCCESS;
}

TableOwner::~TableOwner()
{
    NUFFT_DEVICE_LOCK;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != device) cudaSetDevice(device);
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
}

// Hand the plan's table pointers to a shared owner (after a successful build).
static void adopt_tables(nufft3d_plan *p)
{
    auto t = std::make_shared<TableOwner>();
    t->device = p->device;
    t->ptrs = {p->samples, p->perm, p->inv, p->blocks, p->cand, p->U, p->d, p->d_orig,
               p->tw[0], p->tw[1], p->tw[2], p->tap_rows, p->tap_ent, p->spread_pieces, p->spread_wstart, p->spread_ent};
    p->tables = t;
}

// Free what the plan owns by itself; tables go with the last sharer.
static void free_plan_memory(nufft3d_plan *p)
{
    NUFFT_DEVICE_LOCK;
    auto F = [](void *ptr) {
        if (ptr) cudaFree(ptr);
    };
    if (!p->tables) { // never adopted: free tables directly
        F(p->samples);
        F(p->perm);
        F(p->inv);
        F(p->blocks);
        F(p->cand);
        F(p->U);
        F(p->d);
        F(p->d_orig);
        for (int a = 0; a < 3; ++a) F(p->tw[a]);
        F(p->tap_rows);
        F(p->tap_ent);
        F(p->spread_pieces);
        F(p->spread_wstart);
        F(p->spread_ent);
    }
    F(p->wbuf);
    F(p->work);
    F(p->own_blocks);
    F(p->scratch.B1);
    F(p->scratch.B2);
    if (p->scratch.G != p->scratch.B2) F(p->scratch.G); // 2D: G aliases B2
    F(p->scratch.ks);
    F(p->stage.in);
    F(p->stage.out);
    SolverWork &w = p->solver;
    F(w.x); F(w.r); F(w.p); F(w.q); F(w.v); F(w.vprev); F(w.w1); F(w.w2);
    F(w.partial); F(w.bpart); F(w.scal); F(w.iters);
    profile_release(p);
    if (p->own_stream) cudaStreamDestroy(p->own_stream);
    p->tables.reset();
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

template <typename T>
static int dmalloc(T **ptr, size_t count, int64_t *acc)
{
    NUFFT_DEVICE_LOCK;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)ptr, count * sizeof(T));
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return fail(NUFFT3D_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    if (acc) *acc += (int64_t)(count * sizeof(T));
    return NUFFT3D_SUCCESS;
}

// The stored H (nufft_3d.m:153-212) in tile order: count each row's chunks,
// scan them into row offsets, then fill the rows.  mode 0 = none, 1 = always,
// -1 = when it takes at most half of the free device memory.
static int build_tap_table(nufft3d_plan *p, int mode, std::vector<void *> &tmp, cudaStream_t s)
{
    if (mode == 0 || p->nnz == 0 || !tap_table_applies(p)) return NUFFT3D_SUCCESS;
    const int64_t nnz = p->nnz;
    int maxcnt = 0;
    for (int q = 0; q < 8; ++q) maxcnt = std::max(maxcnt, p->cand_desc.cnt[q]);
    if ((uint64_t)nnz * (uint64_t)((maxcnt + 7) / 8) >= 0xffffffffull) {  // row offsets are 32-bit chunk indices
        if (mode < 0) return NUFFT3D_SUCCESS;
        return fail(NUFFT3D_ERR_SIZE, "too many samples for the stored H");
    }
    uint32_t *cnt = nullptr;
    NUFFT_TRY(dmalloc(&cnt, (size_t)nnz + 1, nullptr));
    tmp.push_back(cnt);
    NUFFT_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (nnz + 1), s));
    NUFFT_TRY(launch_tap_count(p, cnt, s));
    size_t tb = 0;
    NUFFT_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt, cnt, (int)(nnz + 1), s));
    void *tstore = nullptr;
    NUFFT_TRY(dmalloc((char **)&tstore, tb ? tb : 1, nullptr));
    tmp.push_back(tstore);
    uint32_t *rows = nullptr;
    NUFFT_TRY(dmalloc(&rows, (size_t)nnz + 1, nullptr));
    uint32_t total = 0;
    cudaError_t e = cub::DeviceScan::ExclusiveSum(tstore, tb, cnt, rows, (int)(nnz + 1), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, rows + nnz, sizeof(total), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(rows);
        return fail(NUFFT3D_ERR_CUDA, std::string("stored H row scan: ") + cudaGetErrorString(e));
    }
    const uint64_t entries = (uint64_t)total * 8;
    const uint64_t bytes = entries * sizeof(int2);
    if (mode < 0) {
        size_t fr = 0, to = 0;
        if (cudaMemGetInfo(&fr, &to) != cudaSuccess || bytes > fr / 2) {
            cudaGetLastError();
            cudaFree(rows);
            return NUFFT3D_SUCCESS;  // evaluate on the fly instead
        }
    }
    int2 *taps = nullptr;
    const int st = dmalloc(&taps, (size_t)entries, nullptr);
    if (st != NUFFT3D_SUCCESS) {
        cudaFree(rows);
        if (mode < 0) {
            clear_error();
            return NUFFT3D_SUCCESS;
        }
        return st;
    }
    p->tap_rows = rows;
    p->tap_ent = taps;
    p->tap_bytes = (int64_t)(bytes + sizeof(uint32_t) * (nnz + 1));
    p->table_bytes += p->tap_bytes;
    NUFFT_TRY(launch_tap_fill(p, rows, taps, s));
    NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    return NUFFT3D_SUCCESS;
}

std::vector<int4> make_pieces(const std::vector<int32_t> &counts, int S)
{
    std::vector<int4> blocks;
    int64_t off = 0;
    for (size_t t = 0; t < counts.size(); ++t) {
        const int64_t c = counts[t];
        if (c > 0) {
            const int64_t nb = (c + S - 1) / S;
            for (int64_t b = 0; b < nb; ++b) {
                const int64_t b0 = c * b / nb, b1 = c * (b + 1) / nb;
                blocks.push_back(make_int4((int)t, (int)(off + b0), (int)(b1 - b0), 0));
            }
        }
        off += c;
    }
    // largest pieces first: the heavy centre of radial k-space starts early
    std::stable_sort(blocks.begin(), blocks.end(), [](const int4 &a, const int4 &b) { return a.z > b.z; });
    return blocks;
}

static int build_plan(nufft3d_plan *p, const double *om_host, const nufft3d_opts &o)
{
    const int64_t M = p->M;
    const Geom &g = p->geom;
    cudaStream_t s = p->own_stream;
    double *om_dev = nullptr;
    NUFFT_TRY(dmalloc(&om_dev, (size_t)3 * M, nullptr));
    struct Tmp {
        std::vector<void *> ptrs;
        ~Tmp()
        {
            NUFFT_DEVICE_LOCK;
            for (void *q : ptrs) cudaFree(q);
        }
    } tmp;
    tmp.ptrs.push_back(om_dev);
    NUFFT_CUDA_TRY(cudaMemcpyAsync(om_dev, om_host, sizeof(double) * 3 * M, cudaMemcpyHostToDevice, s));

    KeyParams kp;
    kp.u = p->u;
    kp.is2d = g.is2d;
    for (int a = 0; a < 3; ++a) {
        kp.K[a] = g.K[a];
        kp.T[a] = g.T[a];
        kp.nt[a] = g.nt[a];
        kp.Ra[a] = g.Ra[a];
    }
    const uint64_t ntiles64 = (uint64_t)g.nt[0] * g.nt[1] * g.nt[2];
    if (ntiles64 >= 0x7fffffffull) return fail(NUFFT3D_ERR_SIZE, "too many interpolation tiles");
    kp.ntiles = (uint32_t)ntiles64;
    const uint32_t ntiles = kp.ntiles;

    uint32_t *keys = nullptr, *keys_sorted = nullptr;
    int32_t *vals = nullptr;
    NUFFT_TRY(dmalloc(&keys, (size_t)M, nullptr));
    tmp.ptrs.push_back(keys);
    NUFFT_TRY(dmalloc(&keys_sorted, (size_t)M, nullptr));
    tmp.ptrs.push_back(keys_sorted);
    NUFFT_TRY(dmalloc(&vals, (size_t)M, nullptr));
    tmp.ptrs.push_back(vals);
    NUFFT_TRY(dmalloc(&p->perm, (size_t)M, &p->table_bytes));
    const int th = 256;
    const unsigned nbM = (unsigned)((M + th - 1) / th);
    if (M > 0) {
        k_keys<<<nbM, th, 0, s>>>(om_dev, M, kp, keys, vals);
        NUFFT_CUDA_TRY(cudaGetLastError());
    }
    int end_bit = 1;
    while ((1ull << end_bit) <= (uint64_t)ntiles) ++end_bit;
    size_t tb = 0;
    NUFFT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys_sorted, vals, p->perm,
                                                   (int)M, 0, end_bit, s));
    void *tstore = nullptr;
    NUFFT_TRY(dmalloc((char **)&tstore, tb ? tb : 1, nullptr));
    tmp.ptrs.push_back(tstore);
    NUFFT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(tstore, tb, keys, keys_sorted, vals, p->perm,
                                                   (int)M, 0, end_bit, s));
    int32_t *counts = nullptr;
    NUFFT_TRY(dmalloc(&counts, (size_t)ntiles, nullptr));
    tmp.ptrs.push_back(counts);
    NUFFT_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int32_t) * ntiles, s));
    if (M > 0) {
        k_hist<<<nbM, th, 0, s>>>(keys, M, ntiles, counts);
        NUFFT_CUDA_TRY(cudaGetLastError());
    }
    std::vector<int32_t> hc(ntiles);
    NUFFT_CUDA_TRY(cudaMemcpyAsync(hc.data(), counts, sizeof(int32_t) * ntiles, cudaMemcpyDeviceToHost, s));
    NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    int64_t nnz = 0;
    for (uint32_t t = 0; t < ntiles; ++t) nnz += hc[t];
    p->nnz = nnz;

    // tile pieces of at most S samples, split evenly
    p->tile_counts = std::move(hc);
    p->piece_samples = o.max_samples_per_block > 0 ? o.max_samples_per_block : kDefaultPieceSamples;
    {
        const std::vector<int4> blocks = make_pieces(p->tile_counts, p->piece_samples);
        p->n_blocks = (int64_t)blocks.size();
        NUFFT_TRY(dmalloc(&p->blocks, blocks.size(), &p->table_bytes));
        if (!blocks.empty())
            NUFFT_CUDA_TRY(cudaMemcpyAsync(p->blocks, blocks.data(), sizeof(int4) * blocks.size(),
                                           cudaMemcpyHostToDevice, s));
    }

    NUFFT_TRY(dmalloc(&p->samples, (size_t)nnz, &p->table_bytes));
    NUFFT_TRY(dmalloc(&p->inv, (size_t)M, &p->table_bytes));
    NUFFT_CUDA_TRY(cudaMemsetAsync(p->inv, 0xFF, sizeof(int32_t) * (M > 0 ? M : 1), s));
    if (nnz > 0) {
        k_records<<<(unsigned)((nnz + th - 1) / th), th, 0, s>>>(om_dev, p->perm, nnz, kp, p->samples, p->inv);
        NUFFT_CUDA_TRY(cudaGetLastError());
        unsigned long long *tot = nullptr;
        NUFFT_TRY(dmalloc(&tot, 1, nullptr));
        tmp.ptrs.push_back(tot);
        NUFFT_CUDA_TRY(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), s));
        const unsigned nbs = (unsigned)((nnz + th - 1) / th);
        const int rz = g.is2d ? 0 : g.R;
        switch (g.R) {
        case 1: k_count_taps<1><<<nbs, th, 0, s>>>(p->samples, nnz, p->kb.half2, g.radial, rz, tot); break;
        case 2: k_count_taps<2><<<nbs, th, 0, s>>>(p->samples, nnz, p->kb.half2, g.radial, rz, tot); break;
        case 3: k_count_taps<3><<<nbs, th, 0, s>>>(p->samples, nnz, p->kb.half2, g.radial, rz, tot); break;
        default: k_count_taps<4><<<nbs, th, 0, s>>>(p->samples, nnz, p->kb.half2, g.radial, rz, tot); break;
        }
        NUFFT_CUDA_TRY(cudaGetLastError());
        unsigned long long ht = 0;
        NUFFT_CUDA_TRY(cudaMemcpyAsync(&ht, tot, sizeof(ht), cudaMemcpyDeviceToHost, s));
        NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
        p->taps = (double)ht / (double)nnz;
    }

    {
        const CandSet &cs = candidate_set(g.R, g.radial, g.is2d, p->J, g.P[0], g.P[0] * g.P[1]);
        p->n_cand = (int)cs.codes.size();
        NUFFT_TRY(dmalloc(&p->cand, cs.codes.size(), &p->table_bytes));
        NUFFT_CUDA_TRY(
            cudaMemcpyAsync(p->cand, cs.codes.data(), sizeof(int) * cs.codes.size(), cudaMemcpyHostToDevice, s));
        p->cand_desc.list = p->cand;
        p->cand_desc.n = p->n_cand;
        for (int q = 0; q < 8; ++q) {
            p->cand_desc.start[q] = cs.start[q];
            p->cand_desc.cnt[q] = cs.cnt[q];
            p->cand_desc.core[q] = cs.core[q];
        }
    }
    NUFFT_TRY(launch_weight_sum(p, s));
    NUFFT_TRY(build_tap_table(p, o.tap_table, tmp.ptrs, s));
    NUFFT_TRY(build_spread_table(p, o.spread_table, s));
    // deapodization (FP64 on the host, stored FP32 like deap.m:100-101)
    {
        std::vector<double> U = deap_host(p->N, g.K, p->J, p->alpha, g.radial, g.is2d);
        std::vector<float> Uf(U.size());
        for (size_t i = 0; i < U.size(); ++i) Uf[i] = (float)U[i];
        NUFFT_TRY(dmalloc(&p->U, Uf.size(), &p->table_bytes));
        NUFFT_CUDA_TRY(cudaMemcpyAsync(p->U, Uf.data(), sizeof(float) * Uf.size(), cudaMemcpyHostToDevice, s));
        NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    }
    // twiddles (FP64 -> FP32)
    for (int a = 0; a < 3; ++a) {
        const int K = g.K[a];
        if (!fft_factor(K, p->fft[a]))
            return fail(NUFFT3D_ERR_UNSUPPORTED,
                        "oversampled size K=" + std::to_string(K) +
                            " has a prime factor above 13 (FFT radices 2,3,5,7,11,13)");
        std::vector<float2> tw(K);
        for (int j = 0; j < K; ++j) {
            const double ang = -2.0 * M_PI * (double)j / (double)K;
            tw[j] = make_float2((float)std::cos(ang), (float)std::sin(ang));
        }
        NUFFT_TRY(dmalloc(&p->tw[a], (size_t)K, &p->table_bytes));
        NUFFT_CUDA_TRY(cudaMemcpyAsync(p->tw[a], tw.data(), sizeof(float2) * K, cudaMemcpyHostToDevice, s));
        p->fft[a].tw = p->tw[a];
        NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    }
    // density: user supplied (nufft_3d.m:229-237) or density.m
    NUFFT_TRY(dmalloc(&p->d, (size_t)nnz, &p->table_bytes));
    NUFFT_TRY(dmalloc(&p->d_orig, (size_t)M, &p->table_bytes));
    if (o.d) {
        NUFFT_CUDA_TRY(cudaMemcpyAsync(p->d_orig, o.d, sizeof(float) * M, cudaMemcpyHostToDevice, s));
        if (nnz > 0) {
            k_sorted_from_orig<<<(unsigned)((nnz + th - 1) / th), th, 0, s>>>(p->d_orig, p->perm, nnz, p->d);
            NUFFT_CUDA_TRY(cudaGetLastError());
        }
        if (M > 0) {
            k_orig_from_sorted<<<nbM, th, 0, s>>>(p->d, p->inv, M, p->d_orig); // d(~ok) = 0
            NUFFT_CUDA_TRY(cudaGetLastError());
        }
        NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    } else {
        const int iters = o.density_iters > 0 ? o.density_iters : (o.density_iters == 0 ? 20 : 0);
        NUFFT_TRY(run_density(p, iters, s));
    }
    return plan_check_status(p, s);
}

int refresh_density_orig(nufft3d_plan *p, cudaStream_t s)
{
    if (p->M == 0) return NUFFT3D_SUCCESS;
    const int th = 256;
    k_orig_from_sorted<<<(unsigned)((p->M + th - 1) / th), th, 0, s>>>(p->d, p->inv, p->M, p->d_orig);
    NUFFT_CUDA_TRY(cudaGetLastError());
    return NUFFT3D_SUCCESS;
}

} // namespace nufft3d

using namespace nufft3d;

extern "C" int nufft3d_opts_default(nufft3d_opts *o)
{
    if (!o) return fail(NUFFT3D_ERR_ARG, "opts is NULL");
    std::memset(o, 0, sizeof(*o));
    o->J = 4;
    o->u = 2;
    o->alpha = 0;
    o->radial = 1;
    o->gpu = 1;
    o->device = -1;
    o->d = nullptr;
    o->density_iters = 20;
    o->tap_table = -1;
    o->wait_polls = kDefaultWaitPolls;
    o->spread_table = -1;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_plan_create(const double *om, int64_t M, const int32_t *Nin, int n_N,
                                   const nufft3d_opts *opts_in, nufft3d_plan **out)
{
    clear_error();
    if (!out) return fail(NUFFT3D_ERR_ARG, "plan output pointer is NULL");
    *out = nullptr;
    nufft3d_opts o;
    if (opts_in) o = *opts_in;
    else nufft3d_opts_default(&o);
    // nufft_3d.m:60-61
    if (!om || M <= 0) return fail(NUFFT3D_ERR_ARG, "om must be a real array with leading dimension of 3");
    if (M > 0x7fffffffll) return fail(NUFFT3D_ERR_SIZE, "more than 2^31-1 samples");
    for (int64_t i = 0; i < 3 * M; ++i)
        if (!std::isfinite(om[i])) return fail(NUFFT3D_ERR_ARG, "om must be finite");
    if (o.gpu == 0) return fail(NUFFT3D_ERR_UNSUPPORTED, "gpu=0 (CPU path) is not provided by this library");
    if (o.gpu != 1) return fail(NUFFT3D_ERR_UNSUPPORTED, "only gpu=1 (single precision GPU) is implemented");
    // nufft_3d.m:82-84
    if (!(o.u >= 1 && o.u <= 6)) return fail(NUFFT3D_ERR_ARG, "value of u=" + std::to_string(o.u) + " is not recommended");
    if (!(o.J > 0)) return fail(NUFFT3D_ERR_ARG, "J must be positive");
    const int R = (int)std::ceil(o.J / 2);
    if (R < 1 || R > 4) return fail(NUFFT3D_ERR_UNSUPPORTED, "J must satisfy ceil(J/2) <= 4 (J <= 8)");
    // nufft_3d.m:85-92
    double alpha = o.alpha;
    if (alpha == 0) {
        const double q = o.J * o.J * (1 - 0.5 / o.u) * (1 - 0.5 / o.u);
        alpha = M_PI * std::sqrt(o.radial ? q - 0.6 * o.u : q - 0.8);
    }
    if (!(alpha > 0) || !std::isfinite(alpha)) return fail(NUFFT3D_ERR_ARG, "invalid Kaiser-Bessel alpha");
    // nufft_3d.m:96-106
    if (!Nin || !(n_N == 1 || n_N == 3)) return fail(NUFFT3D_ERR_ARG, "N must be scalar or 3-vector of even integers");
    int N[3];
    for (int a = 0; a < 3; ++a) N[a] = n_N == 1 ? Nin[0] : Nin[a];
    if ((N[0] == 0 && N[1] == 0 && N[2] == 0) || N[0] % 2 || N[1] % 2 || N[0] <= 0 || N[1] <= 0 || N[2] < 0)
        return fail(NUFFT3D_ERR_ARG, "N must be an even integer");
    bool all_z0 = true;
    for (int64_t m = 0; m < M && all_z0; ++m) all_z0 = om[3 * m + 2] == 0;
    if (all_z0) N[2] = 1;
    const int is2d = N[2] == 1;
    if (!is2d && (N[2] % 2 || N[2] <= 0)) return fail(NUFFT3D_ERR_ARG, "N must be an even integer");
    // nufft_3d.m:109-111
    int K[3];
    for (int a = 0; a < 3; ++a) K[a] = 2 * (int)std::ceil(N[a] * o.u / 2);
    if (is2d) K[2] = 1;
    if ((double)K[0] * K[1] * K[2] >= 2147483647.0) return fail(NUFFT3D_ERR_SIZE, "N or u too large");
    if (o.wait_polls < 0) return fail(NUFFT3D_ERR_ARG, "wait_polls must be nonnegative");

    int dev = o.device;
    if (dev < 0) {
        if (cudaGetDevice(&dev) != cudaSuccess) return fail(NUFFT3D_ERR_CUDA, "no CUDA device");
    }
    DeviceGuard guard(dev);
    NUFFT_TRY(configure_kernels());

    nufft3d_plan *p = new nufft3d_plan();
    p->device = dev;
    cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, dev);
    for (int a = 0; a < 3; ++a) p->N[a] = N[a];
    p->M = M;
    p->J = o.J;
    p->u = o.u;
    p->alpha = alpha;
    p->radial = o.radial ? 1 : 0;
    p->i0a = bessi0_host(alpha);
    Geom &g = p->geom;
    g.R = R;
    g.radial = p->radial;
    g.is2d = is2d;
    for (int a = 0; a < 3; ++a) {
        g.K[a] = K[a];
        g.Ra[a] = (a == 2 && is2d) ? 0 : R;
        const int t = is2d ? (a == 2 ? 1 : 32) : 8; // the kernels' fixed tile shape
        if (o.tile[a] > 0 && o.tile[a] != t) {
            delete p;
            return fail(NUFFT3D_ERR_UNSUPPORTED, "tile shape is fixed at 8x8x8 (3-D) / 32x32x1 (2-D)");
        }
        g.T[a] = t;
        g.P[a] = t + 2 * g.Ra[a];
        g.nt[a] = (K[a] + t - 1) / t;
    }
    KBParams &kb = p->kb;
    const double half = o.J / 2;
    kb.alpha = (float)alpha;
    kb.inv_half2 = (float)(1.0 / (half * half));
    kb.a2_over = (float)(alpha * alpha / (3.75 * 3.75));
    kb.inv_i0a = (float)(1.0 / p->i0a);
    kb.exp_over_i0a = (float)(std::exp(alpha) / p->i0a);
    kb.half2 = (float)(half * half);
    fit_kb_poly(alpha, p->i0a, kb);
    int cpp = o.max_coils_per_pass > 0 ? o.max_coils_per_pass : 8;
    int cb = 1;
    while (cb * 2 <= cpp && cb < 8) cb *= 2;
    // the kernels also hold the candidate tables
    const CandSet &cset = candidate_set(R, g.radial, is2d, o.J, g.P[0], g.P[0] * g.P[1]);
    Cand cnts{};
    for (int q = 0; q < 8; ++q) cnts.cnt[q] = cset.cnt[q];
    const size_t cand_max = std::max(cand_smem_bytes((int)cset.codes.size()), cand_pairs_bytes(cnts));
    while (cb > 1 && smem_plane_bytes(R, cb) + cand_max > 210 * 1024) cb /= 2;
    if (smem_plane_bytes(R, cb) + cand_max > 220 * 1024) {
        delete p;
        return fail(NUFFT3D_ERR_UNSUPPORTED, "interpolation tile too large for shared memory");
    }
    p->coils_per_pass = cb;
    p->max_coils_per_pass = cb;
    if (cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete p;
        return fail(NUFFT3D_ERR_CUDA, "cudaStreamCreate failed");
    }
    p->wait_polls = o.wait_polls;
    int st = dmalloc(&p->work, 16, nullptr);  // per handle: handles may run concurrently
    if (st == NUFFT3D_SUCCESS && cudaMemset(p->work, 0, 16 * sizeof(int)) != cudaSuccess)
        st = fail(NUFFT3D_ERR_CUDA, "cannot clear the plan's work buffer");
    if (st == NUFFT3D_SUCCESS) st = build_plan(p, om, o);
    if (st != NUFFT3D_SUCCESS) {
        std::string msg = nufft3d_last_error();
        free_plan_memory(p);
        delete p;
        return fail(st, msg);
    }
    adopt_tables(p);
    if (o.verbose) {
        std::printf(" Created nufft_3d plan: N=[%d %d %d] K=[%d %d %d] J=%g u=%g alpha=%g radial=%d\n",
                    N[0], N[1], N[2], K[0], K[1], K[2], o.J, o.u, alpha, p->radial);
        std::printf("  %lld points (out of %lld) are within bounds; %.2f taps/sample; %lld blocks\n",
                    (long long)p->nnz, (long long)M, p->taps, (long long)p->n_blocks);
        if (p->tap_ent)
            std::printf("  stored H: %.1f MB\n", (double)p->tap_bytes / 1e6);
        if (p->spread_ent)
            std::printf("  stored H': %.1f MB\n", (double)p->spread_bytes / 1e6);
    }
    *out = p;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_plan_share(const nufft3d_plan *src, nufft3d_plan **out)
{
    clear_error();
    if (!src || !out) return fail(NUFFT3D_ERR_ARG, "NULL argument");
    *out = nullptr;
    NUFFT_DEVICE_LOCK;
    DeviceGuard guard(src->device);
    nufft3d_plan *p = new nufft3d_plan();
    p->device = src->device;
    for (int a = 0; a < 3; ++a) p->N[a] = src->N[a];
    p->M = src->M;
    p->nnz = src->nnz;
    p->J = src->J;
    p->u = src->u;
    p->alpha = src->alpha;
    p->i0a = src->i0a;
    p->radial = src->radial;
    p->geom = src->geom;
    p->kb = src->kb;
    p->samples = src->samples;
    p->perm = src->perm;
    p->inv = src->inv;
    p->blocks = src->blocks;
    p->n_blocks = src->n_blocks;
    p->tile_counts = src->tile_counts;
    p->piece_samples = src->piece_samples;
    p->max_coils_per_pass = src->max_coils_per_pass;
    p->cand = src->cand;
    p->n_cand = src->n_cand;
    p->cand_desc = src->cand_desc;
    p->sm_count = src->sm_count;
    p->interp_sms = src->interp_sms;
    p->coils_per_pass = src->coils_per_pass;
    p->taps = src->taps;
    p->U = src->U;
    p->d = src->d;
    p->d_orig = src->d_orig;
    for (int a = 0; a < 3; ++a) {
        p->tw[a] = src->tw[a];
        p->fft[a] = src->fft[a];
    }
    p->tap_rows = src->tap_rows;
    p->tap_ent = src->tap_ent;
    p->tap_bytes = src->tap_bytes;
    p->spread_pieces = src->spread_pieces;
    p->spread_wstart = src->spread_wstart;
    p->spread_ent = src->spread_ent;
    p->n_spread_pieces = src->n_spread_pieces;
    p->spread_bytes = src->spread_bytes;
    p->table_bytes = src->table_bytes;
    p->tables = src->tables;
    if (cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        p->tables.reset();
        delete p;
        return fail(NUFFT3D_ERR_CUDA, "cudaStreamCreate failed");
    }
    p->wait_polls = src->wait_polls;
    if (dmalloc(&p->work, 16, nullptr) != NUFFT3D_SUCCESS || cudaMemset(p->work, 0, 16 * sizeof(int)) != cudaSuccess) {
        std::string msg = p->work ? std::string("cannot clear the handle's work buffer") : nufft3d_last_error();
        if (p->work) cudaFree(p->work);
        cudaStreamDestroy(p->own_stream);
        p->tables.reset();
        delete p;
        return fail(NUFFT3D_ERR_NOMEM, msg);
    }
    if (src->own_blocks) {
        // a tuned source: this handle gets its own copy of the piece table
        if (dmalloc(&p->own_blocks, (size_t)std::max<int64_t>(p->n_blocks, 1), nullptr) != NUFFT3D_SUCCESS ||
            cudaMemcpy(p->own_blocks, src->own_blocks, sizeof(int4) * p->n_blocks, cudaMemcpyDeviceToDevice) !=
                cudaSuccess) {
            std::string msg = nufft3d_last_error();
            free_plan_memory(p);
            p->tables.reset();
            delete p;
            return fail(NUFFT3D_ERR_NOMEM, msg.empty() ? std::string("cannot copy the piece table") : msg);
        }
        p->blocks = p->own_blocks;
    }
    *out = p;
    return NUFFT3D_SUCCESS;
}

int nufft3d::rebuild_pieces(nufft3d_plan *p, int S)
{
    if (S < 32) return fail(NUFFT3D_ERR_ARG, "pieces must hold at least 32 samples");
    const std::vector<int4> blocks = make_pieces(p->tile_counts, S);
    int4 *nb = nullptr;
    NUFFT_TRY(dmalloc(&nb, std::max<size_t>(blocks.size(), 1), nullptr));
    cudaStream_t s = p->own_stream;
    cudaError_t e = blocks.empty() ? cudaSuccess
                                   : cudaMemcpyAsync(nb, blocks.data(), sizeof(int4) * blocks.size(),
                                                     cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        NUFFT_DEVICE_LOCK;
        cudaFree(nb);
        return fail(NUFFT3D_ERR_CUDA, std::string("piece table: ") + cudaGetErrorString(e));
    }
    {
        NUFFT_DEVICE_LOCK;
        if (p->own_blocks) cudaFree(p->own_blocks);
    }
    p->own_blocks = nb;
    p->blocks = nb;
    p->n_blocks = (int64_t)blocks.size();
    p->piece_samples = S;
    NUFFT_TRY(launch_weight_sum(p, s));
    NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_plan_set_sms(nufft3d_plan *p, int sms)
{
    clear_error();
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    if (sms < 0) return fail(NUFFT3D_ERR_ARG, "sms must be nonnegative");
    p->interp_sms = sms;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_plan_set_host_copy(nufft3d_plan *p, int mode)
{
    clear_error();
    if (!p) return fail(NUFFT3D_ERR_ARG, "plan is NULL");
    if (mode != 0 && mode != 1) return fail(NUFFT3D_ERR_ARG, "host copy mode must be 0 or 1");
    p->host_copy = mode;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_plan_footprint(const nufft3d_plan *p, int nc, int with_solver, int64_t *bytes)
{
    clear_error();
    if (!p || !bytes || nc < 1) return fail(NUFFT3D_ERR_ARG, "invalid argument");
    const int64_t K1 = p->geom.K[0], K2 = p->geom.K[1], K3 = p->geom.K[2];
    const int64_t N1 = p->N[0], N2 = p->N[1], N3 = p->N[2];
    const int64_t c8 = 8 * (int64_t)nc;
    int64_t b = (K1 * N2 * N3 + K1 * K2 * N3 + (p->geom.is2d ? 0 : K1 * K2 * K3)) * c8 +
                (p->nnz > 0 ? p->nnz : 1) * c8;
    if (with_solver) b += 7 * N1 * N2 * N3 * c8 + 4 * p->nnz;
    *bytes = b;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_plan_destroy(nufft3d_plan *p)
{
    clear_error();
    if (!p) return NUFFT3D_SUCCESS;
    {
        NUFFT_DEVICE_LOCK;
        DeviceGuard guard(p->device);
        if (p->own_stream) cudaStreamSynchronize(p->own_stream);
        free_plan_memory(p);
    }
    delete p;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_plan_info(const nufft3d_plan *p, nufft3d_info *info)
{
    clear_error();
    if (!p || !info) return fail(NUFFT3D_ERR_ARG, "NULL argument");
    for (int a = 0; a < 3; ++a) {
        info->N[a] = p->N[a];
        info->K[a] = p->geom.K[a];
        info->tile[a] = p->geom.T[a];
    }
    info->M = p->M;
    info->nnz = p->nnz;
    info->J = p->J;
    info->u = p->u;
    info->alpha = p->alpha;
    info->radial = p->radial;
    info->n_blocks = p->n_blocks;
    info->taps_per_sample = p->taps;
    info->device_bytes = p->table_bytes + (int64_t)p->scratch.bytes;
    info->tap_table_bytes = p->tap_bytes;
    info->kernel_polynomial = p->kb.poly;
    info->spread_table_bytes = p->spread_bytes;
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_get_deap(const nufft3d_plan *p, float *U)
{
    clear_error();
    if (!p || !U) return fail(NUFFT3D_ERR_ARG, "NULL argument");
    DeviceGuard guard(p->device);
    const size_t n = (size_t)p->N[0] * p->N[1] * p->N[2];
    NUFFT_CUDA_TRY(cudaMemcpy(U, p->U, n * sizeof(float), cudaMemcpyDeviceToHost));
    return NUFFT3D_SUCCESS;
}

extern "C" int nufft3d_get_density(const nufft3d_plan *p, float *d)
{
    clear_error();
    if (!p || !d) return fail(NUFFT3D_ERR_ARG, "NULL argument");
    DeviceGuard guard(p->device);
    NUFFT_CUDA_TRY(cudaMemcpy(d, p->d_orig, (size_t)p->M * sizeof(float), cudaMemcpyDeviceToHost));
    return NUFFT3D_SUCCESS;
}

extern "C" const char *nufft3d_last_error(void) { return g_last_error.c_str(); }

extern "C" const char *nufft3d_version(void) { return "nufft3d-gb300 0.1 (sm_103a)"; }
