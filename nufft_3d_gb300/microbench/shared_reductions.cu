// Shared-memory accumulation throughput on the current GPU: the ceiling for
// the spread's integer reductions.  Each variant adds ITERS values per thread
// into a 32 KB shared array at in-range indices (all < NS) with:
//   0  atomicAdd(float)            (FP32 shared atomics)
//   1  red.shared.add.u32, random addresses across the array
//   2  red.shared.add.u32, one word per lane of a warp-uniform row (no bank conflicts)
//   3  red.shared.add.u64, random addresses
// Prints lane-operations per clock per SM at the measured SM clock.
// Build: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o shared_reductions shared_reductions.cu
#include <cstdio>
#include <cuda_runtime.h>

constexpr int NS = 8192;     // 32-bit words in the shared array
constexpr int ITERS = 4096;

template <int MODE>
__global__ void k(unsigned *out, int salt)
{
    __shared__ unsigned t[NS];
    for (int i = threadIdx.x; i < NS; i += blockDim.x) t[i] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    unsigned h = threadIdx.x * 2654435761u + blockIdx.x * 97u + salt;
    unsigned hw = (threadIdx.x >> 5) * 2654435761u + blockIdx.x * 97u + salt;
    for (int it = 0; it < ITERS; ++it) {
        h = h * 1664525u + 1013904223u;
        hw = hw * 1664525u + 1013904223u;
        if (MODE == 0) {
            atomicAdd(reinterpret_cast<float *>(&t[(h >> 8) & (NS - 1)]), 1.0f);
        } else if (MODE == 1) {
            const unsigned a = (unsigned)__cvta_generic_to_shared(&t[(h >> 8) & (NS - 1)]);
            asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(a), "r"(1u) : "memory");
        } else if (MODE == 2) {
            const unsigned a = (unsigned)__cvta_generic_to_shared(&t[((hw >> 8) & (NS / 32 - 1)) * 32 + lane]);
            asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(a), "r"(1u) : "memory");
        } else {
            const unsigned a = (unsigned)__cvta_generic_to_shared(&t[(h >> 8) & (NS - 2)]);
            asm volatile("red.shared.add.u64 [%0], %1;" ::"r"(a), "l"(1ull) : "memory");
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NS; i += blockDim.x) atomicAdd(&out[i], t[i]);
}

int main()
{
    unsigned *out = nullptr;
    if (cudaMalloc(&out, NS * sizeof(unsigned)) != cudaSuccess) return 1;
    int sms = 0, khz = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, 0);
    const double clk = khz * 1e3;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const char *names[4] = {"atomicAdd f32 (random)", "red.shared.add.u32 (random)",
                            "red.shared.add.u32 (conflict-free)", "red.shared.add.u64 (random)"};
    const int blocks = sms * 4, threads = 512;
    for (int mode = 0; mode < 4; ++mode) {
        for (int rep = 0; rep < 2; ++rep) {
            cudaEventRecord(a);
            if (mode == 0) k<0><<<blocks, threads>>>(out, rep);
            if (mode == 1) k<1><<<blocks, threads>>>(out, rep);
            if (mode == 2) k<2><<<blocks, threads>>>(out, rep);
            if (mode == 3) k<3><<<blocks, threads>>>(out, rep);
            cudaEventRecord(b);
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            const double ops = (double)blocks * threads * ITERS;
            if (rep)
                printf("%-36s %8.3f ms  %6.2f lane-ops/clk/SM (%d SMs, %.0f MHz nominal)\n", names[mode], ms,
                       ops / (ms * 1e-3) / sms / clk, sms, clk / 1e6);
        }
    }
    const cudaError_t e = cudaDeviceSynchronize();
    printf("status: %s\n", cudaGetErrorString(e));
    cudaFree(out);
    return e != cudaSuccess;
}
