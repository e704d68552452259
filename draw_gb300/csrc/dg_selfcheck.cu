// dg_selfcheck.cu -- on-device self-check of the exact-division identity that
// the raster pass uses in place of IEEE division (div_rcp in dg_device.cuh):
// for seeded operand pairs in the ranges the raster pass admits, div_rcp(a, b,
// RN(1/b)) and -a over b must be bit-identical to __fdiv_rn.
#include <cstring>

#include "dg_device.cuh"
#include "dg_host.h"

namespace {

// splitmix64's output mix (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014)
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Sample i of a mode, as (a, b) with a >= 0 (the kernel also checks -a):
// 0: every integer pair 0 <= a <= b <= 4096 (i = b * 4097 + a; others skipped);
// 1: b an integer in [1, 2^24], a an integer in [0, b];
// 2: b integer-valued in [1, 2^101), a integer-valued in [0, 4b);
// 3: a in [1, 2^61) and b in [1, 2^100) with random mantissas.
__device__ __forceinline__ bool div_sample(int mode, uint64_t i, uint64_t seed, float& a, float& b) {
    if (mode == 0) {
        const uint32_t bb = (uint32_t)(i / 4097u), aa = (uint32_t)(i % 4097u);
        if (bb == 0u || aa > bb) return false;
        a = (float)aa;
        b = (float)bb;
        return true;
    }
    const uint64_t h = mix64(i ^ (seed * 0x2545F4914F6CDD1Dull));
    if (mode == 1) {
        const uint32_t bb = 1u + (uint32_t)(h & 0xFFFFFFu);
        a = (float)(uint32_t)((h >> 24) % (bb + 1ull));
        b = (float)bb;
    } else if (mode == 2) {
        const float m = 1.0f + (float)((h >> 8) & 0x7FFFFFu) * 0x1p-23f;
        b = floorf(ldexpf(m, (int)(h % 101u)));
        const float f = (float)((h >> 32) & 0xFFFFFFu) * 0x1p-22f;  // [0, 4)
        a = floorf(__fmul_rn(b, f));
    } else {
        b = ldexpf(1.0f + (float)(h & 0x7FFFFFu) * 0x1p-23f, (int)((h >> 23) % 100u));
        a = ldexpf(1.0f + (float)((h >> 30) & 0x7FFFFFu) * 0x1p-23f, (int)((h >> 53) % 61u));
    }
    return true;
}

__global__ void __launch_bounds__(256) k_check_division(int mode, uint64_t n, uint64_t seed,
                                                        unsigned long long* out) {
    // out[0]: mismatches; out[1]: the first recorded mismatch as a (high word) and b bits
    unsigned long long bad = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float a, b;
        if (!div_sample(mode, i, seed, a, b)) continue;
        const float y = __frcp_rn(b);
        const float q = div_rcp(a, b, y), r = fD(a, b);
        const float qn = div_rcp(-a, b, y), rn = fD(-a, b);
        if (__float_as_uint(q) != __float_as_uint(r) || __float_as_uint(qn) != __float_as_uint(rn)) {
            if (bad == 0) atomicCAS(out + 1, 0ull, ((unsigned long long)__float_as_uint(a) << 32) | __float_as_uint(b));
            bad++;
        }
    }
    if (bad) atomicAdd(out, bad);
}

}  // namespace

dg_status dg_check_division(dg_ctx* c, int32_t mode, uint64_t samples, uint64_t seed, uint64_t* mismatches,
                            float* first_a, float* first_b) {
    if (!c || !mismatches || mode < 0 || mode > 3) return DG_E_INVALID;
    dg_status e = dgh::set_device(c);
    if (e != DG_OK) return e;
    if (mode == 0 && samples > 4097ull * 4097ull) samples = 4097ull * 4097ull;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return DG_E_OOM;
    cudaStream_t s = c->main.stream;
    cudaError_t ce = cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), s);
    if (ce == cudaSuccess) {
        k_check_division<<<(unsigned)c->nsm * 8u, 256, 0, s>>>(mode, samples, seed, d);
        ce = cudaGetLastError();
    }
    unsigned long long h[2] = {0, 0};
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    cudaFree(d);
    if (ce != cudaSuccess) return DG_E_CUDA;
    *mismatches = h[0];
    const uint32_t ab = (uint32_t)(h[1] >> 32), bb = (uint32_t)h[1];
    float fa, fb;
    memcpy(&fa, &ab, 4);
    memcpy(&fb, &bb, 4);
    if (first_a) *first_a = fa;
    if (first_b) *first_b = fb;
    return DG_OK;
}
