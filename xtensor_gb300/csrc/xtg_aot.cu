// xtg_aot.cu — kernels compiled ahead of time by nvcc for sm_103a:
// the seeded synthetic-data generator used by the benchmark workloads.
//
// Element i of the array gets a value from a counter-based generator keyed
// by (seed, i): splitmix64 (Steele, Lea & Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014) of a seed-scrambled index,
// turned into uniforms, Box-Muller normals, sign-random lognormals or
// integers.  The values do not depend on the launch configuration.
#include <cuda_runtime.h>

#include <cstdint>

#include "xtg_internal.h"

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <class T> struct Put {
    static __device__ __forceinline__ T go(double v) { return (T)v; }
};
template <> struct Put<unsigned short> {  // bfloat16 bits, round to nearest even
    static __device__ __forceinline__ unsigned short go(double v) {
        float f = (float)v;
        unsigned u = __float_as_uint(f);
        if ((u & 0x7fffffffu) > 0x7f800000u) return (unsigned short)((u >> 16) | 0x40u);
        u += 0x7fffu + ((u >> 16) & 1u);
        return (unsigned short)(u >> 16);
    }
};

template <class T, bool WIDE>
__global__ void __launch_bounds__(256) k_fill(T* out, long long n, int dist, double p0, double p1, unsigned long long seed) {
    const unsigned long long key = mix64(seed ^ 0xD1B54A32D192ED03ull);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long x = mix64(key + (unsigned long long)i);
        double v;
        if (dist == 3) {
            const long long lo = (long long)p0, hi = (long long)p1;
            const unsigned long long span = (unsigned long long)(hi - lo) + 1ull;
            v = (double)(lo + (long long)(x % span));
            out[i] = Put<T>::go(v);
            continue;
        }
        if (WIDE) {
            const double u1 = ((double)(x >> 11) + 0.5) * 0x1.0p-53;
            const double u2 = ((double)(mix64(x) >> 11) + 0.5) * 0x1.0p-53;
            if (dist == 0) {
                v = p0 + (p1 - p0) * u1;
            } else {
                const double z = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
                v = dist == 1 ? p0 + p1 * z : exp(p0 + p1 * z) * ((x & 1ull) ? -1.0 : 1.0);
            }
        } else {
            const float u1 = ((float)(x >> 40) + 0.5f) * 0x1.0p-24f;
            const float u2 = ((float)((x >> 16) & 0xFFFFFFull) + 0.5f) * 0x1.0p-24f;
            float f;
            if (dist == 0) {
                f = (float)p0 + (float)(p1 - p0) * u1;
            } else {
                const float z = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
                f = dist == 1 ? (float)p0 + (float)p1 * z : expf((float)p0 + (float)p1 * z) * ((x & 1ull) ? -1.0f : 1.0f);
            }
            v = (double)f;
        }
        out[i] = Put<T>::go(v);
    }
}

template <class T, bool WIDE>
xtg_status fill(void* p, long long n, int dist, double p0, double p1, unsigned long long seed, cudaStream_t s) {
    xtgh::DeviceInfo* dev;
    XTG_TRY(xtgh::ensure_device(&dev));
    long long blocks = (n + 255) / 256;
    const long long cap = (long long)dev->sm_count * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_fill<T, WIDE><<<(unsigned)blocks, 256, 0, s>>>((T*)p, n, dist, p0, p1, seed);
    XTG_CUDA(cudaGetLastError());
    xtgh::count_launch();
    return XTG_OK;
}

}  // namespace

extern "C" xtg_status xtg_fill_random(const xtg_array* a, int32_t dist, double p0, double p1, uint64_t seed,
                                      xtg_stream stream) {
    using namespace xtgh;
    if (!a) return fail(XTG_ERR_INVALID, "null array");
    if (dist < 0 || dist > 3) return fail(XTG_ERR_INVALID, "unknown distribution");
    long long n = 1, expect = 1;
    for (int d = a->rank - 1; d >= 0; --d) {
        if (a->shape[d] != 1 && a->strides[d] != expect) return fail(XTG_ERR_UNSUPPORTED, "fill needs a contiguous array");
        expect *= a->shape[d];
        n *= a->shape[d];
    }
    if (n == 0) return XTG_OK;
    if (!a->data) return fail(XTG_ERR_INVALID, "null data");
    cudaStream_t s = (cudaStream_t)stream;
    switch (a->dtype) {
        case XTG_FLOAT32: return fill<float, false>(a->data, n, dist, p0, p1, seed, s);
        case XTG_FLOAT64: return fill<double, true>(a->data, n, dist, p0, p1, seed, s);
        case XTG_BFLOAT16: return fill<unsigned short, false>(a->data, n, dist, p0, p1, seed, s);
        case XTG_INT32: return fill<int, false>(a->data, n, dist, p0, p1, seed, s);
        case XTG_INT64: return fill<long long, true>(a->data, n, dist, p0, p1, seed, s);
        default: return fail(XTG_ERR_UNSUPPORTED, "fill: unsupported dtype");
    }
}
