// Checks div_by_rcp (fauxgl_gb300/csrc/fgc_device.cuh: x / w from the
// correctly rounded reciprocal, Markstein's two-correction scheme) against
// __ddiv_rn on the GPU, bit for bit: seeded operands across the fast path's
// exponent range and its edges, clip-space-like values, quotients next to
// representable numbers and next to midpoints, and operands outside the range
// (zeros, subnormals, infinities, NaN, any bit pattern). Prints
// "ok <cases>" or the first mismatch and exits 1.
// Build: nvcc -gencode arch=compute_103a,code=sm_103a -O3 --fmad=false -std=c++17 divrcp_check.cu
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "../fauxgl_gb300/csrc/fgc_device.cuh"

namespace {

__device__ uint64_t mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ double from_bits(uint64_t b) { return __longlong_as_double((long long)b); }
__device__ uint64_t to_bits(double d) { return (uint64_t)__double_as_longlong(d); }

constexpr uint64_t kMant = 0x000fffffffffffffull;

// sign from bit 0 of r, biased exponent lo + (r >> 1) % span, mantissa m
__device__ double make(uint64_t r, uint64_t m, uint64_t lo, uint64_t span) {
    return from_bits(((r & 1) << 63) | ((lo + ((r >> 1) % span)) << 52) | (m & kMant));
}

__global__ void check(uint64_t seed, uint64_t per_thread, unsigned long long* bad, unsigned long long* first) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint64_t i = 0; i < per_thread; i++) {
        const uint64_t s = mix(seed ^ mix(tid * per_thread + i));
        const uint64_t r1 = mix(s + 1), r2 = mix(s + 2), r3 = mix(s + 3), r4 = mix(s + 4);
        double x, w;
        switch (s & 7) {
            case 0:
            case 1:  // the whole fast-path range, 2^-450 .. 2^450
                x = make(r1, r2, 1023 - 450, 901);
                w = make(r3, r4, 1023 - 450, 901);
                break;
            case 2:  // clip-space-like coordinates
                x = make(r1, r2, 1023 - 12, 24);
                w = make(r3, r4, 1023 - 12, 24);
                break;
            case 3: {  // quotient within a few ulps of a representable q
                const double q = make(r1, r2, 1023 - 40, 80);
                w = make(r3, r4, 1023 - 40, 80);
                x = from_bits(to_bits(__dmul_rn(q, w)) + (r3 >> 40) % 5 - 2);
                break;
            }
            case 4: {  // quotient next to the midpoint between q and its successor
                const double q = make(r1, r2, 1023 - 40, 80);
                w = make(r3, r4, 1023 - 40, 80);
                const double h = from_bits((((to_bits(q) >> 52) & 0x7ff) - 53) << 52);  // half an ulp of |q|
                x = __fma_rn(h, w, __dmul_rn(q, w));
                x = from_bits(to_bits(x) + (r4 >> 40) % 3 - 1);
                break;
            }
            case 5: {  // exponents at and around the fast path's limits
                const uint64_t edges[8] = {621, 622, 623, 624, 1421, 1422, 1423, 1424};
                x = from_bits(((r1 & 1) << 63) | (edges[(r1 >> 8) & 7] << 52) | (r2 & kMant));
                w = from_bits(((r3 & 1) << 63) | (edges[(r3 >> 8) & 7] << 52) | (r4 & kMant));
                if ((r1 >> 16) & 1) x = make(r1 >> 20, r2, 1023 - 12, 24);
                if ((r3 >> 16) & 1) w = make(r3 >> 20, r4, 1023 - 12, 24);
                break;
            }
            case 6:  // any bit pattern
                x = from_bits(r1);
                w = from_bits(r2);
                break;
            default: {  // special operands against ordinary ones
                const uint64_t sp[8] = {0ull, 0x8000000000000000ull, 1ull, 0x000fffffffffffffull,
                                        0x7ff0000000000000ull, 0x7ff8000000000000ull, 0x3ff0000000000000ull,
                                        0x0010000000000000ull};
                x = (r1 >> 8) & 1 ? from_bits(sp[r1 & 7] | ((r1 >> 9) & 1) << 63) : make(r2, r3, 1023 - 12, 24);
                w = (r1 >> 10) & 1 ? from_bits(sp[(r1 >> 11) & 7] | ((r1 >> 14) & 1) << 63) : make(r4, r3, 1023 - 12, 24);
                break;
            }
        }
        const double a = fgc::div_by_rcp(x, w, __drcp_rn(w));
        const double b = __ddiv_rn(x, w);
        if (to_bits(a) != to_bits(b) && !(a != a && b != b)) {
            if (atomicAdd(bad, 1ull) == 0) {
                first[0] = to_bits(x);
                first[1] = to_bits(w);
                first[2] = to_bits(a);
                first[3] = to_bits(b);
            }
        }
    }
}

}  // namespace

int main(int argc, char** argv) {
    const uint64_t per_thread = argc > 1 ? strtoull(argv[1], nullptr, 10) : 256;
    const int blocks = 152 * 8, threads = 256;
    unsigned long long *bad, *first;
    if (cudaMalloc(&bad, 8) != cudaSuccess || cudaMalloc(&first, 32) != cudaSuccess) return 2;
    cudaMemset(bad, 0, 8);
    cudaMemset(first, 0, 32);
    uint64_t cases = 0;
    for (uint64_t seed = 1; seed <= 4; seed++) {
        check<<<blocks, threads>>>(seed * 0x5851F42D4C957F2Dull, per_thread, bad, first);
        cases += (uint64_t)blocks * threads * per_thread;
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        printf("cuda error %s\n", cudaGetErrorString(e));
        return 2;
    }
    unsigned long long nbad = 0, f[4] = {0, 0, 0, 0};
    cudaMemcpy(&nbad, bad, 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(f, first, 32, cudaMemcpyDeviceToHost);
    if (nbad) {
        printf("%llu mismatches of %llu; first x=%016llx w=%016llx got %016llx want %016llx\n", nbad,
               (unsigned long long)cases, f[0], f[1], f[2], f[3]);
        return 1;
    }
    printf("ok %llu\n", (unsigned long long)cases);
    return 0;
}
