// fgc_misc.cu -- clears, box downsample, DepthImage, and the mesh weld.
//
// The weld gives every distinct position bit pattern of a triangle soup one
// vertex-stage slot: equal inputs through the same arithmetic give equal
// outputs, so transforming each distinct position once is bit-identical to
// the reference's per-corner Shader.Vertex calls (shader.go:20-23), and does
// about a sixth of the FP64 work on a closed mesh.
#include "fgc_internal.cuh"

namespace fgc {

__global__ void fill_u32_kernel(uint32_t* p, uint64_t n, uint32_t v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// MakeColor of a 16-bit texel (color.go:25-29): float64(c) / 0xffff per
// channel, once per texture instead of once per bilinear tap.
__global__ void texel_unit_kernel(const ushort4* src, uint64_t n, double* dst) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const ushort4 p = src[i];
        const double d = 65535.0;
        dst[4 * i + 0] = __ddiv_rn((double)p.x, d);
        dst[4 * i + 1] = __ddiv_rn((double)p.y, d);
        dst[4 * i + 2] = __ddiv_rn((double)p.z, d);
        dst[4 * i + 3] = __ddiv_rn((double)p.w, d);
    }
}

__global__ void fill_f64_kernel(double* p, uint64_t n, double v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// Box downsample: output channel = (sum + n/2) / n over the scale*scale block.
__global__ void downsample_kernel(const uint32_t* src, int32_t w, int32_t h, int32_t scale, uint32_t* dst) {
    const int32_t ow = w / scale, oh = h / scale;
    const uint64_t n = (uint64_t)ow * oh;
    const uint32_t cnt = (uint32_t)scale * (uint32_t)scale;
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < n; o += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t ox = (int32_t)(o % ow), oy = (int32_t)(o / ow);
        uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (int32_t dy = 0; dy < scale; dy++) {
            const uint32_t* row = src + (uint64_t)(oy * scale + dy) * w + (uint64_t)ox * scale;
            for (int32_t dx = 0; dx < scale; dx++) {
                uint32_t v = row[dx];
                s0 += v & 0xff;
                s1 += (v >> 8) & 0xff;
                s2 += (v >> 16) & 0xff;
                s3 += v >> 24;
            }
        }
        const uint32_t hlf = cnt / 2;
        dst[o] = ((s0 + hlf) / cnt) | (((s1 + hlf) / cnt) << 8) | (((s2 + hlf) / cnt) << 16) |
                 (((s3 + hlf) / cnt) << 24);
    }
}

// Total order on doubles as unsigned keys (negative values reversed).
__device__ __forceinline__ unsigned long long dkey(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dunkey(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// DepthImage's lo/hi scan (context.go:88-100): values equal to MaxFloat64 and
// NaN are skipped; lo only moves below MaxFloat64, hi above -MaxFloat64.
__global__ void depth_minmax_kernel(const double* d, uint64_t n, unsigned long long* lohi) {
    const double maxf = 1.7976931348623157e308;
    unsigned long long lo = dkey(maxf), hi = dkey(-maxf);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        double v = d[i];
        if (v == maxf || v != v) continue;
        unsigned long long k = dkey(v);
        if (v < maxf && k < lo) lo = k;
        if (v > -maxf && k > hi) hi = k;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long a = __shfl_down_sync(0xffffffffu, lo, o);
        unsigned long long b = __shfl_down_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&lohi[0], lo);
        atomicMax(&lohi[1], hi);
    }
}

// DepthImage's mapping (context.go:102-116): t = (d - lo) / (hi - lo), 1 for
// MaxFloat64, gray = uint16(t * 0xffff).
__global__ void depth_image_kernel(const double* d, uint64_t n, const unsigned long long* lohi, uint16_t* out) {
    const double maxf = 1.7976931348623157e308;
    const double lo = dunkey(lohi[0]), hi = dunkey(lohi[1]);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        double v = d[i];
        double t = __ddiv_rn(__dsub_rn(v, lo), __dsub_rn(hi, lo));
        if (v == maxf) t = 1;
        out[i] = (uint16_t)(go_f2i(__dmul_rn(t, 65535.0)) & 0xffff);
    }
}

// ---------------------------------------------------------------------------
// Weld
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void weld_insert_kernel(const double* cp, uint64_t n, uint32_t* table, uint64_t tmask, uint32_t* slot_of,
                                   uint32_t* minc, unsigned int* status) {
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        const long long bx = __double_as_longlong(cp[3 * c]);
        const long long by = __double_as_longlong(cp[3 * c + 1]);
        const long long bz = __double_as_longlong(cp[3 * c + 2]);
        uint64_t h = mix64((unsigned long long)bx ^ mix64((unsigned long long)by ^ mix64((unsigned long long)bz))) & tmask;
        uint32_t slot = 0xFFFFFFFFu;
        for (uint64_t probe = 0; probe <= tmask; probe++) {
            uint32_t cur = table[h];
            if (cur == 0xFFFFFFFFu) {
                cur = atomicCAS(&table[h], 0xFFFFFFFFu, (uint32_t)c);
                if (cur == 0xFFFFFFFFu) {
                    slot = (uint32_t)h;
                    break;
                }
            }
            if (__double_as_longlong(cp[3 * (uint64_t)cur]) == bx &&
                __double_as_longlong(cp[3 * (uint64_t)cur + 1]) == by &&
                __double_as_longlong(cp[3 * (uint64_t)cur + 2]) == bz) {
                slot = (uint32_t)h;
                break;
            }
            h = (h + 1) & tmask;
        }
        if (slot == 0xFFFFFFFFu) {
            atomicOr(status, ST_POOL_OVERFLOW);
            slot = 0;
        }
        slot_of[c] = slot;
        atomicMin(&minc[slot], (uint32_t)c);
    }
}

__global__ void weld_flag_kernel(const uint32_t* slot_of, const uint32_t* minc, uint64_t n, uint32_t* flag) {
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x)
        flag[c] = (minc[slot_of[c]] == (uint32_t)c) ? 1u : 0u;
}

__global__ void weld_emit_kernel(const double* cp, const uint32_t* slot_of, const uint32_t* minc, const uint32_t* uid,
                                 uint64_t n, double* ux, double* uy, double* uz, uint32_t* corner_uniq) {
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t rep = minc[slot_of[c]];
        const uint32_t u = uid[rep];
        corner_uniq[c] = u;
        if (rep == (uint32_t)c) {
            ux[u] = cp[3 * c];
            uy[u] = cp[3 * c + 1];
            uz[u] = cp[3 * c + 2];
        }
    }
}

__global__ void attrs_kernel(const double* cp, const double* nrm, uint64_t n, APosNrm64* pn64, APosNrm32* pn32) {
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        APosNrm64 a;
        a.px = cp[3 * c];
        a.py = cp[3 * c + 1];
        a.pz = cp[3 * c + 2];
        a.nx = nrm ? nrm[3 * c] : 0.0;
        a.ny = nrm ? nrm[3 * c + 1] : 0.0;
        a.nz = nrm ? nrm[3 * c + 2] : 0.0;
        pn64[c] = a;
        pn32[c] = APosNrm32{(float)a.px, (float)a.py, (float)a.pz, (float)a.nx, (float)a.ny, (float)a.nz};
    }
}

// FP64 pipe throughput probe: eight independent add chains per thread.
__global__ void fp64_rate_kernel(double* out, double a, double b, int iters) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
           x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = __dadd_rn(x0, a); x1 = __dadd_rn(x1, b); x2 = __dadd_rn(x2, a); x3 = __dadd_rn(x3, b);
        x4 = __dadd_rn(x4, a); x5 = __dadd_rn(x5, b); x6 = __dadd_rn(x6, a); x7 = __dadd_rn(x7, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void f64_to_f32_kernel(const double* in, uint64_t n, float* out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

}  // namespace fgc
