// fgc_bin.cu -- integer binning of raster primitives into screen bands.
//
// A band is a contiguous range of L = R*W linear pixel indices (R whole rows).
// Binning by linear index rather than by (x, y) reproduces the reference's
// row wrap-around for free: rasterize only range-checks i = y*W + x against
// [0, W*H) (context.go:223-228), so a fragment left or right of the screen
// lands in the neighbouring row, and a primitive whose index range
// [y0*W + x0, y1*W + x1] meets a band is binned there.
//
// The bins must list primitives in submission order (ties resolve "later
// wins", context.go:248). Count, scan and scatter are all integer and
// deterministic. Every draw of a pass owns a run of binning blocks, a
// [band][block] slab of the count matrix and a run of bands:
//   bin_count    per-block band histograms -> mat[draw][band][block]
//   scan_u32     one exclusive scan of the whole matrix -> off (a draw's
//                bins follow the previous draw's)
//   bin_scatter  per block, warps own consecutive sub-ranges; a stable rank
//                inside each 32-primitive round comes from comparing band
//                ranges across lanes, so the output order is the input order.
#include "fgc_fpjump.cuh"
#include "fgc_internal.cuh"

namespace fgc {

constexpr unsigned int kRetryBits = ST_CLIP_OVERFLOW | ST_POOL_OVERFLOW | ST_LOOKBACK_TIMEOUT;

// A binning block's draw and its share [lo, hi) of the draw's primitives.
struct BinBlock {
    uint32_t item, lblk, nblk;
    bool row_table;
    uint64_t mat0;
    uint64_t lo, hi;
    BandGeom G;
};

__device__ __forceinline__ BinBlock bin_block(const BinParams& P) {
    BinBlock B;
    B.item = find_item(P.starts.blk, P.nitems, blockIdx.x);
    const ItemView& I = P.items[B.item];
    B.lblk = blockIdx.x - I.blk0;
    B.nblk = I.nblk;
    B.mat0 = I.mat0;
    B.G = BandGeom{I.W, I.H, I.R, I.nbands};
    B.row_table = I.row_table != 0;
    // a failed earlier stage means this pass is re-run: bin nothing
    const bool skip = (*P.status & kRetryBits) != 0;
    const uint64_t p0 = P.iout[B.item].prim_start;
    const uint64_t n = skip ? 0 : P.iout[B.item].prim_end - p0;
    const uint64_t chunk = (n + B.nblk - 1) / B.nblk;
    B.lo = p0 + min((uint64_t)B.lblk * chunk, n);
    B.hi = p0 + min((uint64_t)B.lblk * chunk + chunk, n);
    return B;
}

__global__ void __launch_bounds__(256) bin_count_kernel(BinParams P) {
    extern __shared__ uint32_t hist[];
    const BinBlock B = bin_block(P);
    const uint32_t nb = B.G.nbands;
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (uint64_t p = B.lo + threadIdx.x; p < B.hi; p += blockDim.x) {
        uint32_t bl, bh, cnt = 0;
        const PBox bx = P.pbox[p];
        if (prim_bands(B.G, bx, bl, bh)) {
            for (uint32_t b = bl; b <= bh; b++) atomicAdd(&hist[b], 1u);
            if (B.row_table && uses_row_table(bx)) cnt = bh - bl + 1;
        }
        P.pnb[p] = cnt;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) P.mat[B.mat0 + (uint64_t)i * B.nblk + B.lblk] = hist[i];
}

// Row starts of every (primitive, band) pair: the edge values at its first
// row in each of its bands (the first row of the box whose index range meets
// the band, as the raster stage counts them), by the reference's per-row
// adds b12 from the primitive's top row (context.go:275-277). A block takes
// 256 primitives and splits each one's bands into segments of kRowSeg; one
// thread per segment jumps from the top row to the segment's first row (the
// exact serial sum, fgc_fpjump.cuh) and adds row by row from there, so a
// tall primitive no longer holds its warp while the others' lanes idle.
// Gaps above 64 rows between bands are crossed with exact jumps as well.
constexpr uint32_t kRowSeg = 8;

__device__ __forceinline__ double row_advance(double w, double b, int64_t gap) {
    if (gap > 64) return repeat_add(w, b, (uint64_t)gap);
    for (int64_t j = 0; j < gap; j++) w = __dadd_rn(w, b);
    return w;
}

__global__ void __launch_bounds__(256) row_starts_kernel(RowStartParams P) {
    __shared__ uint32_t s_seg[256];     // per primitive of the tile: its first segment
    __shared__ uint64_t s_warp[256 / 32 + 1];
    __shared__ unsigned int s_stop;
    // one read of the status for the whole block (the block's barriers need
    // every thread; another block may set the overflow bit meanwhile)
    if (threadIdx.x == 0) s_stop = *P.status & (kRetryBits | ST_BIN_OVERFLOW);
    __syncthreads();
    if (s_stop) return;
    const uint64_t n = *P.prim_total;
    for (uint64_t t0 = (uint64_t)blockIdx.x * 256; t0 < n; t0 += (uint64_t)gridDim.x * 256) {
        const uint64_t p0 = t0 + threadIdx.x;
        const uint32_t cnt0 = p0 < n ? P.pnb[p0] : 0u;
        uint64_t total;
        const uint64_t first = block_exclusive_scan<256>((cnt0 + kRowSeg - 1) / kRowSeg, s_warp, &total);
        s_seg[threadIdx.x] = (uint32_t)first;
        __syncthreads();
        for (uint32_t sg = threadIdx.x; sg < (uint32_t)total; sg += blockDim.x) {
            // the primitive holding segment sg: the last one starting at or before it
            uint32_t lo = 0, hi = 255;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (s_seg[mid] <= sg) lo = mid;
                else hi = mid - 1;
            }
            const uint64_t p = t0 + lo;
            const uint32_t cnt = P.pnb[p];
            const uint32_t j0 = (sg - s_seg[lo]) * kRowSeg;  // the segment's first band (relative)
            const uint64_t base = P.prs[p];
            if (base + cnt > P.cap) {
                atomicOr(P.status, ST_BIN_OVERFLOW);
                continue;
            }
            uint32_t ilo = 0, ihi = P.nitems - 1;  // the draw holding primitive p
            while (ilo < ihi) {
                const uint32_t mid = (ilo + ihi + 1) >> 1;
                if (P.iout[mid].prim_start <= p) ilo = mid;
                else ihi = mid - 1;
            }
            const ItemView& I = P.items[ilo];
            const BandGeom G{I.W, I.H, I.R, I.nbands};
            const PBox bx = P.pbox[p];
            uint32_t bl, bh;
            if (!prim_bands(G, bx, bl, bh)) continue;
            const RPrim& R = P.prims[p];
            double w0 = R.w0, w1 = R.w1, w2 = R.w2;
            int64_t cur = bx.y0;
            const uint32_t jend = min(cnt, j0 + kRowSeg);
            for (uint32_t j = j0; j < jend && bl + j <= bh; j++) {
                const uint32_t b = bl + j;
                int64_t a = (int64_t)b * I.R - floordiv_w(bx.x1, I.W);
                if (a < bx.y0) a = bx.y0;
                const int64_t gap = a - cur;
                if (gap > 0) {
                    w0 = row_advance(w0, R.b0, gap);
                    w1 = row_advance(w1, R.b1, gap);
                    w2 = row_advance(w2, R.b2, gap);
                    cur = a;
                }
                double* o = P.rstart + 3 * (base + j);
                o[0] = w0;
                o[1] = w1;
                o[2] = w2;
            }
        }
        __syncthreads();
    }
}

// Exclusive scan of n uint32 values, 2048 per logical block, single pass.
constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;

__global__ void __launch_bounds__(kScanBlock) scan_u32_kernel(ScanParams P) {
    __shared__ uint32_t s_tile;
    __shared__ OrderedAllocSmem<kScanBlock> s_alloc;
    const uint32_t tile = block_ticket<kScanBlock>(P.lb, &s_tile);
    const uint64_t base = ((uint64_t)tile * kScanBlock + threadIdx.x) * kScanItems;
    const uint64_t n = P.n_dev ? min(P.n, (uint64_t)*P.n_dev) : P.n;
    uint32_t v[kScanItems];
    uint64_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < n) ? P.in[base + k] : 0u;
        sum += v[k];
    }
    uint64_t excl = ordered_alloc<kScanBlock>(P.lb, tile, sum, s_alloc);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) P.out[base + k] = (uint32_t)excl;
        excl += v[k];
    }
}

__global__ void __launch_bounds__(256) bin_scatter_kernel(BinParams P, int warps) {
    extern __shared__ uint32_t cnt[];
    if (*P.pair_total > P.bin_cap) {
        if (threadIdx.x == 0) atomicOr(P.status, ST_BIN_OVERFLOW);
        return;
    }
    const BinBlock B = bin_block(P);
    const uint32_t nb = B.G.nbands;
    const uint64_t lo = B.lo, hi = B.hi;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t sub = (hi - lo + warps - 1) / warps;
    const uint64_t slo = min(lo + (uint64_t)w * sub, hi);
    const uint64_t shi = min(slo + sub, hi);
    uint32_t* mycnt = cnt + (size_t)w * nb;

    for (uint32_t i = threadIdx.x; i < (uint32_t)warps * nb; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    // phase 1: per-warp band counts
    for (uint64_t p = slo + lane; p < shi; p += 32) {
        uint32_t bl, bh;
        if (prim_bands(B.G, P.pbox[p], bl, bh))
            for (uint32_t b = bl; b <= bh; b++) atomicAdd(&mycnt[b], 1u);
    }
    __syncthreads();
    // phase 2: each warp's starting position per band
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
        uint32_t run = P.off[B.mat0 + (uint64_t)b * B.nblk + B.lblk];
        for (int ww = 0; ww < warps; ww++) {
            uint32_t t = cnt[(size_t)ww * nb + b];
            cnt[(size_t)ww * nb + b] = run;
            run += t;
        }
    }
    __syncthreads();
    // phase 3: stable scatter. A round takes the warp's next 32 primitives
    // (lane order = submission order), lays their (primitive, band) pairs out
    // in that order, and places the pairs 32 at a time: within a group, the
    // pairs of one band are ranked by lane with __match_any_sync, after the
    // pairs of that band from earlier groups and rounds (mycnt).
    __shared__ uint32_t s_off[8][33];
    const unsigned lanes_lt = (1u << lane) - 1u;
    for (uint64_t rb = slo; rb < shi; rb += 32) {
        const uint64_t p = rb + lane;
        uint32_t bl = 1, bh = 0;
        bool has = (p < shi) && prim_bands(B.G, P.pbox[p], bl, bh);
        const uint32_t span = has ? (bh - bl + 1) : 0u;
        uint32_t incl = span;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        s_off[w][lane] = incl - span;
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        for (uint32_t q0 = 0; q0 < total; q0 += 32) {
            const uint32_t q = q0 + lane;
            const bool active = q < total;
            // owner: the last lane whose first pair index is <= q
            int lo = 0, hi = 31;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_off[w][mid] <= q) lo = mid;
                else hi = mid - 1;
            }
            const uint32_t obl = __shfl_sync(0xffffffffu, bl, lo);
            const uint32_t b = active ? obl + (q - s_off[w][lo]) : 0xFFFFFFFFu;
            const unsigned peers = __match_any_sync(0xffffffffu, b);
            if (active) P.bins[mycnt[b] + __popc(peers & lanes_lt)] = (uint32_t)(rb + lo);
            __syncwarp();
            if (active && (peers >> lane) == 1u) mycnt[b] += __popc(peers);  // highest lane of the band
            __syncwarp();
        }
    }
}

}  // namespace fgc
