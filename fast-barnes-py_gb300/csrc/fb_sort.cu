// fb_sort.cu -- sample preparation for the splat: value range, bin keys and a
// deterministic ordering of the samples by grid row.
//
// Replaces the per-sample loop head of _inject_data_{1,2,3}d
// (fastbarnes/interpolation.py:218-322: cell index, skip rule) and
// _normalize_values (:204-212: min/max of the values).
//
// Samples are counted per bin (grid row, or (z, y) row, or x range in 1D) by
// atomics whose returned counts give every sample a slot in its bin, the
// counts are scanned into bin starts, every sample is placed into its slot,
// and finally every bin is sorted by sample index, so the order inside a bin
// is the samples' own order whatever the atomics did.
// The splatting kernel then adds each row's samples in that order.
#include <algorithm>

#include "fb_internal.cuh"
#include "fb_kernels.cuh"

namespace fbg {

// Bin key of every sample (single call: nbins for samples the reference
// skips; batched form: the field's extra bin), its cell record, the count of
// every bin, and the min / max / NaN reduction of the values.  The header and the counts start zeroed (min is kept complemented
// for that reason).  The float64 form divides by the step like the reference
// (interpolation.py:247-248); the float32 form multiplies by its reciprocal.
// Block-wide reduction of the value range (order-preserving integer keys)
// and the NaN flag, then one set of atomics per block on the field header.
__device__ __forceinline__ void range_to_header(unsigned long long kmin, unsigned long long kmax, int nan,
                                                FieldHeader *hdr)
{
    __shared__ unsigned long long s_min[32], s_max[32];
    __shared__ int s_nan[32];
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long a = __shfl_xor_sync(0xffffffffu, kmin, o);
        unsigned long long b = __shfl_xor_sync(0xffffffffu, kmax, o);
        kmin = a < kmin ? a : kmin;
        kmax = b > kmax ? b : kmax;
    }
    nan = __any_sync(0xffffffffu, nan);
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_min[w] = kmin;
        s_max[w] = kmax;
        s_nan[w] = nan;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < nw; q++) {
            kmin = s_min[q] < kmin ? s_min[q] : kmin;
            kmax = s_max[q] > kmax ? s_max[q] : kmax;
            nan |= s_nan[q];
        }
        if (kmin != ~0ull)
            atomicMax(&hdr->vmin_key, ~kmin);
        if (kmax != 0ull)
            atomicMax(&hdr->vmax_key, kmax);
        if (nan)
            atomicExch(&hdr->nan_seen, 1);
    }
}

template <int DIM, typename Real>
__global__ void k_bin_keys(const double *__restrict__ pts, const double *__restrict__ val, int64_t npts,
                           Geometry g, int bin_w, uint32_t nbins, uint32_t *__restrict__ keys,
                           SampleRec<Real> *__restrict__ rec, uint32_t *__restrict__ counts,
                           uint32_t *__restrict__ rank, FieldHeader *hdr)
{
    // float64 instructions kept to the cell coordinates, as in k_batch_keys
    constexpr bool EXACT = sizeof(Real) == 8;
    __shared__ double s_inv[3];
    if (threadIdx.x < 3)
        s_inv[threadIdx.x] = 1.0 / g.step[threadIdx.x];
    __syncthreads();
    unsigned long long kmin = ~0ull, kmax = 0ull;
    int nan = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npts;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double v = val[k];
        const unsigned long long vb = (unsigned long long)__double_as_longlong(v);
        if ((vb & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) {
            nan = 1;
        } else {
            unsigned long long o = dbl_to_ordered(v);
            kmin = o < kmin ? o : kmin;
            kmax = o > kmax ? o : kmax;
        }
        uint32_t key = nbins;
        const double *p = pts + k * DIM;
        double c[3] = {0.0, 0.0, 0.0};
        int ci[3] = {0, 0, 0};
        bool skip = false;
        Real cw[3] = {0, 0, 0};
#pragma unroll
        for (int m = 0; m < DIM; m++) {
            if (EXACT) {
                c[m] = (p[m] - g.x0[m]) / g.step[m];
                ci[m] = __double2int_rz(c[m]);
                skip = skip || !(c[m] >= 0.0);
                cw[m] = (Real)(c[m] - (double)ci[m]);
            } else {
                float f;
                skip = skip || !split_cell_edge(p[m] - g.x0[m], g.step[m], s_inv[m], g.size[m], ci[m], f);
                cw[m] = (Real)f;
            }
            skip = skip || (int64_t)ci[m] >= g.size[m] - 1;
        }
        SampleRec<Real> r;
        r.xi = r.yi = r.zi = 0;
        r.xw = r.yw = r.zw = 0;
        if (!skip) {
            r.xi = ci[0];
            r.yi = ci[1];
            r.zi = ci[2];
            r.xw = cw[0];
            r.yw = cw[1];
            r.zw = cw[2];
            if (DIM == 1)
                key = (uint32_t)(ci[0] / bin_w);
            else if (DIM == 2)
                key = (uint32_t)ci[1];
            else
                key = (uint32_t)((int64_t)ci[2] * g.size[1] + ci[1]);
        }
        r.val = v;
        rec[k] = r;
        keys[k] = key;
        if (key < nbins)
            rank[k] = atomicAdd(&counts[key], 1u);   // the sample's slot in its bin (any order)
    }
    range_to_header(kmin, kmax, nan, hdr);
}

// Exclusive prefix sum of n entries, one block of 1024 threads walking tiles
// of 4096 entries.
__global__ void __launch_bounds__(1024) k_scan_exclusive(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                                                         int64_t n)
{
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry_s;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    uint32_t carry = 0;
    for (int64_t base = 0; base < n; base += 4096) {
        uint32_t x[4];
        uint32_t s = 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t i = base + 4 * t + u;
            x[u] = i < n ? in[i] : 0u;
            s += x[u];
        }
        // inclusive scan of the thread sums
        uint32_t inc = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o)
                inc += y;
        }
        if (lane == 31)
            wsum[w] = inc;
        __syncthreads();
        if (w == 0) {
            uint32_t ws = wsum[lane];
            uint32_t wi = ws;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o)
                    wi += y;
            }
            wsum[lane] = wi - ws;   // exclusive warp offsets
            if (lane == 31)
                carry_s = wi;
        }
        __syncthreads();
        uint32_t run = carry + wsum[w] + inc - s;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t i = base + 4 * t + u;
            if (i < n)
                out[i] = run;
            run += x[u];
        }
        carry += carry_s;
        __syncthreads();
    }
}

// Places every sample into the slot of its bin that the key kernel drew; the
// order inside a bin is fixed later.  Four samples a thread, their loads
// issued together (keys and slots, then the bin starts), so that a thread
// waits on two round trips for all four.
constexpr int kScatterPerThread = 4;
__global__ void k_bin_scatter(const uint32_t *__restrict__ keys, int64_t npts, uint32_t nbins,
                              const uint32_t *__restrict__ start, const uint32_t *__restrict__ rank,
                              uint32_t *__restrict__ sorted, uint32_t *status)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k0 < npts; k0 += kScatterPerThread * stride) {
        uint32_t key[kScatterPerThread], rk[kScatterPerThread], st[kScatterPerThread], nx[kScatterPerThread];
#pragma unroll
        for (int u = 0; u < kScatterPerThread; u++) {
            const int64_t k = k0 + u * stride;
            key[u] = k < npts ? keys[k] : nbins;
            rk[u] = key[u] < nbins ? rank[k] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kScatterPerThread; u++) {
            st[u] = key[u] < nbins ? start[key[u]] : 0u;
            // bounds-check build: the bin's end
            nx[u] = kBoundsCheck && key[u] < nbins ? start[key[u] + 1] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kScatterPerThread; u++) {
            if (key[u] < nbins) {
                const uint32_t pos = st[u] + rk[u];
                if (bounds_ok(!kBoundsCheck || pos < nx[u], status))
                    sorted[pos] = (uint32_t)(k0 + u * stride);
            }
        }
    }
}

constexpr int kWarpSortMax = 1024;   // bins up to this size are sorted by one warp
constexpr int kBinSortWarps = 8;

struct WarpSync {
    __device__ void operator()() const { __syncwarp(); }
};
struct BlockSync {
    __device__ void operator()() const { __syncthreads(); }
};

// Bitonic compare-exchange network over n (a power of two) keys in shared
// memory, threads [0, nthr) cooperating; `sync` orders the steps.
template <typename Sync>
__device__ __forceinline__ void bitonic(uint32_t *s, int n, int t, int nthr, Sync sync)
{
    for (int k = 2; k <= n; k <<= 1) {
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int i = t; i < n / 2; i += nthr) {
                const int lo = ((i & ~(jj - 1)) << 1) | (i & (jj - 1));
                const int hi = lo + jj;
                const bool asc = (lo & k) == 0;
                const uint32_t a = s[lo], b = s[hi];
                if ((a > b) == asc) {
                    s[lo] = b;
                    s[hi] = a;
                }
            }
            sync();
        }
    }
}

// Copies sample record `k` (RW 16-byte words) to position `i` of the sorted
// record array.
__device__ __forceinline__ void copy_rec(const uint4 *__restrict__ rec, uint4 *__restrict__ srec, int rw, uint32_t k,
                                         uint32_t i)
{
    for (int w = 0; w < rw; w++)
        srec[(size_t)i * rw + w] = rec[(size_t)k * rw + w];
}

// Two record copies (the second when `two`), every load issued before the
// first store (records of at most three words), so that the lane waits on
// one round trip, not two.
__device__ __forceinline__ void copy_rec2(const uint4 *__restrict__ rec, uint4 *__restrict__ srec, int rw, uint32_t k0,
                                          uint32_t i0, bool one, uint32_t k1, uint32_t i1, bool two)
{
    uint4 a[3], b[3];
#pragma unroll
    for (int w = 0; w < 3; w++) {
        if (one && w < rw)
            a[w] = rec[(size_t)k0 * rw + w];
        if (two && w < rw)
            b[w] = rec[(size_t)k1 * rw + w];
    }
#pragma unroll
    for (int w = 0; w < 3; w++) {
        if (one && w < rw)
            srec[(size_t)i0 * rw + w] = a[w];
        if (two && w < rw)
            srec[(size_t)i1 * rw + w] = b[w];
    }
}

// Sorts one bin's entries by sample index with one warp: in registers for up
// to 64 entries, in shared memory (`buf`, kWarpSortMax entries) up to
// kWarpSortMax; returns false, leaving a larger bin to the whole block.  The
// bin's sample records are copied into sorted order (rw 16-byte words a
// record).
__device__ __forceinline__ bool sort_one_bin(const uint32_t *__restrict__ start, int64_t b,
                                             uint32_t *__restrict__ sorted, const uint4 *__restrict__ rec,
                                             uint4 *__restrict__ srec, int rw, uint32_t *buf, int lane)
{
    const uint32_t s0 = start[b], c = start[b + 1] - s0;
    if (c == 0)
        return true;
    if (c <= 32) {
        uint32_t x = lane < (int)c ? sorted[s0 + lane] : 0xFFFFFFFFu;
        for (int k = 2; k <= 32; k <<= 1) {
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
                const uint32_t y = __shfl_xor_sync(0xffffffffu, x, jj);
                const bool asc = (lane & k) == 0;
                const bool lower = (lane & jj) == 0;
                x = (lower == asc) ? min(x, y) : max(x, y);
            }
        }
        if (lane < (int)c) {
            sorted[s0 + lane] = x;
            copy_rec(rec, srec, rw, x, s0 + lane);
        }
        return true;
    }
    if (c <= 64) {
        // two keys a lane (elements lane and lane + 32), bitonic network in
        // registers: partners 32 apart sit in the same lane, the others are
        // a shuffle away
        uint32_t x0 = lane < (int)c ? sorted[s0 + lane] : 0xFFFFFFFFu;
        uint32_t x1 = lane + 32 < (int)c ? sorted[s0 + lane + 32] : 0xFFFFFFFFu;
        for (int k = 2; k <= 64; k <<= 1) {
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
                if (jj == 32) {   // k = 64: ascending everywhere
                    const uint32_t lo = min(x0, x1), hi = max(x0, x1);
                    x0 = lo;
                    x1 = hi;
                } else {
                    const uint32_t y0 = __shfl_xor_sync(0xffffffffu, x0, jj);
                    const uint32_t y1 = __shfl_xor_sync(0xffffffffu, x1, jj);
                    const bool lower = (lane & jj) == 0;
                    const bool asc0 = (lane & k) == 0, asc1 = ((lane + 32) & k) == 0;
                    x0 = (lower == asc0) ? min(x0, y0) : max(x0, y0);
                    x1 = (lower == asc1) ? min(x1, y1) : max(x1, y1);
                }
            }
        }
        const bool one = lane < (int)c, two = lane + 32 < (int)c;
        if (one)
            sorted[s0 + lane] = x0;
        if (two)
            sorted[s0 + lane + 32] = x1;
        copy_rec2(rec, srec, rw, x0, s0 + lane, one, x1, s0 + lane + 32, two);
        return true;
    }
    if (c <= kWarpSortMax) {
        int n = 128;
        while (n < (int)c)
            n <<= 1;
        for (int i = lane; i < n; i += 32)
            buf[i] = i < (int)c ? sorted[s0 + i] : 0xFFFFFFFFu;
        __syncwarp();
        bitonic(buf, n, lane, 32, WarpSync());
        for (int i = lane; i < (int)c; i += 32) {
            sorted[s0 + i] = buf[i];
            copy_rec(rec, srec, rw, buf[i], s0 + i);
        }
        return true;
    }
    return false;
}

// Sorts one bin too large for a warp with the whole block: in shared memory
// (`sbuf`, cap entries) when it fits, else in a global scratch area of twice
// the bin size (padded to a power of two with keys that sort last); copies
// its records into sorted order.  Not inlined: the rare path keeps its
// registers out of the common one's (inlined, the bin sort spilled).
__device__ __noinline__ void sort_large_bin(const uint32_t *__restrict__ start, int64_t b, uint32_t *__restrict__ sorted,
                               uint32_t *__restrict__ scratch, const uint4 *__restrict__ rec,
                               uint4 *__restrict__ srec, int rw, uint32_t *sbuf, int cap)
{
    const uint32_t s0 = start[b], c = start[b + 1] - s0;
    int n = 1;
    while (n < (int)c)
        n <<= 1;
    uint32_t *sc = n <= cap ? sbuf : scratch + 2 * (size_t)s0;   // 2c >= n cells of this bin's own region
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        sc[i] = i < (int)c ? sorted[s0 + i] : 0xFFFFFFFFu;
    __syncthreads();
    bitonic(sc, n, threadIdx.x, (int)blockDim.x, BlockSync());
    for (int i = threadIdx.x; i < (int)c; i += blockDim.x) {
        sorted[s0 + i] = sc[i];
        copy_rec(rec, srec, rw, sc[i], s0 + i);
    }
    __syncthreads();
}

// Bitonic network over the 64 entries of each of two bins held by one warp
// (x[q][0]: entry lane of bin q, x[q][1]: entry lane + 32): partners 32 apart
// sit in the same lane, the others a shuffle away; the two bins' steps are
// independent, so their shuffles overlap.
__device__ __forceinline__ void bitonic64_pair(uint32_t (&x)[2][2], int lane)
{
#pragma unroll
    for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            if (jj == 32) {   // k = 64: ascending everywhere
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const uint32_t lo = min(x[q][0], x[q][1]), hi = max(x[q][0], x[q][1]);
                    x[q][0] = lo;
                    x[q][1] = hi;
                }
            } else {
                const bool lower = (lane & jj) == 0;
                const bool asc0 = (lane & k) == 0, asc1 = ((lane + 32) & k) == 0;
                uint32_t y[2][2];
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    y[q][0] = __shfl_xor_sync(0xffffffffu, x[q][0], jj);
                    y[q][1] = __shfl_xor_sync(0xffffffffu, x[q][1], jj);
                }
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    x[q][0] = (lower == asc0) ? min(x[q][0], y[q][0]) : max(x[q][0], y[q][0]);
                    x[q][1] = (lower == asc1) ? min(x[q][1], y[q][1]) : max(x[q][1], y[q][1]);
                }
            }
        }
    }
}

// Sorts every bin's entries by sample index, so each bin lists its samples
// in sample order whatever order the count atomics produced, and copies the
// records (RW 16-byte words each) into that order.  Each warp takes two
// adjacent bins: their starts, entries and records are each fetched with
// one round of loads for both, and bins of up to 64 entries are sorted in
// registers by two interleaved bitonic networks.  A larger bin goes through
// sort_one_bin (shared memory, up to kWarpSortMax) or, beyond that, the whole
// block (sort_large_bin), so one launch covers every bin size.
template <int RW>
__global__ void __launch_bounds__(32 * kBinSortWarps) k_sort_bins(const uint32_t *__restrict__ start, uint32_t nbins,
                                                                  uint32_t *__restrict__ sorted,
                                                                  const uint4 *__restrict__ rec,
                                                                  uint4 *__restrict__ srec,
                                                                  uint32_t *__restrict__ scratch, uint32_t *status)
{
    __shared__ uint32_t buf[kBinSortWarps][kWarpSortMax];
    __shared__ int s_big[kBinSortWarps][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t b0 = ((int64_t)blockIdx.x * kBinSortWarps + w) * 2;   // bins b0, b0 + 1
    const int nb = (int)max((int64_t)0, min((int64_t)2, (int64_t)nbins - b0));
    // starts of both bins and the end of the second: lanes 0 .. nb
    const uint32_t st = lane <= nb ? start[b0 + lane] : 0u;
    const uint32_t sa = __shfl_sync(0xffffffffu, st, 0), sb = __shfl_sync(0xffffffffu, st, 1),
                   sc = __shfl_sync(0xffffffffu, st, 2);
    // bounds-check build: each bin inside the sorted arrays
    const bool ok0 = nb < 1 || bounds_ok(!kBoundsCheck || (sa <= sb && sb <= start[nbins]), status);
    const bool ok1 = nb < 2 || bounds_ok(!kBoundsCheck || (sb <= sc && sc <= start[nbins]), status);
    const uint32_t s0[2] = {sa, sb};
    const int c[2] = {nb >= 1 && ok0 ? (int)(sb - sa) : 0, nb >= 2 && ok1 ? (int)(sc - sb) : 0};
    int big[2] = {0, 0};
    if (c[0] <= 64 && c[1] <= 64) {
        uint32_t x[2][2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            x[q][0] = lane < c[q] ? sorted[s0[q] + lane] : 0xFFFFFFFFu;
            x[q][1] = lane + 32 < c[q] ? sorted[s0[q] + lane + 32] : 0xFFFFFFFFu;
        }
        if (c[0] > 1 || c[1] > 1)
            bitonic64_pair(x, lane);
        // the records of all (up to four) entries of this lane in flight together
        uint4 v[2][2][RW];
#pragma unroll
        for (int q = 0; q < 2; q++)
#pragma unroll
            for (int h = 0; h < 2; h++)
                if (lane + 32 * h < c[q])
#pragma unroll
                    for (int u = 0; u < RW; u++)
                        v[q][h][u] = rec[(size_t)x[q][h] * RW + u];
#pragma unroll
        for (int q = 0; q < 2; q++)
#pragma unroll
            for (int h = 0; h < 2; h++)
                if (lane + 32 * h < c[q]) {
                    const uint32_t pos = s0[q] + lane + 32 * h;
                    sorted[pos] = x[q][h];
#pragma unroll
                    for (int u = 0; u < RW; u++)
                        srec[(size_t)pos * RW + u] = v[q][h][u];
                }
    } else {
        const bool okq[2] = {ok0, ok1};
#pragma unroll
        for (int q = 0; q < 2; q++)
            if (q < nb && okq[q])
                big[q] = sort_one_bin(start, b0 + q, sorted, rec, srec, RW, buf[w], lane) ? 0 : 1;
    }
    if (lane == 0) {
        s_big[w][0] = big[0];
        s_big[w][1] = big[1];
    }
    __syncthreads();
    for (int q = 0; q < kBinSortWarps; q++)
        for (int h = 0; h < 2; h++)
            if (s_big[q][h])
                sort_large_bin(start, ((int64_t)blockIdx.x * kBinSortWarps + q) * 2 + h, sorted, scratch, rec, srec,
                               RW, &buf[0][0], kBinSortWarps * kWarpSortMax);
}

// Launches k_sort_bins for records of rw 16-byte words (2: float32 form, 3:
// float64 form).
cudaError_t launch_sort_bins(const uint32_t *start, uint32_t nbins, uint32_t *sorted, const uint4 *rec, uint4 *srec,
                             int rw, uint32_t *scratch, uint32_t *status, cudaStream_t st)
{
    const unsigned grid = (unsigned)((nbins + 2 * kBinSortWarps - 1) / (2 * kBinSortWarps));
    if (grid == 0)
        return cudaSuccess;
    if (rw == 2)
        k_sort_bins<2><<<grid, 32 * kBinSortWarps, 0, st>>>(start, nbins, sorted, rec, srec, scratch, status);
    else if (rw == 3)
        k_sort_bins<3><<<grid, 32 * kBinSortWarps, 0, st>>>(start, nbins, sorted, rec, srec, scratch, status);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// batched form: the samples of many 2D fields in one set of launches
// ---------------------------------------------------------------------------

// Exclusive scan of counts[0, n) into bin_start (base + the scan) by one
// block of 256 threads (the last block of a field in the key pass), which
// also clears the counts for the next run.  Tiles of 2048 entries, 8
// consecutive ones a thread (two 16-byte loads, the next tile's issued
// before the current tile is scanned): a thread sums its own entries
// serially, so a tile costs one warp scan and three barriers.  The counts
// were built by device-scope atomics: read from L2 (plain loads, as counts
// need not be 16-byte aligned here).
__device__ void last_block_scan(uint32_t *__restrict__ counts, uint32_t *__restrict__ bin_start, int64_t n,
                                uint32_t base0)
{
    constexpr int E = 8, TILE = 256 * E;
    __shared__ uint32_t s_w[8];
    __shared__ uint32_t s_tot;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int64_t ntile = (n + TILE - 1) / TILE;
    uint32_t cur[E], nxt[E];
    auto load = [&](int64_t tile, uint32_t (&v)[E]) {
#pragma unroll
        for (int u = 0; u < E; u++) {
            const int64_t i = tile * TILE + (int64_t)E * t + u;
            v[u] = i < n ? __ldcg(counts + i) : 0u;
        }
    };
    uint32_t carry = base0;
    load(0, cur);
    for (int64_t tile = 0; tile < ntile; tile++) {
        if (tile + 1 < ntile)
            load(tile + 1, nxt);
        const int64_t base = tile * TILE + (int64_t)E * t;
        uint32_t x[E];
        uint32_t sum = 0;
#pragma unroll
        for (int i = 0; i < E; i++) {
            x[i] = cur[i];
            sum += x[i];
        }
        uint32_t inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o)
                inc += y;
        }
        if (lane == 31)
            s_w[w] = inc;
        __syncthreads();
        if (w == 0) {
            const uint32_t v = lane < 8 ? s_w[lane] : 0u;
            uint32_t vi = v;
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, vi, o);
                if (lane >= o)
                    vi += y;
            }
            if (lane < 8)
                s_w[lane] = vi - v;
            if (lane == 7)
                s_tot = vi;
        }
        __syncthreads();
        uint32_t run = carry + s_w[w] + inc - sum;
#pragma unroll
        for (int i = 0; i < E; i++) {
            if (base + i < n)
                bin_start[base + i] = run;
            run += x[i];
        }
#pragma unroll
        for (int i = 0; i < E; i++)
            if (base + i < n)
                counts[base + i] = 0u;
        carry += s_tot;
        __syncthreads();   // s_w / s_tot are rewritten by the next tile
#pragma unroll
        for (int u = 0; u < E; u++)
            cur[u] = nxt[u];
    }
}

// Bin keys and records of one block of one field's samples (256 threads,
// kBatchKeysPerBlock / 256 samples each, taken two at a time with the next
// two's loads issued before the current two are worked on, so that the grid
// is about one wave and every thread has loads in flight); keys are global
// bins: the field's bin offset + row, or + H (the field's last bin, which
// takes the samples the reference skips), so that the bins of a field cover
// its own samples exactly and its bin starts are field-local: the last block
// of each field to finish (a per-field ticket) scans that field's counts
// into its bin starts (base: the field's first global sample) and clears
// them and the ticket for the next run.  The fields' scans run side by side.
// Records are indexed by global sample.
template <typename Real>
__global__ void __launch_bounds__(256, 3) k_batch_keys(const BatchKeyField *__restrict__ fields,
                                                    const uint2 *__restrict__ blocks,
                                                    uint32_t *__restrict__ keys, SampleRec<Real> *__restrict__ rec,
                                                    uint32_t *__restrict__ counts, uint32_t *__restrict__ rank,
                                                    FieldHeader *__restrict__ hdrs, uint32_t *__restrict__ tickets,
                                                    uint32_t *__restrict__ bin_start)
{
    constexpr int PAIRS = kBatchKeysPerBlock / 512;
    static_assert(kBatchKeysPerBlock % 512 == 0, "pairs of samples per thread of 256");
    // Float64 instructions are few per SM on this part, so the loop keeps
    // them to the cell coordinates: the NaN test works on the bits, the
    // upper bound of the skip rule on the truncated cell index (trunc = floor
    // for xc >= 0, and xc >= size - 1 <=> floor(xc) >= size - 1; the
    // conversion saturates), and the float32 form multiplies by 1 / step.
    // NaN coordinates are skipped.
    constexpr bool EXACT = sizeof(Real) == 8;
    const uint2 bt = blocks[blockIdx.x];   // (field, first sample of the block within the field)
    const BatchKeyField f = fields[bt.x];
    unsigned long long kmin = ~0ull, kmax = 0ull;
    int nan = 0;
    const int64_t end = min(f.npts, (int64_t)bt.y + kBatchKeysPerBlock);
    // sample u of pair p: bt.y + p * 512 + u * 256 + threadIdx.x
    double v[2][2], px[2][2], py[2][2];
    auto load = [&](int p, int buf) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int64_t k = (int64_t)bt.y + p * 512 + u * 256 + threadIdx.x;
            if (k < end) {
                v[buf][u] = f.val[k];
                px[buf][u] = f.pts[2 * k];
                py[buf][u] = f.pts[2 * k + 1];
            }
        }
    };
    // slots drawn by the count atomics, stored after the loop: a store
    // right after its atomic would hold the thread on the atomic's round trip
    uint32_t slot[PAIRS][2];
    load(0, 0);
#pragma unroll
    for (int p = 0; p < PAIRS; p++) {
        const int cb = p & 1;
        if (p + 1 < PAIRS)
            load(p + 1, cb ^ 1);
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int64_t k = (int64_t)bt.y + p * 512 + u * 256 + threadIdx.x;
            if (k >= end)
                continue;
            const double vu = v[cb][u];
            const unsigned long long vb = (unsigned long long)__double_as_longlong(vu);
            if ((vb & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) {
                nan = 1;
            } else {
                unsigned long long o = dbl_to_ordered(vu);
                kmin = o < kmin ? o : kmin;
                kmax = o > kmax ? o : kmax;
            }
            int xi, yi;
            Real xw, yw;
            bool skip;
            if (EXACT) {
                const double xc = (px[cb][u] - f.x0[0]) / f.step[0], yc = (py[cb][u] - f.x0[1]) / f.step[1];
                xi = __double2int_rz(xc);
                yi = __double2int_rz(yc);
                skip = !(xc >= 0.0) || !(yc >= 0.0);
                xw = (Real)(xc - (double)xi);
                yw = (Real)(yc - (double)yi);
            } else {
                float xf, yf;
                skip = !split_cell_edge(px[cb][u] - f.x0[0], f.step[0], f.inv_step[0], f.size[0], xi, xf) ||
                       !split_cell_edge(py[cb][u] - f.x0[1], f.step[1], f.inv_step[1], f.size[1], yi, yf);
                xw = (Real)xf;
                yw = (Real)yf;
            }
            skip = skip || (int64_t)xi >= f.size[0] - 1 || (int64_t)yi >= f.size[1] - 1;
            SampleRec<Real> r;
            r.xi = r.yi = r.zi = 0;
            r.xw = r.yw = r.zw = 0;
            uint32_t key = f.bin_offset + (uint32_t)f.size[1];   // the field's bin of skipped samples
            if (!skip) {
                r.xi = xi;
                r.yi = yi;
                r.xw = xw;
                r.yw = yw;
                key = f.bin_offset + (uint32_t)yi;
            }
            r.val = vu;
            const int64_t gk = f.sample_offset + k;
            rec[gk] = r;
            keys[gk] = key;
            slot[p][u] = atomicAdd(&counts[key], 1u);   // the sample's slot in its bin (any order)
        }
    }
#pragma unroll
    for (int p = 0; p < PAIRS; p++)
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int64_t k = (int64_t)bt.y + p * 512 + u * 256 + threadIdx.x;
            if (k < end)
                rank[f.sample_offset + k] = slot[p][u];
        }
    range_to_header(kmin, kmax, nan, hdrs + bt.x);
    // The block's writes are ordered before the ticket by the barrier and
    // one release fence of the thread that takes the ticket.
    __shared__ bool s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t nblk = (uint32_t)((f.npts + kBatchKeysPerBlock - 1) / kBatchKeysPerBlock);
        __threadfence();
        s_last = atomicAdd(&tickets[bt.x], 1u) == nblk - 1;
    }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
    // bins of the field: rows 0 .. H - 1 and the skipped samples' bin H; the
    // entry after them (the next field's first) is the end of the field
    const int64_t nb = f.size[1] + 1;
    last_block_scan(counts + f.bin_offset, bin_start + f.bin_offset, nb, (uint32_t)f.sample_offset);
    if (threadIdx.x == 0) {
        bin_start[f.bin_offset + nb] = (uint32_t)(f.sample_offset + f.npts);
        tickets[bt.x] = 0u;
    }
}

// Scratch layout: counts[nbins + 2] | cursor[nbins + 2] (batched form: the
// key pass's per-field tickets) | large[nbins + 2] (spare) |
// keys[N] | sorted[N] | big-bin scratch[2N] (uint32; its first N entries hold
// the samples' slots in their bins until the scatter), then the sample records
// by sample index and the records in sorted order.
namespace {
struct SortLayout {
    uint32_t *counts, *cursor, *large, *keys, *sorted, *big;
    char *rec, *srec;
    size_t bytes;   // through the sorted records
};

size_t rec_bytes(int precision) { return precision == 0 ? sizeof(SampleRec<double>) : sizeof(SampleRec<float>); }
static_assert(sizeof(SampleRec<double>) % 16 == 0 && sizeof(SampleRec<float>) % 16 == 0,
              "records are copied as 16-byte words");
size_t up256(size_t x) { return (x + 255) / 256 * 256; }

// Byte offsets of the record arrays and of the end of the sorted records.
void sort_offsets(int64_t n, uint32_t nbins, int precision, size_t &rec, size_t &srec, size_t &end)
{
    const size_t nb = (size_t)nbins + 2;
    rec = up256(4 * (3 * nb + 4 * (size_t)n));
    srec = rec + up256(rec_bytes(precision) * (size_t)n);
    end = srec + up256(rec_bytes(precision) * (size_t)n);
}

SortLayout sort_layout(uint32_t *scratch, int64_t n, uint32_t nbins, int precision)
{
    SortLayout l;
    const size_t nb = (size_t)nbins + 2;
    l.counts = scratch;
    l.cursor = l.counts + nb;
    l.large = l.cursor + nb;
    l.keys = l.large + nb;
    l.sorted = l.keys + n;
    l.big = l.sorted + n;
    size_t rec, srec, end;
    sort_offsets(n, nbins, precision, rec, srec, end);
    char *base = reinterpret_cast<char *>(scratch);
    l.rec = base + rec;
    l.srec = base + srec;
    l.bytes = end;
    return l;
}
}  // namespace

size_t sort_scratch_bytes(int64_t npts, uint32_t nbins, int precision)
{
    size_t rec, srec, end;
    sort_offsets(npts, nbins, precision, rec, srec, end);
    return end + 256;
}

size_t batch_sort_scratch_bytes(int64_t ntot, uint32_t nbins, int precision)
{
    size_t rec, srec, end;
    sort_offsets(ntot, nbins, precision, rec, srec, end);
    return end + 256;
}

void sort_sample_arrays(int precision, int64_t npts, uint32_t nbins, uint32_t *scratch, const uint32_t **keys,
                        const void **rec)
{
    const SortLayout l = sort_layout(scratch, npts, nbins, precision);
    *keys = l.keys;
    *rec = l.rec;
}

void batch_sort_views(int precision, int64_t ntot, uint32_t nbins, uint32_t *scratch, const uint32_t **sorted_idx,
                      const void **recs)
{
    const SortLayout l = sort_layout(scratch, ntot, nbins, precision);
    *sorted_idx = l.sorted;
    *recs = l.srec;
}


cudaError_t batch_sort(int precision, const BatchKeyField *d_fields, const uint2 *d_blocks, uint32_t nblocks,
                       int64_t ntot, uint32_t nbins, FieldHeader *hdrs, int nfields, uint32_t *scratch,
                       uint32_t *bin_start, const uint32_t **sorted_idx, const void **recs, cudaStream_t st)
{
    // keys, with every field's bin starts scanned by its last block; the bin
    // counts and the per-field tickets stay zero between runs (the key pass
    // clears them; the plan clears them once at creation, and writes the bin
    // starts of fields without samples, which no run touches)
    const SortLayout l = sort_layout(scratch, ntot, nbins, precision);
    cudaError_t e = cudaMemsetAsync(hdrs, 0, sizeof(FieldHeader) * (size_t)nfields, st);
    if (e != cudaSuccess)
        return e;
    *sorted_idx = l.sorted;
    *recs = l.srec;
    if (nblocks > 0) {
        uint32_t *tickets = l.cursor;
        if (precision == 0)
            k_batch_keys<double><<<nblocks, 256, 0, st>>>(d_fields, d_blocks, l.keys,
                                                          reinterpret_cast<SampleRec<double> *>(l.rec), l.counts,
                                                          l.big, hdrs, tickets, bin_start);
        else
            k_batch_keys<float><<<nblocks, 256, 0, st>>>(d_fields, d_blocks, l.keys,
                                                         reinterpret_cast<SampleRec<float> *>(l.rec), l.counts, l.big,
                                                         hdrs, tickets, bin_start);
    }
    if (ntot > 0) {
        uint32_t *status = reinterpret_cast<uint32_t *>(&hdrs->error);
        int blocks = (int)std::min<int64_t>((ntot + 256 * kScatterPerThread - 1) / (256 * kScatterPerThread),
                                            (int64_t)1 << 22);
        k_bin_scatter<<<blocks, 256, 0, st>>>(l.keys, ntot, nbins, bin_start, l.big, l.sorted, status);
        const int rw = (int)(rec_bytes(precision) / 16);
        const uint4 *rec4 = reinterpret_cast<const uint4 *>(l.rec);
        uint4 *srec4 = reinterpret_cast<uint4 *>(l.srec);
        e = launch_sort_bins(bin_start, nbins, l.sorted, rec4, srec4, rw, l.big, status, st);
        if (e != cudaSuccess)
            return e;
    }
    return cudaGetLastError();
}

cudaError_t sort_samples(int precision, const double *pts, const double *val, int64_t npts, const Geometry &g,
                         int bin_w, uint32_t nbins, FieldHeader *hdr, uint32_t *scratch, uint32_t *bin_start,
                         const uint32_t **sorted_idx, const void **recs, cudaStream_t st)
{
    const SortLayout l = sort_layout(scratch, npts, nbins, precision);
    cudaError_t e = cudaMemsetAsync(hdr, 0, sizeof(FieldHeader), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(l.counts, 0, sizeof(uint32_t) * 3 * ((size_t)nbins + 2), st);
    if (e != cudaSuccess)
        return e;
    *sorted_idx = l.sorted;
    *recs = l.srec;
    if (npts > 0) {
        int blocks = (int)std::min<int64_t>((npts + 255) / 256, (int64_t)1 << 22);
#define FBG_KEYS(D, R)                                                                                            \
    k_bin_keys<D, R><<<blocks, 256, 0, st>>>(pts, val, npts, g, bin_w, nbins, l.keys,                              \
                                             reinterpret_cast<SampleRec<R> *>(l.rec), l.counts, l.big, hdr)
        if (precision == 0) {
            if (g.dim == 1)
                FBG_KEYS(1, double);
            else if (g.dim == 2)
                FBG_KEYS(2, double);
            else
                FBG_KEYS(3, double);
        } else {
            if (g.dim == 1)
                FBG_KEYS(1, float);
            else if (g.dim == 2)
                FBG_KEYS(2, float);
            else
                FBG_KEYS(3, float);
        }
#undef FBG_KEYS
    }
    k_scan_exclusive<<<1, 1024, 0, st>>>(l.counts, bin_start, (int64_t)nbins + 1);
    if (npts > 0) {
        int blocks = (int)std::min<int64_t>((npts + 256 * kScatterPerThread - 1) / (256 * kScatterPerThread),
                                            (int64_t)1 << 22);
        k_bin_scatter<<<blocks, 256, 0, st>>>(l.keys, npts, nbins, bin_start, l.big, l.sorted,
                                              reinterpret_cast<uint32_t *>(&hdr->error));
        const int rw = (int)(rec_bytes(precision) / 16);
        const uint4 *rec4 = reinterpret_cast<const uint4 *>(l.rec);
        uint4 *srec4 = reinterpret_cast<uint4 *>(l.srec);
        e = launch_sort_bins(bin_start, nbins, l.sorted, rec4, srec4, rw, l.big,
                             reinterpret_cast<uint32_t *>(&hdr->error), st);
        if (e != cudaSuccess)
            return e;
    }
    return cudaGetLastError();
}

}  // namespace fbg
