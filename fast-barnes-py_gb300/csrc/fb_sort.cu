// fb_sort.cu -- sample preparation for the splat: value range, bin keys and a
// deterministic ordering of the samples by grid row.
//
// Replaces the per-sample loop head of _inject_data_{1,2,3}d
// (fastbarnes/interpolation.py:218-322: cell index, skip rule) and
// _normalize_values (:204-212: min/max of the values).
//
// Samples are counted per bin (grid row, or (z, y) row, or x range in 1D),
// the counts are scanned into bin starts, every sample is placed into its bin
// with an atomic cursor, and finally every bin is sorted by sample index, so
// the order inside a bin is the samples' own order whatever the atomics did.
// The splatting kernel then adds each row's samples in that order.
#include <algorithm>

#include "fb_internal.cuh"
#include "fb_kernels.cuh"

namespace fbg {

// Bin key of every sample (nbins for samples the reference skips), its cell
// record, the count of every bin, and the min / max / NaN reduction of the
// values.  The header and the counts start zeroed (min is kept complemented
// for that reason).  The float64 form divides by the step like the reference
// (interpolation.py:247-248); the float32 form multiplies by its reciprocal.
template <int DIM, typename Real>
__global__ void k_bin_keys(const double *__restrict__ pts, const double *__restrict__ val, int64_t npts,
                           Geometry g, int bin_w, uint32_t nbins, uint32_t *__restrict__ keys,
                           SampleRec<Real> *__restrict__ rec, uint32_t *__restrict__ counts, FieldHeader *hdr)
{
    constexpr bool EXACT = sizeof(Real) == 8;
    const double inv0 = 1.0 / g.step[0], inv1 = 1.0 / g.step[1], inv2 = 1.0 / g.step[2];
    unsigned long long kmin = ~0ull, kmax = 0ull;
    int nan = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npts;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double v = val[k];
        if (isnan(v)) {
            nan = 1;
        } else {
            unsigned long long o = dbl_to_ordered(v);
            kmin = o < kmin ? o : kmin;
            kmax = o > kmax ? o : kmax;
        }
        uint32_t key = nbins;
        const double *p = pts + k * DIM;
        const double xc = EXACT ? (p[0] - g.x0[0]) / g.step[0] : (p[0] - g.x0[0]) * inv0;
        double yc = 0.0, zc = 0.0;
        bool skip = xc < 0.0 || xc >= (double)(g.size[0] - 1);
        if (DIM >= 2) {
            yc = EXACT ? (p[1] - g.x0[1]) / g.step[1] : (p[1] - g.x0[1]) * inv1;
            skip = skip || yc < 0.0 || yc >= (double)(g.size[1] - 1);
        }
        if (DIM == 3) {
            zc = EXACT ? (p[2] - g.x0[2]) / g.step[2] : (p[2] - g.x0[2]) * inv2;
            skip = skip || zc < 0.0 || zc >= (double)(g.size[2] - 1);
        }
        SampleRec<Real> r;
        r.xi = r.yi = r.zi = 0;
        r.xw = r.yw = r.zw = 0;
        if (!skip) {
            const int64_t xi = (int64_t)xc, yi = (int64_t)yc, zi = (int64_t)zc;
            r.xi = (int32_t)xi;
            r.yi = (int32_t)yi;
            r.zi = (int32_t)zi;
            r.xw = (Real)(xc - (double)xi);
            r.yw = (Real)(yc - (double)yi);
            r.zw = (Real)(zc - (double)zi);
            if (DIM == 1)
                key = (uint32_t)(xi / bin_w);
            else if (DIM == 2)
                key = (uint32_t)yi;
            else
                key = (uint32_t)(zi * g.size[1] + yi);
        }
        r.val = v;
        rec[k] = r;
        keys[k] = key;
        if (key < nbins)
            atomicAdd(&counts[key], 1u);
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long a = __shfl_xor_sync(0xffffffffu, kmin, o);
        unsigned long long b = __shfl_xor_sync(0xffffffffu, kmax, o);
        kmin = a < kmin ? a : kmin;
        kmax = b > kmax ? b : kmax;
    }
    nan = __any_sync(0xffffffffu, nan);
    if ((threadIdx.x & 31) == 0) {
        if (kmin != ~0ull)
            atomicMax(&hdr->vmin_key, ~kmin);
        if (kmax != 0ull)
            atomicMax(&hdr->vmax_key, kmax);
        if (nan)
            atomicExch(&hdr->nan_seen, 1);
    }
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

// Places every sample into its bin; the order inside a bin is fixed later.
__global__ void k_bin_scatter(const uint32_t *__restrict__ keys, int64_t npts, uint32_t nbins,
                              const uint32_t *__restrict__ start, uint32_t *__restrict__ cursor,
                              uint32_t *__restrict__ sorted)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npts;
         k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t key = keys[k];
        if (key < nbins)
            sorted[start[key] + atomicAdd(&cursor[key], 1u)] = (uint32_t)k;
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

// Sorts every bin's entries by sample index: one warp per bin, in registers for
// up to 32 entries, in shared memory up to kWarpSortMax; larger bins are listed
// for k_sort_large.
__global__ void __launch_bounds__(32 * kBinSortWarps) k_sort_bins(const uint32_t *__restrict__ start, uint32_t nbins,
                                                                  uint32_t *__restrict__ sorted,
                                                                  uint32_t *__restrict__ large)
{
    __shared__ uint32_t buf[kBinSortWarps][kWarpSortMax];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t b = (int64_t)blockIdx.x * kBinSortWarps + w;
    if (b >= nbins)
        return;
    const uint32_t s0 = start[b], c = start[b + 1] - s0;
    if (c <= 1)
        return;
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
        if (lane < (int)c)
            sorted[s0 + lane] = x;
        return;
    }
    if (c <= kWarpSortMax) {
        int n = 64;
        while (n < (int)c)
            n <<= 1;
        uint32_t *s = buf[w];
        for (int i = lane; i < n; i += 32)
            s[i] = i < (int)c ? sorted[s0 + i] : 0xFFFFFFFFu;
        __syncwarp();
        bitonic(s, n, lane, 32, WarpSync());
        for (int i = lane; i < (int)c; i += 32)
            sorted[s0 + i] = s[i];
        return;
    }
    if (lane == 0) {
        const uint32_t slot = atomicAdd(&large[0], 1u);
        large[1 + slot] = (uint32_t)b;
    }
}

// Sorts the bins too large for one warp, one block per bin at a time, in a
// scratch area of twice the bin size (padded to a power of two with keys that
// sort last).
__global__ void __launch_bounds__(1024) k_sort_large(const uint32_t *__restrict__ start, uint32_t *__restrict__ sorted,
                                                     const uint32_t *__restrict__ large,
                                                     uint32_t *__restrict__ scratch)
{
    const uint32_t nlarge = large[0];
    for (uint32_t q = blockIdx.x; q < nlarge; q += gridDim.x) {
        const uint32_t b = large[1 + q];
        const uint32_t s0 = start[b], c = start[b + 1] - s0;
        int n = 1;
        while (n < (int)c)
            n <<= 1;
        uint32_t *s = scratch + 2 * (size_t)s0;   // 2c >= n cells of this bin's own region
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            s[i] = i < (int)c ? sorted[s0 + i] : 0xFFFFFFFFu;
        __syncthreads();
        bitonic(s, n, threadIdx.x, (int)blockDim.x, BlockSync());
        for (int i = threadIdx.x; i < (int)c; i += blockDim.x)
            sorted[s0 + i] = s[i];
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// batched form: the samples of many 2D fields in one set of launches
// ---------------------------------------------------------------------------

// Bin keys and records of one block of one field's samples; keys are global
// bins (the field's bin offset + row), records indexed by global sample.
template <typename Real>
__global__ void k_batch_keys(const BatchKeyField *__restrict__ fields, const uint2 *__restrict__ blocks,
                             uint32_t skip_key, uint32_t *__restrict__ keys, SampleRec<Real> *__restrict__ rec,
                             uint32_t *__restrict__ counts, FieldHeader *__restrict__ hdrs)
{
    constexpr bool EXACT = sizeof(Real) == 8;
    const uint2 bt = blocks[blockIdx.x];   // (field, first sample of the block within the field)
    const BatchKeyField f = fields[bt.x];
    const double inv0 = 1.0 / f.step[0], inv1 = 1.0 / f.step[1];
    unsigned long long kmin = ~0ull, kmax = 0ull;
    int nan = 0;
    const int64_t end = min(f.npts, (int64_t)bt.y + kBatchKeysPerBlock);
    for (int64_t k = (int64_t)bt.y + threadIdx.x; k < end; k += blockDim.x) {
        const double v = f.val[k];
        if (isnan(v)) {
            nan = 1;
        } else {
            unsigned long long o = dbl_to_ordered(v);
            kmin = o < kmin ? o : kmin;
            kmax = o > kmax ? o : kmax;
        }
        const double *p = f.pts + 2 * k;
        const double xc = EXACT ? (p[0] - f.x0[0]) / f.step[0] : (p[0] - f.x0[0]) * inv0;
        const double yc = EXACT ? (p[1] - f.x0[1]) / f.step[1] : (p[1] - f.x0[1]) * inv1;
        const bool skip = xc < 0.0 || yc < 0.0 || xc >= (double)(f.size[0] - 1) || yc >= (double)(f.size[1] - 1);
        SampleRec<Real> r;
        r.xi = r.yi = r.zi = 0;
        r.xw = r.yw = r.zw = 0;
        uint32_t key = skip_key;
        if (!skip) {
            const int64_t xi = (int64_t)xc, yi = (int64_t)yc;
            r.xi = (int32_t)xi;
            r.yi = (int32_t)yi;
            r.xw = (Real)(xc - (double)xi);
            r.yw = (Real)(yc - (double)yi);
            key = f.bin_offset + (uint32_t)yi;
        }
        r.val = v;
        const int64_t gk = f.sample_offset + k;
        rec[gk] = r;
        keys[gk] = key;
        if (key < skip_key)
            atomicAdd(&counts[key], 1u);
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long a = __shfl_xor_sync(0xffffffffu, kmin, o);
        unsigned long long b = __shfl_xor_sync(0xffffffffu, kmax, o);
        kmin = a < kmin ? a : kmin;
        kmax = b > kmax ? b : kmax;
    }
    nan = __any_sync(0xffffffffu, nan);
    if ((threadIdx.x & 31) == 0) {
        FieldHeader *hdr = hdrs + bt.x;
        if (kmin != ~0ull)
            atomicMax(&hdr->vmin_key, ~kmin);
        if (kmax != 0ull)
            atomicMax(&hdr->vmax_key, kmax);
        if (nan)
            atomicExch(&hdr->nan_seen, 1);
    }
}

// Device-wide exclusive scan in three steps: sums of 4096-entry tiles, an
// exclusive scan of the tile sums (one block), and every tile scanned from
// its offset.
__global__ void __launch_bounds__(1024) k_tile_sums(const uint32_t *__restrict__ in, int64_t n,
                                                    uint32_t *__restrict__ sums)
{
    __shared__ uint32_t ws[32];
    const int64_t base = (int64_t)blockIdx.x * 4096;
    uint32_t s = 0;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int64_t i = base + 4 * threadIdx.x + u;
        s += i < n ? in[i] : 0u;
    }
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t t = ws[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1)
            t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0)
            sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) k_tile_scan(const uint32_t *__restrict__ in, int64_t n,
                                                    const uint32_t *__restrict__ offs, uint32_t *__restrict__ out)
{
    __shared__ uint32_t wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int64_t base = (int64_t)blockIdx.x * 4096;
    uint32_t x[4], s = 0;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int64_t i = base + 4 * t + u;
        x[u] = i < n ? in[i] : 0u;
        s += x[u];
    }
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
        const uint32_t v = wsum[lane];
        uint32_t wi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o)
                wi += y;
        }
        wsum[lane] = wi - v;
    }
    __syncthreads();
    uint32_t run = offs[blockIdx.x] + wsum[w] + inc - s;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int64_t i = base + 4 * t + u;
        if (i < n)
            out[i] = run;
        run += x[u];
    }
}

size_t batch_sort_scratch_bytes(int64_t ntot, uint32_t nbins, int precision)
{
    const size_t tiles = ((size_t)nbins + 1 + 4095) / 4096;
    return sort_scratch_bytes(ntot, nbins, precision) + 8 * tiles + 256;
}

void batch_sort_views(int precision, int64_t ntot, uint32_t nbins, uint32_t *scratch, const uint32_t **sorted_idx,
                      const void **recs)
{
    const size_t words = 3 * ((size_t)nbins + 2) + 4 * (size_t)ntot;
    *sorted_idx = scratch + 3 * ((size_t)nbins + 2) + (size_t)ntot;
    *recs = reinterpret_cast<char *>(scratch) + (4 * words + 255) / 256 * 256;
    (void)precision;
}

cudaError_t batch_sort(int precision, const BatchKeyField *d_fields, const uint2 *d_blocks, uint32_t nblocks,
                       int64_t ntot, uint32_t nbins, FieldHeader *hdrs, int nfields, uint32_t *scratch,
                       uint32_t *bin_start, const uint32_t **sorted_idx, const void **recs, cudaStream_t st)
{
    uint32_t *counts = scratch;
    uint32_t *cursor = counts + (nbins + 2);
    uint32_t *large = cursor + (nbins + 2);
    uint32_t *keys = large + (nbins + 2);
    uint32_t *sorted = keys + ntot;
    uint32_t *big = sorted + ntot;
    const size_t words = 3 * ((size_t)nbins + 2) + 4 * (size_t)ntot;
    char *rec = reinterpret_cast<char *>(scratch) + (4 * words + 255) / 256 * 256;
    const size_t recb = precision == 0 ? sizeof(SampleRec<double>) : sizeof(SampleRec<float>);
    uint32_t *tsum = reinterpret_cast<uint32_t *>(rec + ((recb * (size_t)ntot + 255) / 256 * 256));
    cudaError_t e = cudaMemsetAsync(hdrs, 0, sizeof(FieldHeader) * (size_t)nfields, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * 3 * ((size_t)nbins + 2), st);
    if (e != cudaSuccess)
        return e;
    *sorted_idx = sorted;
    *recs = rec;
    if (nblocks > 0) {
        if (precision == 0)
            k_batch_keys<double><<<nblocks, 256, 0, st>>>(d_fields, d_blocks, nbins, keys,
                                                           reinterpret_cast<SampleRec<double> *>(rec), counts, hdrs);
        else
            k_batch_keys<float><<<nblocks, 256, 0, st>>>(d_fields, d_blocks, nbins, keys,
                                                          reinterpret_cast<SampleRec<float> *>(rec), counts, hdrs);
    }
    const int64_t n = (int64_t)nbins + 1;
    const unsigned tiles = (unsigned)((n + 4095) / 4096);
    k_tile_sums<<<tiles, 1024, 0, st>>>(counts, n, tsum);
    uint32_t *toff = tsum + tiles;
    k_scan_exclusive<<<1, 1024, 0, st>>>(tsum, toff, (int64_t)tiles);
    k_tile_scan<<<tiles, 1024, 0, st>>>(counts, n, toff, bin_start);
    if (ntot > 0) {
        int blocks = (int)std::min<int64_t>((ntot + 255) / 256, 152 * 8);
        k_bin_scatter<<<blocks, 256, 0, st>>>(keys, ntot, nbins, bin_start, cursor, sorted);
        k_sort_bins<<<(unsigned)((nbins + kBinSortWarps - 1) / kBinSortWarps), 32 * kBinSortWarps, 0, st>>>(
            bin_start, nbins, sorted, large);
        k_sort_large<<<64, 1024, 0, st>>>(bin_start, sorted, large, big);
    }
    return cudaGetLastError();
}

// Scratch layout: counts[nbins + 2] | cursor[nbins + 2] | large[nbins + 2] |
// keys[N] | sorted[N] | big-bin scratch[2N] (uint32), then the sample records.
size_t sort_scratch_bytes(int64_t npts, uint32_t nbins, int precision)
{
    const size_t words = 3 * ((size_t)nbins + 2) + 4 * (size_t)npts;
    const size_t rec = precision == 0 ? sizeof(SampleRec<double>) : sizeof(SampleRec<float>);
    return (4 * words + 255) / 256 * 256 + rec * (size_t)npts + 256;
}

cudaError_t sort_samples(int precision, const double *pts, const double *val, int64_t npts, const Geometry &g,
                         int bin_w, uint32_t nbins, FieldHeader *hdr, uint32_t *scratch, uint32_t *bin_start,
                         const uint32_t **sorted_idx, const void **recs, cudaStream_t st)
{
    uint32_t *counts = scratch;
    uint32_t *cursor = counts + (nbins + 2);
    uint32_t *large = cursor + (nbins + 2);
    uint32_t *keys = large + (nbins + 2);
    uint32_t *sorted = keys + npts;
    uint32_t *big = sorted + npts;
    const size_t words = 3 * ((size_t)nbins + 2) + 4 * (size_t)npts;
    void *rec = reinterpret_cast<char *>(scratch) + (4 * words + 255) / 256 * 256;
    cudaError_t e = cudaMemsetAsync(hdr, 0, sizeof(FieldHeader), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * 3 * ((size_t)nbins + 2), st);
    if (e != cudaSuccess)
        return e;
    *sorted_idx = sorted;
    *recs = rec;
    if (npts > 0) {
        int blocks = (int)std::min<int64_t>((npts + 255) / 256, 152 * 8);
#define FBG_KEYS(D, R)                                                                                            \
    k_bin_keys<D, R><<<blocks, 256, 0, st>>>(pts, val, npts, g, bin_w, nbins, keys,                                \
                                             reinterpret_cast<SampleRec<R> *>(rec), counts, hdr)
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
    k_scan_exclusive<<<1, 1024, 0, st>>>(counts, bin_start, (int64_t)nbins + 1);
    if (npts > 0) {
        int blocks = (int)std::min<int64_t>((npts + 255) / 256, 152 * 8);
        k_bin_scatter<<<blocks, 256, 0, st>>>(keys, npts, nbins, bin_start, cursor, sorted);
        k_sort_bins<<<(unsigned)((nbins + kBinSortWarps - 1) / kBinSortWarps), 32 * kBinSortWarps, 0, st>>>(
            bin_start, nbins, sorted, large);
        k_sort_large<<<64, 1024, 0, st>>>(bin_start, sorted, large, big);
    }
    return cudaGetLastError();
}

}  // namespace fbg
