// fb_sort.cu -- sample preparation for the splat: value range, bin keys and a
// stable, deterministic counting sort of the samples by grid row.
//
// Replaces the per-sample loop head of _inject_data_{1,2,3}d
// (fastbarnes/interpolation.py:218-322: cell index, skip rule) and
// _normalize_values (:204-212: min/max of the values).  The reference adds the
// samples in index order; the splatting kernel keeps that order inside every
// row because the sort below is stable (LSD radix sort, 8-bit digits, ranks
// resolved warp-serially in index order).
#include "fb_internal.cuh"
#include "fb_kernels.cuh"

namespace fbg {

constexpr int kSortItems = 64;                  // keys per lane per tile
constexpr int kSortTile = 32 * kSortItems;      // keys per warp tile
constexpr int kSortWarps = 4;                   // warps (tiles) per block

__global__ void k_header_init(FieldHeader *h)
{
    h->vmin_key = ~0ull;
    h->vmax_key = 0ull;
    h->nan_seen = 0;
    h->error = 0;
}

// Bin key of every sample (nbins for samples the reference skips) and the
// min / max / NaN reduction of the values.
template <int DIM>
__global__ void k_bin_keys(const double *__restrict__ pts, const double *__restrict__ val, int64_t npts,
                           Geometry g, int bin_w, uint32_t nbins, uint32_t *__restrict__ keys,
                           FieldHeader *hdr)
{
    unsigned long long kmin = ~0ull, kmax = 0ull;
    int nan = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npts;
         k += (int64_t)gridDim.x * blockDim.x) {
        double v = val[k];
        if (isnan(v)) {
            nan = 1;
        } else {
            unsigned long long o = dbl_to_ordered(v);
            kmin = o < kmin ? o : kmin;
            kmax = o > kmax ? o : kmax;
        }
        uint32_t key = nbins;
        const double *p = pts + k * DIM;
        double xc = (p[0] - g.x0[0]) / g.step[0];
        if (DIM == 1) {
            if (!(xc < 0.0 || xc >= (double)(g.size[0] - 1)))
                key = (uint32_t)((int64_t)xc / bin_w);
        } else if (DIM == 2) {
            double yc = (p[1] - g.x0[1]) / g.step[1];
            if (!(xc < 0.0 || yc < 0.0 || xc >= (double)(g.size[0] - 1) || yc >= (double)(g.size[1] - 1)))
                key = (uint32_t)(int64_t)yc;
        } else {
            double yc = (p[1] - g.x0[1]) / g.step[1];
            double zc = (p[2] - g.x0[2]) / g.step[2];
            if (!(xc < 0.0 || yc < 0.0 || zc < 0.0 || xc >= (double)(g.size[0] - 1) ||
                  yc >= (double)(g.size[1] - 1) || zc >= (double)(g.size[2] - 1)))
                key = (uint32_t)((int64_t)zc * g.size[1] + (int64_t)yc);
        }
        keys[k] = key;
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
            atomicMin(&hdr->vmin_key, kmin);
        if (kmax != 0ull)
            atomicMax(&hdr->vmax_key, kmax);
        if (nan)
            atomicExch(&hdr->nan_seen, 1);
    }
}

// Per-warp-tile histogram of one 8-bit digit, stored digit-major:
// hist[d * ntiles + tile].
__global__ void k_radix_hist(const uint32_t *__restrict__ keys, int64_t n, int shift,
                             uint32_t *__restrict__ hist, int64_t ntiles)
{
    __shared__ uint32_t cnt[kSortWarps][256];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t tile = (int64_t)blockIdx.x * kSortWarps + w;
    for (int d = lane; d < 256; d += 32)
        cnt[w][d] = 0;
    __syncwarp();
    if (tile < ntiles) {
        const int64_t base = tile * kSortTile;
        for (int s = 0; s < kSortItems; s++) {
            int64_t i = base + s * 32 + lane;
            if (i < n)
                atomicAdd(&cnt[w][(keys[i] >> shift) & 255u], 1u);
        }
        __syncwarp();
        for (int d = lane; d < 256; d += 32)
            hist[(int64_t)d * ntiles + tile] = cnt[w][d];
    }
}

// Exclusive prefix sum of n entries in place, one block of 1024 threads.
__global__ void k_scan_exclusive(uint32_t *data, int64_t n)
{
    __shared__ uint32_t part[1024];
    const int t = threadIdx.x;
    const int64_t per = (n + 1023) / 1024;
    const int64_t b = t * per, e = b + per < n ? b + per : n;
    uint32_t s = 0;
    for (int64_t i = b; i < e; i++)
        s += data[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint32_t v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - s;
    for (int64_t i = b; i < e; i++) {
        uint32_t x = data[i];
        data[i] = run;
        run += x;
    }
}

// Stable scatter of one digit: inside a warp tile the keys are ranked in index
// order, 32 at a time; lanes with equal digits are ranked by lane.
__global__ void k_radix_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                                uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, int64_t n,
                                int shift, const uint32_t *__restrict__ offs, int64_t ntiles,
                                int first)
{
    __shared__ uint32_t cur[kSortWarps][256];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t tile = (int64_t)blockIdx.x * kSortWarps + w;
    if (tile >= ntiles)
        return;
    for (int d = lane; d < 256; d += 32)
        cur[w][d] = offs[(int64_t)d * ntiles + tile];
    __syncwarp();
    const uint32_t lt = (1u << lane) - 1u;
    const int64_t base = tile * kSortTile;
    for (int s = 0; s < kSortItems; s++) {
        int64_t i = base + s * 32 + lane;
        bool valid = i < n;
        uint32_t key = valid ? kin[i] : 0u;
        uint32_t v = valid ? (first ? (uint32_t)i : vin[i]) : 0u;
        uint32_t d = valid ? ((key >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt);
        uint32_t pos = valid ? cur[w][d] + rank : 0u;
        __syncwarp();
        if (valid && lane == 31 - __clz(peers))
            cur[w][d] += __popc(peers);
        __syncwarp();
        if (valid) {
            kout[pos] = key;
            vout[pos] = v;
        }
    }
}

// bin_start[b] = first sorted position whose key is >= b, b in [0, nbins].
__global__ void k_bin_start(const uint32_t *__restrict__ skeys, int64_t n, uint32_t *__restrict__ start,
                            uint32_t nbins)
{
    int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b > nbins)
        return;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (skeys[mid] < (uint32_t)b)
            lo = mid + 1;
        else
            hi = mid;
    }
    start[b] = (uint32_t)lo;
}

size_t sort_scratch_bytes(int64_t npts)
{
    int64_t ntiles = (npts + kSortTile - 1) / kSortTile;
    if (ntiles < 1)
        ntiles = 1;
    return (size_t)4 * (4 * (size_t)npts + 256 * (size_t)ntiles) + 256;
}

// Orders the samples of one field by bin.  Scratch layout (uint32):
// keys[N] | keys_alt[N] | idx[N] | idx_alt[N] | hist[256 * ntiles].
cudaError_t sort_samples(const double *pts, const double *val, int64_t npts, const Geometry &g,
                         int bin_w, uint32_t nbins, FieldHeader *hdr, uint32_t *scratch,
                         uint32_t *bin_start, const uint32_t **sorted_idx, cudaStream_t st)
{
    k_header_init<<<1, 1, 0, st>>>(hdr);
    int64_t ntiles = (npts + kSortTile - 1) / kSortTile;
    uint32_t *keys = scratch, *keys2 = scratch + npts, *idx = scratch + 2 * npts, *idx2 = scratch + 3 * npts;
    uint32_t *hist = scratch + 4 * npts;
    if (npts > 0) {
        int blocks = (int)((npts + 255) / 256);
        if (blocks > 152 * 16)
            blocks = 152 * 16;
        if (g.dim == 1)
            k_bin_keys<1><<<blocks, 256, 0, st>>>(pts, val, npts, g, bin_w, nbins, keys, hdr);
        else if (g.dim == 2)
            k_bin_keys<2><<<blocks, 256, 0, st>>>(pts, val, npts, g, bin_w, nbins, keys, hdr);
        else
            k_bin_keys<3><<<blocks, 256, 0, st>>>(pts, val, npts, g, bin_w, nbins, keys, hdr);
        int bits = 32 - __builtin_clz(nbins | 1u);
        int passes = (bits + 7) / 8;
        int sblocks = (int)((ntiles + kSortWarps - 1) / kSortWarps);
        const uint32_t *ki = keys, *vi = nullptr;
        uint32_t *ko = keys2, *vo = idx;
        for (int p = 0; p < passes; p++) {
            k_radix_hist<<<sblocks, 32 * kSortWarps, 0, st>>>(ki, npts, 8 * p, hist, ntiles);
            k_scan_exclusive<<<1, 1024, 0, st>>>(hist, 256 * ntiles);
            k_radix_scatter<<<sblocks, 32 * kSortWarps, 0, st>>>(ki, vi, ko, vo, npts, 8 * p, hist, ntiles,
                                                                p == 0);
            // next pass reads what this one wrote
            const uint32_t *nk = ko, *nv = vo;
            ko = (ko == keys2) ? keys : keys2;
            vo = (vo == idx) ? idx2 : idx;
            ki = nk;
            vi = nv;
        }
        *sorted_idx = vi;
        k_bin_start<<<(int)((nbins + 1 + 255) / 256), 256, 0, st>>>(ki, npts, bin_start, nbins);
    } else {
        *sorted_idx = idx;
        cudaMemsetAsync(bin_start, 0, sizeof(uint32_t) * (nbins + 1), st);
    }
    return cudaGetLastError();
}

}  // namespace fbg
