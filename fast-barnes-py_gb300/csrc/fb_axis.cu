// fb_axis.cu -- the n-fold box-and-tail convolution along one grid axis.
//
// Replaces _convolve_tail_{1,2,3}d / _accumulate_tail_array
// (fastbarnes/interpolation.py:372-533) and, for the first axis, the splat of
// _inject_data_{1,2,3}d (:218-322); for the last axis it also applies the NaN
// mask (:420-430) and the quotient (vg / wg + offset) of :367.
//
// One CTA holds `lines_per_cta` whole lines (or halo-extended tiles of long
// lines) of both the value and the weight field in shared memory and runs all
// `passes` box passes there, so every grid point crosses HBM once per axis.
//
// Inside a pass every thread owns a chunk of K consecutive cells of one line.
// It starts from the exact window sums at both chunk ends (anchors, summed
// from per-chunk partial sums of the previous pass that lie entirely inside
// the window, so nothing cancels), slides forward over the first half of the
// chunk and backward over the second half, keeps the K outputs in registers,
// and writes them back in place after a barrier.  With K odd, the 32 lanes of
// a warp (32 consecutive chunks of one line) address 32 different banks.
//
// Window semantics are the reference's (interpolation.py:500-523): out[k] =
// sum_{|d|<=T} in[k+d] + alpha * (in[k-T-1] + in[k+T+1]), in[] = 0 outside
// [0, L).  Inside a tile the region beyond the tile's input extent reads as 0
// too; the halo of passes*(T+1) cells absorbs that, and only the tile's own
// cells are stored.
#include <algorithm>

#include "fb_internal.cuh"
#include "fb_kernels.cuh"

namespace fbg {

template <bool GUARD, typename Real>
__device__ __forceinline__ Real rd(const Real *__restrict__ s, int e, int E)
{
    if (GUARD)
        return (unsigned)e < (unsigned)E ? s[e] : Real(0);
    return s[e];
}

template <typename Real>
struct PassCoef {
    Real alpha;   // tail weight (unscaled form) or alpha / (2T+1+2alpha) (scaled form)
    Real inv;     // 1 (unscaled) or 1 / (2T+1+2alpha)
    bool scaled;
    __device__ __forceinline__ Real out(Real acc, Real tails) const
    {
        return scaled ? fma(acc, inv, alpha * tails) : fma(alpha, tails, acc);
    }
};

// Slides the window over the chunk [k0, k0 + K) of one line: forward from A0
// (window at k0) over the first half, backward from A1 (window at k0 + K) over
// the second half.
template <typename Real, int K, bool GUARD>
__device__ __forceinline__ void slide(const Real *__restrict__ s, int E, int k0, int T, Real A0, Real A1,
                                      const PassCoef<Real> &c, Real (&o)[K])
{
    constexpr int H = K / 2;
    Real acc = A0;
    Real prev = rd<GUARD>(s, k0 - T - 1, E);
#pragma unroll
    for (int i = 0; i < H; i++) {
        const int k = k0 + i;
        const Real nw = rd<GUARD>(s, k + T + 1, E);
        const Real od = rd<GUARD>(s, k - T, E);
        o[i] = c.out(acc, prev + nw);
        acc += nw;
        acc -= od;
        prev = od;
    }
    acc = A1;
    Real od = rd<GUARD>(s, k0 + K - 1 - T, E);
#pragma unroll
    for (int i = K - 1; i >= H; i--) {
        const int k = k0 + i;
        const Real nw = rd<GUARD>(s, k + T + 1, E);
        acc -= nw;
        acc += od;
        const Real tl = rd<GUARD>(s, k - T - 1, E);
        o[i] = c.out(acc, tl + nw);
        od = tl;
    }
}

// Narrow kernels (T <= TD_MAX): every output is summed directly from the
// K + 2T + 2 inputs the chunk needs, held in registers.  Sliding a window of
// only a few cells over 16 steps would carry the rounding error of large
// values that have already left the window.
template <typename Real, int K, int TD, bool GUARD>
__device__ __forceinline__ void direct_pass(const Real *__restrict__ s, int E, int k0, const PassCoef<Real> &c,
                                            Real (&o)[K])
{
    constexpr int NX = K + 2 * TD + 2;
    Real x[NX];
#pragma unroll
    for (int m = 0; m < NX; m++)
        x[m] = rd<GUARD>(s, k0 - TD - 1 + m, E);
#pragma unroll
    for (int i = 0; i < K; i++) {
        Real acc = x[i + 1];
#pragma unroll
        for (int d = 2; d <= 2 * TD + 1; d++)
            acc += x[i + d];
        o[i] = c.out(acc, x[i] + x[i + 2 * TD + 2]);
    }
}

template <typename Real>
struct DirectMax;
template <>
struct DirectMax<float> {
    static constexpr int T = 8;
};
template <>
struct DirectMax<double> {
    static constexpr int T = 3;
};

template <typename Real, int K, int TD>
__device__ __forceinline__ bool try_direct(int T, const Real *s, int E, int k0, bool guard, const PassCoef<Real> &c,
                                           Real (&o)[K])
{
    if constexpr (TD > DirectMax<Real>::T) {
        return false;
    } else {
        if (T != TD)
            return try_direct<Real, K, TD + 1>(T, s, E, k0, guard, c, o);
        if (guard)
            direct_pass<Real, K, TD, true>(s, E, k0, c, o);
        else
            direct_pass<Real, K, TD, false>(s, E, k0, c, o);
        return true;
    }
}

// Sums of a chunk used to build the next pass's anchors: the whole chunk (S),
// its first r2 cells (Pre) and its cells from r1 on (Suf).  Cells at or beyond
// the line extent count as zero.
template <typename Real, int K>
__device__ __forceinline__ void chunk_partials(const Real (&o)[K], int k0, int E, int r1, int r2, Real &S,
                                               Real &Pre, Real &Suf)
{
    Real s = 0, p = 0, u = 0;
#pragma unroll
    for (int i = 0; i < K; i++) {
        const Real x = (k0 + i < E) ? o[i] : Real(0);
        s += x;
        p += (i < r2) ? x : Real(0);
        u += (i >= r1) ? x : Real(0);
    }
    S = s;
    Pre = p;
    Suf = u;
}

template <typename Real>
__device__ __forceinline__ Real part_at(const Real *__restrict__ a, int m, int nch)
{
    return (unsigned)m < (unsigned)nch ? a[m] : Real(0);
}

// Window sums at k0 = jK and k0 + K from the chunk partials (T >= 1):
// window [k0-T, k0+T] = Suf[m1] + S[m1+1 .. m2-1] + Pre[m2], m1 = j - d1,
// m2 = j + d2 (d1 = ceil(T/K), d2 = floor((T+1)/K)).
template <typename Real>
__device__ __forceinline__ void anchors(const Real *__restrict__ S, const Real *__restrict__ Pre,
                                        const Real *__restrict__ Suf, int nch, int j, int d1, int d2,
                                        Real &A0, Real &A1)
{
    const int m1 = j - d1, m2 = j + d2;
    Real mid = 0;
    for (int m = m1 + 2; m <= m2 - 1; m++)
        mid += part_at(S, m, nch);
    const bool two = (m2 - m1) >= 2;
    A0 = part_at(Suf, m1, nch) + (two ? part_at(S, m1 + 1, nch) : Real(0)) + mid + part_at(Pre, m2, nch);
    A1 = part_at(Suf, m1 + 1, nch) + mid + (two ? part_at(S, m2, nch) : Real(0)) + part_at(Pre, m2 + 1, nch);
}

__device__ __forceinline__ int64_t line_base(const AxisLaunch &a, const Geometry &g, int64_t line)
{
    if (a.axis == 0)
        return line * a.L;
    if (a.axis == 1) {
        const int64_t W = g.size[0];
        return (line / W) * (W * g.size[1]) + (line % W);
    }
    return line;
}

// Accumulates the contributions of the samples in sorted positions [beg, end)
// to one line buffer pair, in sorted order.  Lanes take 32 consecutive
// samples; lanes hitting the same cell add one after the other in lane order,
// so the result does not depend on scheduling.
template <typename Real, int DIM>
__device__ void splat_range(Real *__restrict__ lv, Real *__restrict__ lw, int E, int64_t e0, int64_t line,
                            uint32_t beg, uint32_t end, const Geometry &g, const SampleView &sv,
                            double offset, int lane)
{
    const uint32_t lt = (1u << lane) - 1u;
    int64_t zl = 0, yl = 0;
    if (DIM == 2)
        yl = line;
    if (DIM == 3) {
        zl = line / g.size[1];
        yl = line % g.size[1];
    }
    for (uint32_t r = beg; r < end; r += 32) {
        const uint32_t i = r + lane;
        const bool valid = i < end;
        int64_t xi = 0;
        double xw = 0.0, row_w = 1.0, wz = 1.0, v = 0.0;
        if (valid) {
            const uint32_t idx = sv.sorted_idx[i];
            const double *p = sv.pts + (int64_t)idx * DIM;
            const double xc = (p[0] - g.x0[0]) / g.step[0];
            xi = (int64_t)xc;
            xw = xc - (double)xi;
            v = sv.val[idx] - offset;
            if (DIM >= 2) {
                const double yc = (p[1] - g.x0[1]) / g.step[1];
                const int64_t yi = (int64_t)yc;
                const double yw = yc - (double)yi;
                row_w = (yi == yl) ? (1.0 - yw) : yw;
            }
            if (DIM == 3) {
                const double zc = (p[2] - g.x0[2]) / g.step[2];
                const int64_t zi = (int64_t)zc;
                const double zw = zc - (double)zi;
                wz = (zi == zl) ? (1.0 - zw) : zw;
            }
        }
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const int64_t ec = xi + c - e0;
            const bool ok = valid && ec >= 0 && ec < E;
            const unsigned act = __ballot_sync(0xffffffffu, ok);
            if (act == 0u)
                continue;
            // corner weight (wx * wy) * wz, the reference's product order
            const double wx = c ? xw : (1.0 - xw);
            double w = wx;
            if (DIM >= 2)
                w = wx * row_w;
            if (DIM == 3)
                w = w * wz;
            const Real cv = (Real)(w * v);
            const Real cw = (Real)w;
            const int key = ok ? (int)ec : -1 - lane;
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            const int rank = __popc(peers & lt);
            const int cnt = ok ? __popc(peers) : 0;
            const int maxc = __reduce_max_sync(0xffffffffu, cnt);
            for (int q = 0; q < maxc; q++) {
                if (ok && rank == q) {
                    lv[ec] += cv;
                    lw[ec] += cw;
                }
                __syncwarp();
            }
        }
    }
}

template <typename Real, int DIM>
__device__ void splat_line(Real *lv, Real *lw, int E, int64_t e0, int64_t line, const Geometry &g,
                           const SampleView &sv, double offset, int lane)
{
    if (DIM == 1) {
        const int64_t lo = e0 >= 1 ? e0 - 1 : 0;
        const int64_t hi = e0 + E - 1;
        int64_t b0 = lo / sv.bin_w, b1 = hi / sv.bin_w;
        if (b1 > (int64_t)sv.nbins - 1)
            b1 = (int64_t)sv.nbins - 1;
        if (b0 <= b1)
            splat_range<Real, 1>(lv, lw, E, e0, line, sv.bin_start[b0], sv.bin_start[b1 + 1], g, sv, offset,
                                 lane);
    } else if (DIM == 2) {
        // samples whose lower corner row is line - 1 or line, in that order
        const int64_t b0 = line >= 1 ? line - 1 : line;
        splat_range<Real, 2>(lv, lw, E, e0, line, sv.bin_start[b0], sv.bin_start[line + 1], g, sv, offset,
                             lane);
    } else {
        const int64_t H = g.size[1];
        const int64_t z = line / H, y = line % H;
        for (int dz = 1; dz >= 0; dz--) {
            if (z - dz < 0)
                continue;
            const int64_t rb = (z - dz) * H;
            const int64_t b0 = y >= 1 ? rb + y - 1 : rb + y;
            splat_range<Real, 3>(lv, lw, E, e0, line, sv.bin_start[b0], sv.bin_start[rb + y + 1], g, sv, offset,
                                 lane);
        }
    }
}

// SPLAT_DIM: 0 = the lines are loaded from src_v / src_w, 1..3 = they are
// filled by splatting the samples of a field of that dimension.  K: chunk
// length (odd), chosen per launch by chunk_k().
template <typename Real, int K, int SPLAT_DIM>
__global__ void __launch_bounds__(1024, 1) k_axis(const AxisLaunch a, const Geometry g, const SampleView sv)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *sm = reinterpret_cast<Real *>(smem_raw);
    const int NL = a.lines_per_cta;
    const int P = a.line_pitch;
    const int CP = a.chunks_pad;
    Real *part = sm + (size_t)NL * 2 * P;   // [NL][2][3][CP]

    const int64_t group = blockIdx.x / a.ntiles;
    const int64_t tile = blockIdx.x % a.ntiles;
    const int64_t line0 = group * NL;
    const int nl = (int)min((int64_t)NL, a.nlines - line0);
    const int64_t t0 = tile * a.tile_len;
    const int64_t t1 = min(a.L, t0 + a.tile_len);
    const int64_t e0 = max((int64_t)0, t0 - (int64_t)a.halo);
    const int64_t e1 = min(a.L, t1 + (int64_t)a.halo);
    const int E = (int)(e1 - e0);
    const int nch = (E + K - 1) / K;

    const int tid = threadIdx.x;
    const int lf = tid / CP;   // (line, field) of this thread: line lf / 2, field lf % 2
    const int my = lf >> 1;
    const int j = tid - lf * CP;
    const bool active = my < nl && j < nch;
    const int k0 = j * K;
    const int T = a.T;
    const int d1 = (T + K - 1) / K, d2 = (T + 1) / K;
    const int r1 = d1 * K - T, r2 = (T + 1) - d2 * K;
    const double offset = (SPLAT_DIM != 0 || a.store_quot) ? field_offset(sv.hdr) : 0.0;

    // ---- fill -------------------------------------------------------------
    if (SPLAT_DIM == 0) {
        const Real *sv_ = reinterpret_cast<const Real *>(a.src_v);
        const Real *sw_ = reinterpret_cast<const Real *>(a.src_w);
        if (a.axis == 0) {
            for (int ln = 0; ln < nl; ln++) {
                const int64_t b = line_base(a, g, line0 + ln) + e0;
                for (int e = tid; e < E; e += blockDim.x) {
                    sm[(ln * 2 + 0) * P + e] = sv_[b + e];
                    sm[(ln * 2 + 1) * P + e] = sw_[b + e];
                }
            }
        } else {
            const int64_t st = a.elem_stride;
            for (int idx = tid; idx < nl * E; idx += blockDim.x) {
                const int ln = idx % nl, e = idx / nl;
                const int64_t gi = line_base(a, g, line0 + ln) + (e0 + e) * st;
                sm[(ln * 2 + 0) * P + e] = sv_[gi];
                sm[(ln * 2 + 1) * P + e] = sw_[gi];
            }
        }
    } else {
        for (int ln = 0; ln < nl; ln++)
            for (int e = tid; e < E; e += blockDim.x) {
                sm[(ln * 2 + 0) * P + e] = Real(0);
                sm[(ln * 2 + 1) * P + e] = Real(0);
            }
        __syncthreads();
        // the first warp of every line's value-field threads splats that line
        if (my < nl && (lf & 1) == 0 && j < 32)
            splat_line<Real, SPLAT_DIM>(sm + (my * 2 + 0) * P, sm + (my * 2 + 1) * P, E, e0, line0 + my, g, sv,
                                        offset, j);
    }
    __syncthreads();

    Real *ln_ = sm + lf * P;                  // this thread's line buffer
    Real *pp = part + (size_t)lf * 3 * CP;    // S | Pre | Suf of that line

    // direct sums only in the short-chunk kernels (the long chunk serves T > 32)
    const bool direct = (K == K64) && T <= DirectMax<Real>::T;
    // partials of the filled data (anchors of the first sliding pass)
    if (active && !direct) {
        Real o[K];
#pragma unroll
        for (int i = 0; i < K; i++)
            o[i] = (k0 + i < E) ? ln_[min(k0 + i, E - 1)] : Real(0);
        chunk_partials<Real, K>(o, k0, E, r1, r2, pp[j], pp[CP + j], pp[2 * CP + j]);
    }

    PassCoef<Real> coef;
    coef.scaled = a.inv_norm != 1.0;
    coef.inv = (Real)a.inv_norm;
    coef.alpha = coef.scaled ? (Real)(a.alpha * a.inv_norm) : (Real)a.alpha;

    for (int pass = 0; pass < a.passes; pass++) {
        __syncthreads();
        Real o[K];
        Real S = 0, Pr = 0, Su = 0;
        if (active) {
            const bool guard = (k0 - T - 1 < 0) || (k0 + K + T >= E);
            if constexpr (K == K64) {
                if (direct)
                    try_direct<Real, K, 0>(T, ln_, E, k0, guard, coef, o);
            }
            if (!direct) {
                Real A0, A1;
                anchors(pp, pp + CP, pp + 2 * CP, nch, j, d1, d2, A0, A1);
                if (guard)
                    slide<Real, K, true>(ln_, E, k0, T, A0, A1, coef, o);
                else
                    slide<Real, K, false>(ln_, E, k0, T, A0, A1, coef, o);
                chunk_partials<Real, K>(o, k0, E, r1, r2, S, Pr, Su);
            }
        }
        __syncthreads();
        if (active) {
            if (k0 + K <= E) {
#pragma unroll
                for (int i = 0; i < K; i++)
                    ln_[k0 + i] = o[i];
            } else {
#pragma unroll
                for (int i = 0; i < K; i++)
                    if (k0 + i < E)
                        ln_[k0 + i] = o[i];
            }
            if (!direct) {
                pp[j] = S;
                pp[CP + j] = Pr;
                pp[2 * CP + j] = Su;
            }
        }
    }
    __syncthreads();

    // ---- store ------------------------------------------------------------
    const int s0 = (int)(t0 - e0), s1 = (int)(t1 - e0);   // this tile's own cells
    const int ns = s1 - s0;
    if (a.store_quot) {
        const Real thr = (Real)a.thr;
        for (int idx = tid; idx < nl * ns; idx += blockDim.x) {
            int ln, e;
            if (a.axis == 0) {
                ln = idx / ns;
                e = s0 + idx % ns;
            } else {
                ln = idx % nl;
                e = s0 + idx / nl;
            }
            const Real v = sm[(ln * 2 + 0) * P + e];
            const Real w = sm[(ln * 2 + 1) * P + e];
            const int64_t gi = line_base(a, g, line0 + ln) + (e0 + e) * a.elem_stride;
            if (sizeof(Real) == 8) {
                double q = (w < thr) ? __longlong_as_double(0x7ff8000000000000ll) : (double)v / (double)w + offset;
                if (a.out_f64)
                    reinterpret_cast<double *>(a.out)[gi] = q;
                else
                    reinterpret_cast<float *>(a.out)[gi] = (float)q;
            } else {
                float q = (w < thr) ? __int_as_float(0x7fc00000) : (float)v / (float)w + (float)offset;
                if (a.out_f64)
                    reinterpret_cast<double *>(a.out)[gi] = (double)q;
                else
                    reinterpret_cast<float *>(a.out)[gi] = q;
            }
        }
    } else {
        Real *dv = reinterpret_cast<Real *>(a.dst_v);
        Real *dw = reinterpret_cast<Real *>(a.dst_w);
        for (int idx = tid; idx < nl * ns; idx += blockDim.x) {
            int ln, e;
            if (a.axis == 0) {
                ln = idx / ns;
                e = s0 + idx % ns;
            } else {
                ln = idx % nl;
                e = s0 + idx / nl;
            }
            const int64_t gi = line_base(a, g, line0 + ln) + (e0 + e) * a.elem_stride;
            dv[gi] = sm[(ln * 2 + 0) * P + e];
            dw[gi] = sm[(ln * 2 + 1) * P + e];
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Chunk length per launch.  Every output is at most K/2 sliding steps from an
// exact anchor; in float32 that distance must stay short against the window
// 2T+1, so windows up to 65 cells use the short chunk (and T <= 8 sums
// directly), wider ones the long chunk with half the anchor overhead.
static int chunk_k(int precision, int T)
{
    if (precision == 0)
        return K64;
    return T <= 32 ? K64 : K32;
}
static int real_size(int precision) { return precision == 0 ? 8 : 4; }

static size_t smem_limit()
{
    static int lim = -1;
    if (lim < 0) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0)
            v = 227 * 1024;
        lim = v;
    }
    return (size_t)lim;
}

AxisPlanLimits axis_limits(int precision, int T)
{
    AxisPlanLimits l;
    l.smem_limit = smem_limit();
    const int K = chunk_k(precision, T), sz = real_size(precision);
    // largest extent E with one line per CTA: threads and shared memory
    // a line takes two thread groups (value, weight) of chunks_pad threads
    int e_thr = kMaxLineThreads / 2 * K;
    int lo = 1, hi = e_thr;
    while (lo < hi) {
        int mid = (lo + hi + 1) / 2;
        int nch = (mid + K - 1) / K;
        int cp = (nch + 31) / 32 * 32;
        size_t pitch = (size_t)(mid + 31) / 32 * 32 + 2;
        size_t b = 2 * pitch * sz + 6 * (size_t)cp * sz;
        if (2 * cp <= kMaxLineThreads && b <= l.smem_limit)
            lo = mid;
        else
            hi = mid - 1;
    }
    l.extent_max = lo;
    return l;
}

size_t axis_smem_bytes(int precision, const AxisLaunch &a)
{
    const int sz = real_size(precision);
    return (size_t)a.lines_per_cta * (2 * (size_t)a.line_pitch * sz + 6 * (size_t)a.chunks_pad * sz);
}

bool axis_shape(int precision, AxisLaunch &a)
{
    const int K = chunk_k(precision, a.T);
    int64_t E = a.tile_len + 2 * (int64_t)a.halo;
    if (E > a.L)
        E = a.L;
    const int nch = (int)((E + K - 1) / K);
    const int cp = (nch + 31) / 32 * 32;
    if (2 * cp > kMaxLineThreads)
        return false;
    a.extent_max = (int)E;
    a.chunks_pad = cp;
    a.line_pitch = (int)((E + 31) / 32 * 32 + 2);
    // lines per CTA: contiguous rows want ~256-512 threads; strided axes want
    // 32-byte row segments (8 floats / 4 doubles) for sector-sized loads.
    int want = a.axis == 0 ? std::max(1, 256 / cp) : (precision == 0 ? 4 : 8);
    int nl = std::max(1, std::min<int>(want, kMaxLineThreads / (2 * cp)));
    if (nl > a.nlines)
        nl = (int)a.nlines;
    while (nl > 1) {
        a.lines_per_cta = nl;
        if (axis_smem_bytes(precision, a) <= smem_limit())
            break;
        nl--;
    }
    a.lines_per_cta = nl;
    return axis_smem_bytes(precision, a) <= smem_limit();
}

template <typename Real, int K, int SD>
static cudaError_t launch_one(const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st)
{
    const size_t smem = axis_smem_bytes(sizeof(Real) == 8 ? 0 : 1, a);
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(k_axis<Real, K, SD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem_limit());
        if (e != cudaSuccess)
            return e;
        configured = smem_limit();
    }
    const int64_t groups = (a.nlines + a.lines_per_cta - 1) / a.lines_per_cta;
    const int64_t blocks = groups * a.ntiles;
    const int threads = a.lines_per_cta * 2 * a.chunks_pad;
    k_axis<Real, K, SD><<<(unsigned)blocks, threads, smem, st>>>(a, g, sv);
    return cudaGetLastError();
}

template <typename Real, int K>
static cudaError_t launch_k(int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st)
{
    switch (sd) {
    case 0: return launch_one<Real, K, 0>(a, g, sv, st);
    case 1: return launch_one<Real, K, 1>(a, g, sv, st);
    case 2: return launch_one<Real, K, 2>(a, g, sv, st);
    default: return launch_one<Real, K, 3>(a, g, sv, st);
    }
}

cudaError_t launch_axis(int precision, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                        cudaStream_t st)
{
    const int sd = a.fill_splat ? g.dim : 0;
    if (precision == 0)
        return launch_k<double, K64>(sd, a, g, sv, st);
    if (chunk_k(precision, a.T) == K64)
        return launch_k<float, K64>(sd, a, g, sv, st);
    return launch_k<float, K32>(sd, a, g, sv, st);
}

cudaError_t launch_lines(int precision, void *data, int64_t nlines, int64_t len, int T, double alpha, int passes,
                         int normalize, cudaStream_t st)
{
    AxisLaunch a{};
    a.axis = 0;
    a.L = len;
    a.elem_stride = 1;
    a.nlines = nlines;
    a.tile_len = len;
    a.ntiles = 1;
    a.halo = 0;
    a.passes = passes;
    a.T = T;
    a.alpha = alpha;
    a.inv_norm = normalize ? 1.0 / (2.0 * T + 1.0 + 2.0 * alpha) : 1.0;
    a.fill_splat = 0;
    a.store_quot = 0;
    a.src_v = data;
    a.src_w = data;
    a.dst_v = data;
    a.dst_w = data;
    if (!axis_shape(precision, a))
        return cudaErrorInvalidValue;
    Geometry g{};
    g.dim = 1;
    g.size[0] = len;
    g.size[1] = g.size[2] = 1;
    SampleView sv{};
    return launch_axis(precision, a, g, sv, st);
}

}  // namespace fbg
