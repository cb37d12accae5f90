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

// ---------------------------------------------------------------------------
// one line of one field, seen by one thread: cell e lives at s[e * ES]
// ---------------------------------------------------------------------------

template <bool GUARD, int ES, typename Real>
__device__ __forceinline__ Real rd(const Real *__restrict__ s, int e, int E)
{
    if (GUARD)
        return (unsigned)e < (unsigned)E ? s[e * ES] : Real(0);
    return s[e * ES];
}

template <typename Real, bool SCALED>
struct PassCoef {
    Real alpha;   // tail weight (alpha * inv when scaled)
    Real inv;     // 1 / (2T+1+2alpha)
    __device__ __forceinline__ Real out(Real acc, Real tails) const
    {
        if (SCALED)
            return fma(acc, inv, alpha * tails);
        return fma(alpha, tails, acc);
    }
};

// Slides the window over the chunk [k0, k0 + K): forward from A0 (window at
// k0) over the first half, backward from A1 (window at k0 + K) over the rest.
template <typename Real, int K, int ES, bool GUARD, bool SCALED>
__device__ __forceinline__ void slide(const Real *__restrict__ s, int E, int k0, int T, Real A0, Real A1,
                                      const PassCoef<Real, SCALED> &c, Real (&o)[K])
{
    constexpr int H = K / 2;
    Real acc = A0;
    Real prev = rd<GUARD, ES>(s, k0 - T - 1, E);
#pragma unroll
    for (int i = 0; i < H; i++) {
        const int k = k0 + i;
        const Real nw = rd<GUARD, ES>(s, k + T + 1, E);
        const Real od = rd<GUARD, ES>(s, k - T, E);
        o[i] = c.out(acc, prev + nw);
        acc += nw;
        acc -= od;
        prev = od;
    }
    acc = A1;
    Real od = rd<GUARD, ES>(s, k0 + K - 1 - T, E);
#pragma unroll
    for (int i = K - 1; i >= H; i--) {
        const int k = k0 + i;
        const Real nw = rd<GUARD, ES>(s, k + T + 1, E);
        acc -= nw;
        acc += od;
        const Real tl = rd<GUARD, ES>(s, k - T - 1, E);
        o[i] = c.out(acc, tl + nw);
        od = tl;
    }
}

// Narrow kernels (T <= DirectMax): every output is summed directly from the
// K + 2T + 2 inputs the chunk needs, held in registers.  Sliding a window of
// only a few cells over K/2 steps would carry the rounding error of large
// values that have already left the window.
template <typename Real, int K, int ES, int TD, bool GUARD, bool SCALED>
__device__ __forceinline__ void direct_pass(const Real *__restrict__ s, int E, int k0,
                                            const PassCoef<Real, SCALED> &c, Real (&o)[K])
{
    constexpr int NX = K + 2 * TD + 2;
    Real x[NX];
#pragma unroll
    for (int m = 0; m < NX; m++)
        x[m] = rd<GUARD, ES>(s, k0 - TD - 1 + m, E);
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

template <typename Real, int K, int ES, int TD, bool SCALED>
__device__ __forceinline__ void direct_dispatch(int T, const Real *s, int E, int k0, bool guard,
                                                const PassCoef<Real, SCALED> &c, Real (&o)[K])
{
    if constexpr (TD <= DirectMax<Real>::T) {
        if (T != TD) {
            direct_dispatch<Real, K, ES, TD + 1, SCALED>(T, s, E, k0, guard, c, o);
            return;
        }
        if (guard)
            direct_pass<Real, K, ES, TD, true, SCALED>(s, E, k0, c, o);
        else
            direct_pass<Real, K, ES, TD, false, SCALED>(s, E, k0, c, o);
    }
}

// Sums of a chunk that the next pass's anchors are built from: the whole
// chunk (S), its first r2 cells (Pre) and its cells from r1 on (Suf).  Cells
// at or beyond the line extent count as zero (tail chunk only).
template <typename Real, int K, bool TAIL>
__device__ __forceinline__ void chunk_partials(const Real (&o)[K], int k0, int E, int r1, int r2, Real &S,
                                               Real &Pre, Real &Suf)
{
    Real s = 0, p = 0, u = 0;
#pragma unroll
    for (int i = 0; i < K; i++) {
        const Real x = (!TAIL || k0 + i < E) ? o[i] : Real(0);
        s += x;
        if (i < r2)
            p += x;
        if (i >= r1)
            u += x;
    }
    S = s;
    Pre = p;
    Suf = u;
}

template <typename Real, int PS>
__device__ __forceinline__ Real part_at(const Real *__restrict__ a, int m, int nch)
{
    return (unsigned)m < (unsigned)nch ? a[m * PS] : Real(0);
}

// Window sums at k0 = jK and k0 + K from the chunk partials (T >= 1):
// window [k0-T, k0+T] = Suf[m1] + S[m1+1 .. m2-1] + Pre[m2], m1 = j - d1,
// m2 = j + d2 (d1 = ceil(T/K), d2 = floor((T+1)/K)).  Every term is a sum of
// cells inside the window: nothing is subtracted.
template <typename Real, int PS>
__device__ __forceinline__ void anchors(const Real *__restrict__ S, const Real *__restrict__ Pre,
                                        const Real *__restrict__ Suf, int nch, int j, int d1, int d2,
                                        Real &A0, Real &A1)
{
    const int m1 = j - d1, m2 = j + d2;
    Real mid = 0;
    for (int m = m1 + 2; m <= m2 - 1; m++)
        mid += part_at<Real, PS>(S, m, nch);
    const bool two = (m2 - m1) >= 2;
    A0 = part_at<Real, PS>(Suf, m1, nch) + (two ? part_at<Real, PS>(S, m1 + 1, nch) : Real(0)) + mid +
         part_at<Real, PS>(Pre, m2, nch);
    A1 = part_at<Real, PS>(Suf, m1 + 1, nch) + mid + (two ? part_at<Real, PS>(S, m2, nch) : Real(0)) +
         part_at<Real, PS>(Pre, m2 + 1, nch);
}

// One box pass of one thread's chunk: outputs into o, next partials into S/P/U.
template <typename Real, int K, int ES, int PS, bool SCALED>
__device__ __forceinline__ void run_pass(const Real *__restrict__ ln, const Real *__restrict__ pp, int QS, int E,
                                         int nch, int j, int T, int d1, int d2, int r1, int r2, bool direct,
                                         const PassCoef<Real, SCALED> &c, Real (&o)[K], Real &S, Real &P, Real &U)
{
    const int k0 = j * K;
    const bool guard = (k0 - T - 1 < 0) || (k0 + K + T >= E);
    if constexpr (K == K64) {
        if (direct) {
            direct_dispatch<Real, K, ES, 0, SCALED>(T, ln, E, k0, guard, c, o);
            return;
        }
    }
    Real A0, A1;
    anchors<Real, PS>(pp, pp + QS, pp + 2 * QS, nch, j, d1, d2, A0, A1);
    if (guard)
        slide<Real, K, ES, true, SCALED>(ln, E, k0, T, A0, A1, c, o);
    else
        slide<Real, K, ES, false, SCALED>(ln, E, k0, T, A0, A1, c, o);
    if (k0 + K <= E)
        chunk_partials<Real, K, false>(o, k0, E, r1, r2, S, P, U);
    else
        chunk_partials<Real, K, true>(o, k0, E, r1, r2, S, P, U);
}

template <typename Real>
__device__ __forceinline__ Real quotient(Real v, Real w, Real thr, double offset);
template <>
__device__ __forceinline__ double quotient<double>(double v, double w, double thr, double offset)
{
    // NaN where the weight is below the mask level, else vg / wg + offset
    return (w < thr) ? __longlong_as_double(0x7ff8000000000000ll) : v / w + offset;
}
template <>
__device__ __forceinline__ float quotient<float>(float v, float w, float thr, double offset)
{
    return (w < thr) ? __int_as_float(0x7fc00000) : v / w + (float)offset;
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

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------

template <int G, typename Real>
struct Vec;   // 16-byte vector of Real
template <int G>
struct Vec<G, float> {
    using T = float4;
};
template <int G>
struct Vec<G, double> {
    using T = double2;
};

// Column-layout group width: 32 bytes of each line-segment row.
template <typename Real>
struct ColG {
    static constexpr int G = 32 / sizeof(Real);
};

// SPLAT_DIM: 0 = the lines are loaded from src_v / src_w, 1..3 = they are
// filled by splatting the samples of a field of that dimension (rows layout).
// LAYOUT: 0 = rows, 1 = columns.  K: chunk length (odd).
template <typename Real, int K, int SPLAT_DIM, int LAYOUT>
__global__ void __launch_bounds__(1024, 1) k_axis(const AxisLaunch a, const Geometry g, const SampleView sv)
{
    constexpr int G = ColG<Real>::G;
    constexpr int ES = LAYOUT == 0 ? 1 : G;   // cell stride inside a line buffer
    constexpr int PS = LAYOUT == 0 ? 1 : G;   // chunk stride inside a partials array
    constexpr int VPR = 16 / sizeof(Real);    // cells per 16-byte vector
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *sm = reinterpret_cast<Real *>(smem_raw);
    const int P = a.line_pitch;
    const int CP = a.chunks_pad;
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;

    const int64_t group = blockIdx.x / a.ntiles;
    const int64_t tile = blockIdx.x - group * a.ntiles;
    const int64_t t0 = tile * a.tile_len;
    const int64_t t1 = min(a.L, t0 + a.tile_len);
    const int64_t e0 = max((int64_t)0, t0 - (int64_t)a.halo);
    const int64_t e1 = min(a.L, t1 + (int64_t)a.halo);
    const int E = (int)(e1 - e0);
    const int nch = (E + K - 1) / K;

    // lines of this CTA and their HBM base (cell e0 of the line)
    int nl;                  // lines present
    int64_t line0 = 0;       // rows: first line index
    int64_t gbase = 0;       // columns: HBM index of (line 0 of the group, cell e0)
    bool vec_ok = false;     // columns: 16-byte row segments are aligned
    if (LAYOUT == 0) {
        line0 = group * a.lines_per_cta;
        nl = (int)min((int64_t)a.lines_per_cta, a.nlines - line0);
    } else {
        const int64_t o = group / a.xblocks, xb = group - o * a.xblocks;
        nl = (int)min((int64_t)G, a.width - xb * G);
        gbase = o * a.outer_stride + xb * G + e0 * a.elem_stride;
        vec_ok = nl == G && (gbase % VPR) == 0 && (a.elem_stride % VPR) == 0;
    }

    // this thread's line / field / chunk
    int lf, f, ln_i, j;
    Real *ln;
    Real *pp;
    int QS;
    if (LAYOUT == 0) {
        lf = tid / CP;
        j = tid - lf * CP;
        f = lf & 1;
        ln_i = lf >> 1;
        ln = sm + (size_t)lf * P;
        QS = CP;
        pp = sm + (size_t)a.lines_per_cta * 2 * P + (size_t)lf * 3 * CP + j;
    } else {
        const int tpf = G * CP;
        f = tid / tpf;
        const int r = tid - f * tpf;
        ln_i = r % G;
        j = r / G;
        lf = f;
        ln = sm + (size_t)f * P * G + ln_i;
        QS = CP * G;
        pp = sm + (size_t)2 * P * G + (size_t)f * 3 * CP * G + ln_i + (size_t)j * G;
    }
    // pp points at S[j]; the anchors index relative to chunk 0
    Real *pp0 = pp - (size_t)j * PS;
    const bool active = ln_i < nl && j < nch && f < 2;
    const int T = a.T;
    const int d1 = (T + K - 1) / K, d2 = (T + 1) / K;
    const int r1 = d1 * K - T, r2 = (T + 1) - d2 * K;
    const double offset = (SPLAT_DIM != 0 || a.store_quot) ? field_offset(sv.hdr) : 0.0;

    // ---- fill -------------------------------------------------------------
    if (SPLAT_DIM != 0) {
        // rows layout: zero the line buffers, then one warp per line splats
        float4 *z4 = reinterpret_cast<float4 *>(sm);
        const int n4 = (int)((size_t)a.lines_per_cta * 2 * P * sizeof(Real) / 16);
        for (int i = tid; i < n4; i += nthr)
            z4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        if (ln_i < nl && f == 0 && j < 32)
            splat_line<Real, SPLAT_DIM>(sm + (size_t)(ln_i * 2) * P, sm + (size_t)(ln_i * 2 + 1) * P, E, e0,
                                        line0 + ln_i, g, sv, offset, j);
    } else if (LAYOUT == 0) {
        const Real *src[2] = {reinterpret_cast<const Real *>(a.src_v), reinterpret_cast<const Real *>(a.src_w)};
        for (int q = 0; q < 2 * nl; q++) {
            const Real *s_ = src[q & 1] + (line0 + (q >> 1)) * a.L + e0;
            Real *d_ = sm + (size_t)((q >> 1) * 2 + (q & 1)) * P;
            for (int e = tid; e < E; e += nthr)
                d_[e] = s_[e];
        }
    } else {
        const Real *src[2] = {reinterpret_cast<const Real *>(a.src_v), reinterpret_cast<const Real *>(a.src_w)};
        const int64_t es = a.elem_stride;
        if (vec_ok) {
            using V = typename Vec<G, Real>::T;
            constexpr int VR = G / VPR;   // vectors per row (2)
            const int nv = E * VR;
#pragma unroll 1
            for (int ff = 0; ff < 2; ff++) {
                V *d_ = reinterpret_cast<V *>(sm + (size_t)ff * P * G);
                const Real *s_ = src[ff] + gbase;
#pragma unroll 4
                for (int i = tid; i < nv; i += nthr) {
                    const int row = i / VR, h = i - row * VR;
                    d_[i] = *reinterpret_cast<const V *>(s_ + row * es + h * VPR);
                }
            }
        } else {
            for (int ff = 0; ff < 2; ff++) {
                Real *d_ = sm + (size_t)ff * P * G;
                const Real *s_ = src[ff] + gbase;
                for (int i = tid; i < E * G; i += nthr) {
                    const int row = i / G, gg = i - row * G;
                    d_[i] = gg < nl ? s_[row * es + gg] : Real(0);
                }
            }
        }
    }
    __syncthreads();

    // ---- passes -----------------------------------------------------------
    const bool direct = (K == K64) && T <= DirectMax<Real>::T;
    if (active && !direct) {
        // partials of the filled data
        Real o[K];
        const int k0 = j * K;
#pragma unroll
        for (int i = 0; i < K; i++)
            o[i] = (k0 + i < E) ? ln[(k0 + i) * ES] : Real(0);
        Real S, Pr, Su;
        chunk_partials<Real, K, true>(o, k0, E, r1, r2, S, Pr, Su);
        pp[0] = S;
        pp[QS] = Pr;
        pp[2 * QS] = Su;
    }

    PassCoef<Real, false> cu;
    cu.alpha = (Real)a.alpha;
    cu.inv = (Real)1;
    PassCoef<Real, true> cs;
    cs.alpha = (Real)(a.alpha * a.inv_norm);
    cs.inv = (Real)a.inv_norm;

    for (int pass = 0; pass < a.passes; pass++) {
        __syncthreads();
        Real o[K];
        Real S = 0, Pr = 0, Su = 0;
        if (active) {
            if (a.scaled)
                run_pass<Real, K, ES, PS, true>(ln, pp0, QS, E, nch, j, T, d1, d2, r1, r2, direct, cs, o, S, Pr, Su);
            else
                run_pass<Real, K, ES, PS, false>(ln, pp0, QS, E, nch, j, T, d1, d2, r1, r2, direct, cu, o, S, Pr,
                                                 Su);
        }
        __syncthreads();
        if (active) {
            const int k0 = j * K;
            if (k0 + K <= E) {
#pragma unroll
                for (int i = 0; i < K; i++)
                    ln[(k0 + i) * ES] = o[i];
            } else {
#pragma unroll
                for (int i = 0; i < K; i++)
                    if (k0 + i < E)
                        ln[(k0 + i) * ES] = o[i];
            }
            if (!direct) {
                pp[0] = S;
                pp[QS] = Pr;
                pp[2 * QS] = Su;
            }
        }
    }
    __syncthreads();

    // ---- store ------------------------------------------------------------
    const int s0 = (int)(t0 - e0), s1 = (int)(t1 - e0);   // this tile's own cells
    const Real thr = (Real)a.thr;
    if (LAYOUT == 0) {
        for (int q = 0; q < nl; q++) {
            const Real *v_ = sm + (size_t)(q * 2) * P;
            const Real *w_ = v_ + P;
            const int64_t gb = (line0 + q) * a.L + e0;
            if (a.store_quot) {
                if (a.out_f64) {
                    double *o_ = reinterpret_cast<double *>(a.out) + gb;
                    for (int e = s0 + tid; e < s1; e += nthr)
                        o_[e] = (double)quotient<Real>(v_[e], w_[e], thr, offset);
                } else {
                    float *o_ = reinterpret_cast<float *>(a.out) + gb;
                    for (int e = s0 + tid; e < s1; e += nthr)
                        o_[e] = (float)quotient<Real>(v_[e], w_[e], thr, offset);
                }
            } else {
                Real *dv = reinterpret_cast<Real *>(a.dst_v) + gb;
                Real *dw = reinterpret_cast<Real *>(a.dst_w) + gb;
                for (int e = s0 + tid; e < s1; e += nthr) {
                    dv[e] = v_[e];
                    dw[e] = w_[e];
                }
            }
        }
    } else {
        const int64_t es = a.elem_stride;
        const Real *v_ = sm;
        const Real *w_ = sm + (size_t)P * G;
        if (a.store_quot) {
            // 4 cells of one row per thread: one 16-byte float32 store
            const int nq = (s1 - s0) * (G / 4);
            const bool q_vec = nl == G && !a.out_f64 && (gbase % 4) == 0 && (es % 4) == 0;
            for (int i = tid; i < nq; i += nthr) {
                const int row = s0 + i / (G / 4), c4 = (i % (G / 4)) * 4;
                Real q4[4];
#pragma unroll
                for (int u = 0; u < 4; u++)
                    q4[u] = quotient<Real>(v_[row * G + c4 + u], w_[row * G + c4 + u], thr, offset);
                const int64_t gi = gbase + row * es + c4;
                if (q_vec) {
                    *reinterpret_cast<float4 *>(reinterpret_cast<float *>(a.out) + gi) =
                        make_float4((float)q4[0], (float)q4[1], (float)q4[2], (float)q4[3]);
                } else {
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        if (c4 + u < nl) {
                            if (a.out_f64)
                                reinterpret_cast<double *>(a.out)[gi + u] = (double)q4[u];
                            else
                                reinterpret_cast<float *>(a.out)[gi + u] = (float)q4[u];
                        }
                    }
                }
            }
        } else {
            Real *dst[2] = {reinterpret_cast<Real *>(a.dst_v), reinterpret_cast<Real *>(a.dst_w)};
            if (vec_ok) {
                using V = typename Vec<G, Real>::T;
                constexpr int VR = G / VPR;
                const int nv = (s1 - s0) * VR;
                for (int ff = 0; ff < 2; ff++) {
                    const V *s_ = reinterpret_cast<const V *>(sm + (size_t)ff * P * G) + s0 * VR;
                    Real *d_ = dst[ff] + gbase;
                    for (int i = tid; i < nv; i += nthr) {
                        const int row = s0 + i / VR, h = i - (row - s0) * VR;
                        *reinterpret_cast<V *>(d_ + row * es + h * VPR) = s_[i];
                    }
                }
            } else {
                for (int ff = 0; ff < 2; ff++) {
                    const Real *s_ = sm + (size_t)ff * P * G;
                    Real *d_ = dst[ff] + gbase;
                    for (int i = tid; i < (s1 - s0) * G; i += nthr) {
                        const int row = s0 + i / G, gg = i % G;
                        if (gg < nl)
                            d_[row * es + gg] = s_[row * G + gg];
                    }
                }
            }
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
static int col_g(int precision) { return 32 / real_size(precision); }

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

static int pitch_of(int64_t E) { return (int)((E + 31) / 32 * 32); }

size_t axis_smem_bytes(int precision, const AxisLaunch &a)
{
    const size_t sz = real_size(precision);
    if (a.layout == 0)
        return (size_t)a.lines_per_cta * (2 * (size_t)a.line_pitch + 6 * (size_t)a.chunks_pad) * sz;
    const size_t G = col_g(precision);
    return (2 * (size_t)a.line_pitch * G + 6 * (size_t)a.chunks_pad * G) * sz;
}

static int threads_of(int precision, const AxisLaunch &a)
{
    if (a.layout == 0)
        return a.lines_per_cta * 2 * a.chunks_pad;
    return 2 * col_g(precision) * a.chunks_pad;
}

AxisPlanLimits axis_limits(int precision, int T)
{
    // the longest extent a rows-layout CTA (one line) and a columns-layout CTA
    // (G lines) can hold; the plan uses the one of its layout
    AxisPlanLimits l;
    l.smem_limit = smem_limit();
    const int K = chunk_k(precision, T);
    int best_rows = 0, best_cols = 0;
    for (int lay = 0; lay < 2; lay++) {
        int lo = 1, hi = kMaxLineThreads * K;
        while (lo < hi) {
            int mid = (lo + hi + 1) / 2;
            AxisLaunch a{};
            a.layout = lay;
            a.lines_per_cta = 1;
            a.line_pitch = pitch_of(mid);
            int nch = (mid + K - 1) / K;
            int unit = lay == 0 ? 32 : 32 / col_g(precision);
            a.chunks_pad = (nch + unit - 1) / unit * unit;
            if (threads_of(precision, a) <= kMaxLineThreads && axis_smem_bytes(precision, a) <= l.smem_limit)
                lo = mid;
            else
                hi = mid - 1;
        }
        (lay == 0 ? best_rows : best_cols) = lo;
    }
    l.extent_max = best_rows;
    l.extent_max_cols = best_cols;
    return l;
}

bool axis_shape(int precision, AxisLaunch &a)
{
    const int K = chunk_k(precision, a.T);
    int64_t E = a.tile_len + 2 * (int64_t)a.halo;
    if (E > a.L)
        E = a.L;
    const int nch = (int)((E + K - 1) / K);
    const int unit = a.layout == 0 ? 32 : 32 / col_g(precision);
    a.chunks_pad = (nch + unit - 1) / unit * unit;
    a.extent_max = (int)E;
    a.line_pitch = pitch_of(E);
    if (a.layout == 1) {
        a.lines_per_cta = col_g(precision);
        return threads_of(precision, a) <= kMaxLineThreads && axis_smem_bytes(precision, a) <= smem_limit();
    }
    // rows: ~512 threads per CTA
    int nl = std::max(1, std::min<int>(std::max(1, 256 / a.chunks_pad), kMaxLineThreads / (2 * a.chunks_pad)));
    if (nl > a.nlines)
        nl = (int)a.nlines;
    for (; nl >= 1; nl--) {
        a.lines_per_cta = nl;
        if (axis_smem_bytes(precision, a) <= smem_limit() && threads_of(precision, a) <= kMaxLineThreads)
            return true;
    }
    return false;
}

template <typename Real, int K, int SD, int LAY>
static cudaError_t launch_one(const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st)
{
    const int prec = sizeof(Real) == 8 ? 0 : 1;
    const size_t smem = axis_smem_bytes(prec, a);
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_axis<Real, K, SD, LAY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem_limit());
        if (e != cudaSuccess)
            return e;
        configured = true;
    }
    const int64_t groups = a.layout == 0 ? (a.nlines + a.lines_per_cta - 1) / a.lines_per_cta
                                         : a.outer_count * a.xblocks;
    const int64_t blocks = groups * a.ntiles;
    k_axis<Real, K, SD, LAY><<<(unsigned)blocks, threads_of(prec, a), smem, st>>>(a, g, sv);
    return cudaGetLastError();
}

template <typename Real, int K>
static cudaError_t launch_k(int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st)
{
    if (a.layout == 1)
        return launch_one<Real, K, 0, 1>(a, g, sv, st);
    switch (sd) {
    case 0: return launch_one<Real, K, 0, 0>(a, g, sv, st);
    case 1: return launch_one<Real, K, 1, 0>(a, g, sv, st);
    case 2: return launch_one<Real, K, 2, 0>(a, g, sv, st);
    default: return launch_one<Real, K, 3, 0>(a, g, sv, st);
    }
}

cudaError_t launch_axis(int precision, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                        cudaStream_t st)
{
    const int sd = a.fill_splat ? g.dim : 0;
    if (a.layout == 1 && a.fill_splat)
        return cudaErrorInvalidValue;
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
    a.layout = 0;
    a.L = len;
    a.elem_stride = 1;
    a.nlines = nlines;
    a.tile_len = len;
    a.ntiles = 1;
    a.halo = 0;
    a.passes = passes;
    a.T = T;
    a.alpha = alpha;
    a.scaled = normalize ? 1 : 0;
    a.inv_norm = 1.0 / (2.0 * T + 1.0 + 2.0 * alpha);
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
