// fb_axis_impl.cuh -- the n-fold box-and-tail convolution along one grid axis
// (device code and launch templates; instantiated per precision in
// fb_axis_f32.cu / fb_axis_f64.cu, planned in fb_axis.cu).
//
// Replaces _convolve_tail_{1,2,3}d / _accumulate_tail_array
// (fastbarnes/interpolation.py:372-533) and, for the first axis, the splat of
// _inject_data_{1,2,3}d (:218-322); for the last axis it also applies the NaN
// mask (:420-430) and the quotient (vg / wg + offset) of :367.
//
// The value and the weight field travel together as one cell (v, w): a float2
// in the float32 form, whose two halves every pass updates with one packed
// instruction (add / fma .f32x2 via __fadd2_rn / __ffma2_rn), or a double2 in
// the float64 form.  Cells are
// interleaved the same way in HBM between axes.
//
// One CTA holds whole lines (or halo-extended tiles of long lines) in shared
// memory and runs all `passes` box passes there, so every grid point crosses
// HBM once per axis.  Rows layout (axis 0): lines_per_cta consecutive rows,
// line buffers [e].  Columns layout (axes 1, 2): G adjacent lines interleaved
// [e][G], G cells = 32 bytes, so one 32-byte sector of a grid row is one row of
// the CTA's buffer and loads / stores are plain 16-byte vector copies.
//
// Inside a pass every thread owns a chunk of K consecutive cells of one line.
// It starts from the exact window sums at both chunk ends (anchors, summed
// from per-chunk partial sums of the previous pass that lie entirely inside
// the window, so nothing cancels), slides forward over the first half of the
// chunk and backward over the second half, keeps the K outputs in registers,
// and writes them back in place after a barrier (the last pass of a columns
// launch stores them to HBM from registers instead).  K is odd, so the lanes
// of a warp (consecutive chunks) spread over all banks.  Narrow kernels sum
// every output directly from registers instead.
//
// Window semantics are the reference's (interpolation.py:500-523): out[k] =
// sum_{|d|<=T} in[k+d] + alpha * (in[k-T-1] + in[k+T+1]), in[] = 0 outside
// [0, L).  Inside a tile the region beyond the tile's input extent reads as 0
// too; the halo of passes*(T+1) cells absorbs that, and only the tile's own
// cells are stored.
#pragma once
#include <string.h>

#include <algorithm>

#include "fb_internal.cuh"
#include "fb_kernels.cuh"

namespace fbg {

// ---------------------------------------------------------------------------
// (v, w) cells and their arithmetic
// ---------------------------------------------------------------------------

template <typename Real>
struct CellOf;
template <>
struct CellOf<float> {
    using T = float2;
};
template <>
struct CellOf<double> {
    using T = double2;
};

// float32 pairs: the packed .f32x2 instructions through CUDA's intrinsics
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as one packed fma: b * -1 is exact, so the result is the rounded difference
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
// float64 pairs: adds, subtracts and products through the _rn intrinsics, so
// that the compiler never fuses a product into a following add (the splat's
// w * v + cell would otherwise become an fma in some kernels and not in others)
__device__ __forceinline__ double2 cadd(double2 a, double2 b)
{
    return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}
__device__ __forceinline__ double2 csub(double2 a, double2 b)
{
    return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y));
}
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c)
{
    return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y));
}

template <typename C>
__device__ __forceinline__ C czero();
template <>
__device__ __forceinline__ float2 czero<float2>() { return make_float2(0.f, 0.f); }
template <>
__device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }

template <typename C>
__device__ __forceinline__ C csplat(double x);
template <>
__device__ __forceinline__ float2 csplat<float2>(double x) { return make_float2((float)x, (float)x); }
template <>
__device__ __forceinline__ double2 csplat<double2>(double x) { return make_double2(x, x); }
// both halves from a value already in the cell's precision
template <typename C>
__device__ __forceinline__ C cpair(float x);
template <typename C>
__device__ __forceinline__ C cpair(double x);
template <>
__device__ __forceinline__ float2 cpair<float2>(float x) { return make_float2(x, x); }
template <>
__device__ __forceinline__ double2 cpair<double2>(double x) { return make_double2(x, x); }

// 16-byte asynchronous global -> shared copies (no registers held while the
// data is in flight, so a thread can have all of its copies outstanding)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Bulk copy of `bytes` (a multiple of 16) from shared to global memory, both
// addresses 16-byte aligned, by the tensor memory accelerator; the shared
// data was written by the CTA's threads before a barrier, so the issuing
// thread first orders those writes before the copy's reads (proxy fence).
__device__ __forceinline__ void bulk_store(void *gmem, const void *smem, unsigned bytes)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(gmem), "r"(s), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}
// Waits until the issuing thread's bulk copies have read their shared source.
__device__ __forceinline__ void bulk_store_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// mbarriers and bulk loads (tensor memory accelerator)
// ---------------------------------------------------------------------------

constexpr uint64_t kWaitLimitNs = 1000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t a, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase of parity `parity` to complete; false after
// kWaitLimitNs without completion.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity)
{
    if (mbar_try_wait(a, parity))
        return true;
    const uint64_t t0 = global_ns();
    for (uint32_t n = 1;; n++) {
        if (mbar_try_wait(a, parity))
            return true;
        if ((n & 63u) == 0u && global_ns() - t0 > kWaitLimitNs)
            return false;
    }
}

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to shared memory, completing on mbarrier `mbar`.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA) accesses of the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---------------------------------------------------------------------------
// one line seen by one thread: cell e lives at s[e * ES]; the line buffer has
// zero cells on both sides (T + 1 before the line, up to the end of the last
// chunk + T + 1 after it), so no read needs a bounds check
// ---------------------------------------------------------------------------

template <typename C, bool SCALED>
struct PassCoef {
    C alpha;   // tail weight (alpha * inv when scaled), both halves
    C inv;     // 1 / (2T+1+2alpha), both halves
    __device__ __forceinline__ C out(C acc, C tails) const
    {
        if (SCALED)
            return cfma(acc, inv, cmul(alpha, tails));
        return cfma(alpha, tails, acc);
    }
};

// Sliding passes move every thread's chunk by T + 1 cells, alternately to the
// left and back to the right, so that the window cells on one side of the new
// chunk are exactly the thread's own previous chunk, still in registers: a
// pass reads one cell per output from shared memory (the other side of the
// window) instead of two.  F grid: chunk j = [jK, jK + K); A grid: chunk j =
// [jK - T - 1, jK - T - 1 + K).  Even passes go F -> A ("left"), odd passes
// A -> F ("right").  Needs 2T + 1 >= K.
//
// Window sums (anchors) come from the previous pass's per-chunk sums S and
// one partial sum X of r = (2T + 1) mod K cells (the last r cells of an F
// chunk, the first r of an A chunk): whole pieces inside the window, nothing
// subtracted.  The thread slides forward from the anchor at its chunk start
// over the first half and backward from the one at its chunk end over the
// rest; the two halves are independent, so their steps are interleaved.
//
// Left pass: own previous chunk P = F chunk j at b = jK, outputs at
// a = b - T - 1; s[m] = cell b - 2T - 2 + m.  Output i: window
// [b + i - 2T - 1, b + i - 1], tails s[i] and P[i].
// A chunk wholly left of the line (a + K <= 0) would read below the buffer's
// zero cells; its reads are moved up to the buffer start (lo), and its
// outputs are cleared afterwards anyway.
template <typename C, int K, int ES, bool SCALED>
__device__ __forceinline__ void pass_left(const C *__restrict__ ln, int b, int T, int lo, C A0, C A1,
                                          const PassCoef<C, SCALED> &c, C (&o)[K])
{
    constexpr int H = K / 2;
    const C *s = ln + max(b - 2 * T - 2, lo) * ES;
    C af = A0, ab = A1;          // windows at a and a + K
    C prev = s[0];
    C nb = s[K * ES];
#pragma unroll
    for (int i = 0; i < H; i++) {
        // forward: output i, then the window moves to i + 1 (+P[i], -s[i+1])
        const C x = s[(i + 1) * ES];
        const C pf = o[i];
        o[i] = c.out(af, cadd(prev, pf));
        af = cadd(af, csub(pf, x));
        prev = x;
        // backward: the window moves to k (+s[k+1], -P[k]), then output k
        const int k = K - 1 - i;
        const C y = s[k * ES];
        const C pk = o[k];
        ab = cadd(ab, csub(nb, pk));
        o[k] = c.out(ab, cadd(y, pk));
        nb = y;
    }
    {
        const C y = s[H * ES];
        const C pk = o[H];
        ab = cadd(ab, csub(nb, pk));
        o[H] = c.out(ab, cadd(y, pk));
    }
}

// Right pass: own previous chunk P = A chunk j at b = jK - T - 1, outputs at
// a = b + T + 1 = jK; s[m] = cell b + 2T + 2 + m.  Output i: window
// [b + i + 1, b + i + 2T + 1], tails P[i] and s[i].  A0 is the window at a,
// A1 the one at a + K - 1.
// A chunk wholly right of the line (a >= E) reads as if it started at E - 1
// (inside the buffer's zero cells); its outputs are cleared afterwards.
template <typename C, int K, int ES, bool SCALED>
__device__ __forceinline__ void pass_right(const C *__restrict__ ln, int b, int T, int E, C A0, C A1,
                                           const PassCoef<C, SCALED> &c, C (&o)[K])
{
    constexpr int H = K / 2;
    const C *s = ln + (min(b + T + 1, E - 1) + T + 1) * ES;
    C af = A0, ab = A1;
    C hi = s[(K - 1) * ES];
#pragma unroll
    for (int i = 0; i < H; i++) {
        // forward: output i, then the window moves to i + 1 (+s[i], -P[i+1])
        const C x = s[i * ES];
        const C pf = o[i];
        o[i] = c.out(af, cadd(pf, x));
        af = cadd(af, csub(x, o[i + 1]));
        // backward: output k, then the window moves to k - 1 (+P[k], -s[k-1])
        const int k = K - 1 - i;
        const C pk = o[k];
        o[k] = c.out(ab, cadd(pk, hi));
        const C lo = s[(k - 1) * ES];
        ab = cadd(ab, csub(pk, lo));
        hi = lo;
    }
    o[H] = c.out(ab, cadd(o[H], hi));
}

// Narrow kernels (T <= DirectMax): every output is summed directly from the
// K + 2T + 2 inputs the chunk needs, held in registers.  Sliding a window of
// only a few cells over K/2 steps would carry the rounding error of large
// values that have already left the window.
template <typename C, int K, int ES, int TD, bool SCALED>
__device__ __forceinline__ void direct_pass(const C *__restrict__ s, int k0, const PassCoef<C, SCALED> &c, C (&o)[K])
{
    constexpr int NX = K + 2 * TD + 2;
    C x[NX];
    const C *lo = s + (k0 - TD - 1) * ES;
#pragma unroll
    for (int m = 0; m < NX; m++)
        x[m] = lo[m * ES];
#pragma unroll
    for (int i = 0; i < K; i++) {
        C acc = x[i + 1];
#pragma unroll
        for (int d = 2; d <= 2 * TD + 1; d++)
            acc = cadd(acc, x[i + d]);
        o[i] = c.out(acc, cadd(x[i], x[i + 2 * TD + 2]));
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

template <typename Real, typename C, int K, int ES, int TD, bool SCALED>
__device__ __forceinline__ void direct_dispatch(int T, const C *s, int k0, const PassCoef<C, SCALED> &c, C (&o)[K])
{
    if constexpr (TD <= DirectMax<Real>::T) {
        if (T != TD) {
            direct_dispatch<Real, C, K, ES, TD + 1, SCALED>(T, s, k0, c, o);
            return;
        }
        direct_pass<C, K, ES, TD, SCALED>(s, k0, c, o);
    }
}

// Pairwise sum of o[LO..HI) (zero for an empty range): a tree of depth
// log2(HI - LO), so the sums do not wait on a chain of dependent adds.
template <int LO, int HI, typename C, int K>
__device__ __forceinline__ C tree_sum(const C (&o)[K])
{
    if constexpr (HI <= LO) {
        return czero<C>();
    } else if constexpr (HI - LO == 1) {
        return o[LO];
    } else {
        constexpr int M = (LO + HI) / 2;
        return cadd(tree_sum<LO, M>(o), tree_sum<M, HI>(o));
    }
}

// The sums a chunk leaves for the next pass: S = o[0] + S1 with S1 the sum
// of o[1..K-1], and X = the first R cells (PRE) or the last R cells (suffix),
// each accumulated once over disjoint segments (pairwise).
template <typename C, int K, int R, bool PRE>
__device__ __forceinline__ void chunk_sums_fixed(const C (&o)[K], C &S, C &S1, C &X)
{
    constexpr int B = PRE ? (R > 0 ? R : 1) : (K - R > 1 ? K - R : 1);   // segment split inside [1, K)
    const C a = tree_sum<1, B>(o), z = tree_sum<B, K>(o);
    S1 = cadd(a, z);
    S = cadd(o[0], S1);
    if (PRE)
        X = R == 0 ? czero<C>() : cadd(o[0], a);       // o[0] + o[1..R-1]
    else
        X = R == 0 ? czero<C>() : (R == K ? S : z);    // o[K-R..K-1]
}

template <typename C, int K, bool PRE>
__device__ __forceinline__ void chunk_sums(const C (&o)[K], int r, C &S, C &S1, C &X)
{
#define FBG_CS(RR)                                                                                                  \
    case RR:                                                                                                        \
        if constexpr (RR < K)                                                                                       \
            chunk_sums_fixed<C, K, RR, PRE>(o, S, S1, X);                                                           \
        break;
    switch (r) {
        FBG_CS(0) FBG_CS(1) FBG_CS(2) FBG_CS(3) FBG_CS(4) FBG_CS(5) FBG_CS(6) FBG_CS(7) FBG_CS(8) FBG_CS(9)
        FBG_CS(10) FBG_CS(11) FBG_CS(12) FBG_CS(13) FBG_CS(14) FBG_CS(15) FBG_CS(16) FBG_CS(17) FBG_CS(18)
        FBG_CS(19) FBG_CS(20) FBG_CS(21) FBG_CS(22) FBG_CS(23) FBG_CS(24) FBG_CS(25) FBG_CS(26) FBG_CS(27)
        FBG_CS(28) FBG_CS(29) FBG_CS(30) FBG_CS(31) FBG_CS(32)
    default: break;
    }
#undef FBG_CS
}
static_assert(K32 <= 33 && K64 <= 33, "chunk_sums lists r up to 32");

// Outputs outside the line [0, E) are zero (the line's own zeros).
template <typename C, int K>
__device__ __forceinline__ void clip_chunk(C (&o)[K], int a, int E)
{
    if (a < 0 || a + K > E) {
#pragma unroll
        for (int i = 0; i < K; i++)
            if (a + i < 0 || a + i >= E)
                o[i] = czero<C>();
    }
}

// NaN where the weight is below the mask level, else vg / wg + offset
// (interpolation.py:428-430, :367); `offset` already in the form's precision.
// The float32 form divides with __fdividef (within 2 ulp; the weights stay
// far below its 2^126 limit: unscaled sums are capped at 1e24 by the plan).
__device__ __forceinline__ double quotient_div(double v, double w) { return v / w; }
__device__ __forceinline__ float quotient_div(float v, float w) { return __fdividef(v, w); }

// Drops the `nbits` least significant bits of a float64 mantissa, rounding the
// kept part the way the reference's demo does (demo/quantization.py:23-37:
// int(m * 2^(53 - nbits) + 0.5), a truncation toward zero, then
// ldexp); NaN stays NaN.
__device__ __forceinline__ double quantize(double x, int nbits)
{
    if (nbits <= 0 || x != x)
        return x;
    const int sh = 53 - nbits;
    int e;
    const double m = frexp(x, &e);
    return ldexp(trunc(m * ldexp(1.0, sh) + 0.5), e - sh);
}

template <typename Real>
__device__ __forceinline__ Real quotient(Real v, Real w, Real thr, Real offset)
{
    const Real nan = sizeof(Real) == 8 ? (Real)__longlong_as_double(0x7ff8000000000000ll)
                                       : (Real)__int_as_float(0x7fc00000);
    return (w < thr) ? nan : quotient_div(v, w) + offset;
}

// ---------------------------------------------------------------------------
// the splat (first axis, rows layout)
// ---------------------------------------------------------------------------

// One staged sample of one line: lower x cell, x offset, the line's row
// weights (wy, wz of the reference's corner products) and the centred value.
template <typename Real>
struct StageRec {
    int32_t xi;
    Real xw, wy, wz, v;
};
constexpr int kStage = 128;   // records staged per line per round

// Sorted-sample ranges feeding one line (at most two, 3D).
struct LineRanges {
    uint32_t b[2], e[2];
    int n;
};

template <int DIM>
__device__ __forceinline__ LineRanges line_ranges(int64_t line, int64_t e0, int E, const Geometry &g,
                                                  const SampleView &sv, const uint32_t *__restrict__ bin_start)
{
    LineRanges r;
    r.n = 0;
    if (DIM == 1) {
        const int64_t lo = e0 >= 1 ? e0 - 1 : 0;
        const int64_t hi = e0 + E - 1;
        int64_t b0 = lo / sv.bin_w, b1 = hi / sv.bin_w;
        if (b1 > (int64_t)sv.nbins - 1)
            b1 = (int64_t)sv.nbins - 1;
        if (b0 <= b1) {
            r.b[0] = bin_start[b0];
            r.e[0] = bin_start[b1 + 1];
            r.n = 1;
        }
    } else if (DIM == 2) {
        // samples whose lower corner row is line - 1 or line, in that order
        const int64_t b0 = line >= 1 ? line - 1 : line;
        r.b[0] = bin_start[b0];
        r.e[0] = bin_start[line + 1];
        r.n = 1;
    } else {
        const int64_t H = g.size[1];
        const int64_t z = line / H, y = line % H;
        for (int dz = 1; dz >= 0; dz--) {
            if (z - dz < 0)
                continue;
            const int64_t rb = (z - dz) * H;
            const int64_t b0 = y >= 1 ? rb + y - 1 : rb + y;
            r.b[r.n] = bin_start[b0];
            r.e[r.n] = bin_start[rb + y + 1];
            r.n++;
        }
    }
    return r;
}

// Position `pos` of the concatenated ranges -> sorted position.
__device__ __forceinline__ uint32_t range_at(const LineRanges &r, uint32_t pos)
{
    const uint32_t n0 = r.n > 0 ? r.e[0] - r.b[0] : 0u;
    return pos < n0 ? r.b[0] + pos : r.b[1] + (pos - n0);
}

__device__ __forceinline__ uint32_t range_total(const LineRanges &r)
{
    uint32_t t = 0;
    for (int q = 0; q < r.n; q++)
        t += r.e[q] - r.b[q];
    return t;
}

// The staged form of one sample for one line: (1 - yw) if the line is the
// sample's lower row, yw if it is the upper one (likewise in z).
template <int DIM, typename Real>
__device__ __forceinline__ StageRec<Real> make_stage(const SampleRec<Real> &r, int64_t line, const Geometry &g,
                                                     double offset)
{
    StageRec<Real> s;
    s.xi = r.xi;
    s.xw = r.xw;
    s.v = (Real)(r.val - offset);
    s.wy = (Real)1;
    s.wz = (Real)1;
    if (DIM == 2) {
        s.wy = (r.yi == line) ? ((Real)1 - r.yw) : r.yw;
    } else if (DIM == 3) {
        const int64_t zl = line / g.size[1], yl = line % g.size[1];
        s.wy = (r.yi == yl) ? ((Real)1 - r.yw) : r.yw;
        s.wz = (r.zi == zl) ? ((Real)1 - r.zw) : r.zw;
    }
    return s;
}

// Adds `cnt` staged records to one line, in order.  Lanes take 32 consecutive
// records; lanes hitting the same cell add one after the other in lane order,
// so the result does not depend on scheduling.
template <typename Real, typename C, int DIM>
__device__ void apply_recs(C *__restrict__ line, int E, int64_t e0, const StageRec<Real> *__restrict__ rec, int cnt,
                           int lane)
{
    const uint32_t lt = (1u << lane) - 1u;
    for (int r = 0; r < cnt; r += 32) {
        const bool valid = r + lane < cnt;
        StageRec<Real> rc;
        rc.xi = 0;
        rc.xw = rc.wy = rc.wz = rc.v = (Real)0;
        if (valid)
            rc = rec[r + lane];
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const int64_t ec = (int64_t)rc.xi + c - e0;
            const bool ok = valid && ec >= 0 && ec < E;
            if (__ballot_sync(0xffffffffu, ok) == 0u)
                continue;
            // corner weight (wx * wy) * wz, the reference's product order
            const Real wx = c ? rc.xw : ((Real)1 - rc.xw);
            Real w = wx;
            if (DIM >= 2)
                w = wx * rc.wy;
            if (DIM == 3)
                w = w * rc.wz;
            C add;
            add.x = w * rc.v;
            add.y = w;
            const int key = ok ? (int)ec : -1 - lane;
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            const int rank = __popc(peers & lt);
            const int maxc = __reduce_max_sync(0xffffffffu, ok ? __popc(peers) : 0);
            for (int q = 0; q < maxc; q++) {
                if (ok && rank == q)
                    line[ec] = cadd(line[ec], add);
                __syncwarp();
            }
        }
    }
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------

// Stores one thread's final chunk of a column (cells a0 .. a0 + K - 1 of the
// tile, HBM cell gb + cell * elem_stride), the tile's own cells [s0, s1) only:
// the quotient (float32 or float64 result) on the last axis, else the cell.
template <typename Real, typename C, int K>
__device__ __forceinline__ void store_chunk_columns(const AxisLaunch &a, const TilePtrs &fp, int64_t gb, int a0,
                                                    int s0, int s1, Real thr, Real offs, const C (&o)[K])
{
    // One pointer stepped by the row stride (no 64-bit multiply per cell).
    // (A path without the range test for chunks wholly inside [s0, s1),
    // chosen per warp, measured slower.)
    const int64_t es = a.elem_stride;
    if (!a.store_quot) {
        C *d_ = reinterpret_cast<C *>(fp.dst) + gb + (int64_t)a0 * es;
#pragma unroll
        for (int i = 0; i < K; i++, d_ += es)
            if (a0 + i >= s0 && a0 + i < s1)
                *d_ = o[i];
    } else if (a.out_f64) {
        double *d_ = reinterpret_cast<double *>(fp.out) + gb + (int64_t)a0 * es;
#pragma unroll
        for (int i = 0; i < K; i++, d_ += es)
            if (a0 + i >= s0 && a0 + i < s1)
                *d_ = (double)quotient<Real>(o[i].x, o[i].y, thr, offs);
    } else {
        float *d_ = reinterpret_cast<float *>(fp.out) + gb + (int64_t)a0 * es;
#pragma unroll
        for (int i = 0; i < K; i++, d_ += es)
            if (a0 + i >= s0 && a0 + i < s1)
                *d_ = (float)quotient<Real>(o[i].x, o[i].y, thr, offs);
    }
}

// Column-layout group: G adjacent lines, B bytes of each grid row, V 16-byte
// vectors a row.
template <typename C>
struct ColG {
    static constexpr int B = sizeof(C) == 8 ? kColBytesF32 : kColBytesF64;
    static constexpr int G = B / (int)sizeof(C);
    static constexpr int V = B / 16;
};

// SPLAT_DIM: 0 = the lines are loaded from src, 1..3 = they are filled by
// splatting the samples of a field of that dimension (rows layout).
// LAYOUT: 0 = rows, 1 = columns.  K: chunk length (odd).
// MODE: 0 = sliding windows, 1 = direct sums (narrow kernels).
// One tile of one launch: line group `group`, tile `tile` along the lines.
template <typename Real, int K, int MODE, int SPLAT_DIM, int LAYOUT>
__device__ __forceinline__ void axis_tile(const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                                          const TilePtrs &fp, int64_t group, int64_t tile, unsigned char *smem_raw)
{
    using C = typename CellOf<Real>::T;
    constexpr int G = LAYOUT == 0 ? 1 : ColG<C>::G;
    constexpr int ES = G;   // cell stride inside a line buffer
    constexpr int PS = G;   // chunk stride inside a partials array
    C *cells = reinterpret_cast<C *>(smem_raw);
    const int P = a.line_pitch;    // cells per line slot, zero pads included
    const int HP = a.line_pad;     // zero cells before cell 0 of a line
    const int CP = a.chunks_pad;
    const int PP = a.part_pitch;   // partial-sum slots per line, zero pads included
    const int PF = a.part_pad;     // zero slots before chunk 0
    const int NLC = LAYOUT == 0 ? a.lines_per_cta : G;   // line slots in this CTA
    C *part = cells + (size_t)NLC * P;                    // [3][NLC][PP] (rows) / [3][PP][G] (columns)
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;

    const int64_t t0 = tile * a.tile_len;
    const int64_t t1 = min(a.L, t0 + a.tile_len);
    const int64_t e0 = max((int64_t)0, t0 - (int64_t)a.halo);
    const int64_t e1 = min(a.L, t1 + (int64_t)a.halo);
    const int E = (int)(e1 - e0);
    const int nch = (E + K - 1) / K;

    // lines of this CTA and their HBM position (cell e0 of the line)
    int nl;                  // lines present
    int64_t line0 = 0;       // rows: first line index
    int64_t gbase = 0;       // columns: HBM cell index of (line 0 of the group, cell e0)
    bool vec_ok = false;     // columns: the group's rows are whole aligned 32-byte segments
    if (LAYOUT == 0) {
        line0 = group * a.lines_per_cta;
        nl = (int)min((int64_t)a.lines_per_cta, a.nlines - line0);
    } else {
        const uint32_t o32 = (uint32_t)group / (uint32_t)a.xblocks;
        const int64_t o = o32, xb = group - o * a.xblocks;
        nl = (int)min((int64_t)G, a.width - xb * G);
        gbase = o * a.outer_stride + xb * G + e0 * a.elem_stride;
        vec_ok = nl == G && (gbase % G) == 0 && (a.elem_stride % G) == 0;
    }

    // this thread's line / chunk
    int li, j;
    C *ln;
    const C *pp0;
    int QS;
    if (LAYOUT == 0) {
        li = NLC == 1 ? 0 : tid / CP;
        j = tid - li * CP;
        ln = cells + (size_t)li * P + HP;
        QS = NLC * PP;
        pp0 = part + (size_t)li * PP + PF;
    } else {
        j = tid / G;
        li = tid - j * G;
        ln = cells + (size_t)HP * G + li;
        QS = PP * G;
        pp0 = part + (size_t)PF * G + li;
    }
    C *pw = const_cast<C *>(pp0) + (size_t)j * PS;   // this chunk's S slot
    const int T = a.T;
    // sliding passes need the chunks of both grids that touch [0, E)
    const int nact = MODE == 1 ? nch : (E + T + 1 + K - 1) / K;
    bool active = li < nl && j < nact;
    const int q = (2 * T + 1) / K, r = (2 * T + 1) - q * K;
    // bounds-check build: every pass window of this thread inside the buffers
    if (kBoundsCheck && active)
        active = bounds_ok(pass_windows_in(j, K, T, E, HP, P, PP, PF, q, MODE == 1),
                           fp.hdr ? &fp.hdr->error : nullptr);
    // The loads that nothing else waits for go first -- a columns launch's
    // cell rows (asynchronous copies) and a splat's bin starts -- then the
    // field's offset (thread 0) and the zeroing of the buffers run while
    // they are in flight, and one barrier publishes it all.
    const C *csrc = reinterpret_cast<const C *>(fp.src) + gbase;
    const int64_t es = a.elem_stride;
    C *dcell = cells + (size_t)HP * G;
    if (LAYOUT == 1 && SPLAT_DIM == 0 && vec_ok) {
        // V 16-byte asynchronous copies per row of G cells
        constexpr int V = ColG<C>::V;
        const int nv = V * E;
        uint4 *d_ = reinterpret_cast<uint4 *>(dcell);
        for (int i = tid; i < nv; i += nthr) {
            const int row = i / V, h = i - row * V;
            cp_async16(d_ + i, reinterpret_cast<const char *>(csrc + row * es) + 16 * h);
        }
    }
    LineRanges rg;
    rg.n = 0;
    uint32_t total = 0;
    __shared__ uint32_t s_tot[16];   // splat: records of each line of the CTA (at most 16 lines)
    if (SPLAT_DIM != 0 && li < nl) {
        rg = line_ranges<SPLAT_DIM>(line0 + li, e0, E, g, sv, fp.bin_start);
        total = range_total(rg);
    }
    // The field's offset and the float32 form's scalar parameters are
    // computed once per CTA: float64 instructions (including conversions to
    // float32) are scarce, and every thread needs them.
    __shared__ double s_offset;
    __shared__ Real s_par[5];   // alpha, alpha * inv_norm, inv_norm, thr, offset in the form's precision
    if (tid == 0) {
        const double off = (SPLAT_DIM != 0 || a.store_quot) ? field_offset(fp.hdr) : 0.0;
        s_offset = off;
        s_par[0] = (Real)a.alpha;
        s_par[1] = (Real)(a.alpha * a.inv_norm);
        s_par[2] = (Real)a.inv_norm;
        s_par[3] = (Real)a.thr;
        s_par[4] = (Real)off;
    }
    {
        // partial sums start at zero (their pad slots stay zero)
        float4 *z4 = reinterpret_cast<float4 *>(part);
        const int n4 = (int)((size_t)2 * QS * sizeof(C) / 16);
        for (int i = tid; i < n4; i += nthr)
            z4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (SPLAT_DIM != 0) {
        // zero the line buffers
        float4 *z4 = reinterpret_cast<float4 *>(cells);
        const int n4 = (int)((size_t)NLC * P * sizeof(C) / 16);
        for (int i = tid; i < n4; i += nthr)
            z4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (li < nl && j == 0)
            s_tot[li] = total;
    } else if (LAYOUT == 1) {
        // zero pad rows before and after the lines (V 16-byte vectors a row)
        constexpr int V = ColG<C>::V;
        uint4 *z = reinterpret_cast<uint4 *>(cells);
        const int back = P - HP - E;
        for (int i = tid; i < V * (HP + back); i += nthr) {
            const int r = i / V;
            z[V * (r < HP ? r : HP + E + (r - HP)) + (i - r * V)] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    __syncthreads();
    const double offset = s_offset;
    const int s0 = (int)(t0 - e0), s1 = (int)(t1 - e0);   // this tile's own cells
    const Real thr = s_par[3];
    const Real offs = s_par[4];
    // Columns: the last pass stores its outputs from registers (no
    // write-back, barrier and read of the line buffer).  Loads stay
    // asynchronous copies: chunk-wise loads into registers were slower.
    const bool dio = LAYOUT == 1 && SPLAT_DIM == 0 && a.passes > 0 && a.quant_bits <= 0;

    // ---- fill -------------------------------------------------------------
    if constexpr (SPLAT_DIM != 0) {
        // stage each line's samples with all of the line's threads, then the
        // line's first warp adds them in order
        StageRec<Real> *stage = reinterpret_cast<StageRec<Real> *>(part + (size_t)2 * QS);
        const SampleRec<Real> *recs = reinterpret_cast<const SampleRec<Real> *>(sv.rec);
        uint32_t most = 0;
        for (int q = 0; q < nl; q++)
            most = max(most, s_tot[q]);
        const uint32_t rounds = (most + kStage - 1) / kStage;
        StageRec<Real> *my_stage = stage + (size_t)li * kStage;
        for (uint32_t rr = 0; rr < rounds; rr++) {
            const uint32_t base = rr * kStage;
            if (li < nl) {
                for (int q = j; q < kStage; q += CP) {
                    const uint32_t pos = base + q;
                    if (pos < total) {
                        const uint32_t idx = range_at(rg, pos);
                        if (bounds_ok(idx < (uint64_t)sv.npts, &fp.hdr->error))
                            my_stage[q] = make_stage<SPLAT_DIM, Real>(recs[idx], line0 + li, g, offset);
                    }
                }
            }
            __syncthreads();
            if (li < nl && j < 32 && base < total)
                apply_recs<Real, C, SPLAT_DIM>(ln, E, e0, my_stage, (int)min((uint32_t)kStage, total - base), j);
            __syncthreads();
        }
    } else if (LAYOUT == 0) {
        // zero pads on both sides of every line, then the lines
        const int back = P - HP - E;
        for (int q = 0; q < nl; q++) {
            C *sl = cells + (size_t)q * P;
            for (int e = tid; e < HP + back; e += nthr)
                sl[e < HP ? e : HP + E + (e - HP)] = czero<C>();
        }
        if (a.plain) {
            // single-field lines: the value half only
            const Real *src = reinterpret_cast<const Real *>(fp.src);
            for (int q = 0; q < nl; q++) {
                const Real *s_ = src + (line0 + q) * a.L + e0;
                C *d_ = cells + (size_t)q * P + HP;
                for (int e = tid; e < E; e += nthr) {
                    C c = czero<C>();
                    c.x = s_[e];
                    d_[e] = c;
                }
            }
        } else {
            const C *src = reinterpret_cast<const C *>(fp.src);
            for (int q = 0; q < nl; q++) {
                const C *s_ = src + (line0 + q) * a.L + e0;
                C *d_ = cells + (size_t)q * P + HP;
                for (int e = tid; e < E; e += nthr)
                    d_[e] = s_[e];
            }
        }
    } else {
        if (vec_ok) {
            cp_async_wait_all();
        } else {
            for (int i = tid; i < E * G; i += nthr) {
                const int row = i / G, gg = i - row * G;
                dcell[i] = gg < nl ? csrc[row * es + gg] : czero<C>();
            }
        }
    }
    __syncthreads();

    // ---- passes -----------------------------------------------------------
    PassCoef<C, false> cu;
    cu.alpha = cpair<C>(s_par[0]);
    cu.inv = cpair<C>((Real)1);
    PassCoef<C, true> cs;
    cs.alpha = cpair<C>(s_par[1]);
    cs.inv = cpair<C>(s_par[2]);

    if constexpr (MODE == 1) {
        // direct sums, F grid every pass
        for (int pass = 0; pass < a.passes; pass++) {
            __syncthreads();
            C o[K];
            const int k0 = j * K;
            if (active) {
                if (a.scaled)
                    direct_dispatch<Real, C, K, ES, 0, true>(T, ln, k0, cs, o);
                else
                    direct_dispatch<Real, C, K, ES, 0, false>(T, ln, k0, cu, o);
            }
            if (dio && pass + 1 == a.passes) {
                if (active)
                    store_chunk_columns<Real, C, K>(a, fp, gbase + li, k0, s0, s1, thr, offs, o);
                break;
            }
            // per-cell checks only in warps holding the line's last chunk
            const bool edge_warp = __any_sync(0xffffffffu, active && k0 + K > E);
            __syncthreads();
            if (active) {
                if (!edge_warp) {
#pragma unroll
                    for (int i = 0; i < K; i++)
                        ln[(k0 + i) * ES] = o[i];
                } else {
#pragma unroll
                    for (int i = 0; i < K; i++)
                        if (k0 + i < E)
                            ln[(k0 + i) * ES] = o[i];
                }
            }
        }
    } else {
        // the thread's chunk lives in o[] from pass to pass
        C o[K];
        C own_s = czero<C>(), own_s1 = czero<C>();
        if (active) {
            const int b = j * K;   // F chunk of the filled line (zero cells past E)
#pragma unroll
            for (int i = 0; i < K; i++)
                o[i] = ln[(b + i) * ES];
            C X;
            chunk_sums<C, K, false>(o, r, own_s, own_s1, X);
            pw[0] = own_s;
            pw[QS] = X;
        }
        const C *pS = pp0;
        const C *pX = pp0 + QS;
        for (int pass = 0; pass < a.passes; pass++) {
            __syncthreads();
            const bool left = (pass & 1) == 0;
            const bool more = pass + 1 < a.passes;
            const int a0 = left ? j * K - T - 1 : j * K;   // this pass's chunk
            // Chunks reaching outside the line need per-cell clearing and
            // stores; decided per warp (a uniform branch), so that warps
            // without such a chunk skip the checks altogether.
            const bool edge_warp = __any_sync(0xffffffffu, active && (a0 < 0 || a0 + K > E));
            C X = czero<C>();
            if (active) {
                C mid = czero<C>();
                if (left) {
                    for (int m = 1; m < q; m++)
                        mid = cadd(mid, pS[(j - m) * PS]);
                    const C A0 = cadd(cadd(pX[(j - q - 1) * PS], pS[(j - q) * PS]), mid);
                    const C A1 = cadd(cadd(pX[(j - q) * PS], mid), own_s);
                    const int b = j * K;
                    if (a.scaled)
                        pass_left<C, K, ES, true>(ln, b, T, -HP, A0, A1, cs, o);
                    else
                        pass_left<C, K, ES, false>(ln, b, T, -HP, A0, A1, cu, o);
                } else {
                    for (int m = 1; m < q; m++)
                        mid = cadd(mid, pS[(j + m) * PS]);
                    const int b = j * K - T - 1;
                    // cell b + qK + r = jK + T (moved inside the buffer for a
                    // chunk wholly right of the line, like its other reads)
                    const C A0 = cadd(cadd(cadd(own_s1, mid), pX[(j + q) * PS]), ln[(min(j * K, E - 1) + T) * ES]);
                    const C A1 = cadd(cadd(mid, pS[(j + q) * PS]), pX[(j + q + 1) * PS]);
                    if (a.scaled)
                        pass_right<C, K, ES, true>(ln, b, T, E, A0, A1, cs, o);
                    else
                        pass_right<C, K, ES, false>(ln, b, T, E, A0, A1, cu, o);
                }
                if (edge_warp)
                    clip_chunk(o, a0, E);
                if (more) {
                    // the next pass goes the other way: it needs the first r
                    // cells of an A chunk, the last r of an F chunk
                    if (left)
                        chunk_sums<C, K, true>(o, r, own_s, own_s1, X);
                    else
                        chunk_sums<C, K, false>(o, r, own_s, own_s1, X);
                }
            }
            if (dio && !more) {
                if (active)
                    store_chunk_columns<Real, C, K>(a, fp, gbase + li, a0, s0, s1, thr, offs, o);
                break;
            }
            __syncthreads();
            if (active) {
                // Unchecked: outputs outside [0, E) were cleared above, and
                // every chunk position, -(T + 1) .. nact * K - 1, lies inside
                // the line buffer (its zero pads), so writing those zeros
                // back keeps the pads zero.  (A checked write-back in the
                // warps holding edge chunks made every other warp wait for
                // them at the next barrier.)
#pragma unroll
                for (int i = 0; i < K; i++)
                    ln[(a0 + i) * ES] = o[i];
                if (more) {
                    pw[0] = own_s;
                    pw[QS] = X;
                }
            }
        }
    }
    if (dio)
        return;   // stored from registers by the last pass
    __syncthreads();

    // ---- store ------------------------------------------------------------
    if (LAYOUT == 0) {
        for (int q = 0; q < nl; q++) {
            const C *c_ = cells + (size_t)q * P + HP;
            const int64_t gb = (line0 + q) * a.L + e0;
            if (a.store_quot) {
                if (a.out_f64) {
                    double *o_ = reinterpret_cast<double *>(fp.out) + gb;
                    for (int e = s0 + tid; e < s1; e += nthr) {
                        const C c = c_[e];
                        o_[e] = quantize((double)quotient<Real>(c.x, c.y, thr, offs), a.quant_bits);
                    }
                } else {
                    float *o_ = reinterpret_cast<float *>(fp.out) + gb;
                    for (int e = s0 + tid; e < s1; e += nthr) {
                        const C c = c_[e];
                        o_[e] = (float)quotient<Real>(c.x, c.y, thr, offs);
                    }
                }
            } else if (a.plain) {
                Real *d_ = reinterpret_cast<Real *>(fp.dst) + gb;
                for (int e = s0 + tid; e < s1; e += nthr)
                    d_[e] = c_[e].x;
            } else {
                C *d_ = reinterpret_cast<C *>(fp.dst) + gb;
                if (sizeof(C) == 16 ||
                    (((gb + s0) & 1) == 0 && ((HP + s0) & 1) == 0 && ((s1 - s0) & 1) == 0)) {
                    // the line's cells as one bulk copy shared -> global
                    // (tensor memory accelerator), issued by one thread after
                    // the barrier above: both ends 16-byte aligned, a
                    // multiple of 16 bytes
                    if (tid == 0)
                        bulk_store(d_ + s0, c_ + s0, (unsigned)((s1 - s0) * sizeof(C)));
                } else if (sizeof(C) == 8 && ((gb + s0) & 1) == 0 && ((HP + s0) & 1) == 0) {
                    // pairs of float2 cells as 16-byte vectors
                    const int np = (s1 - s0) / 2;
                    const uint4 *sv4 = reinterpret_cast<const uint4 *>(c_ + s0);
                    uint4 *dv4 = reinterpret_cast<uint4 *>(d_ + s0);
                    for (int e = tid; e < np; e += nthr)
                        dv4[e] = sv4[e];
                    if (((s1 - s0) & 1) && tid == 0)
                        d_[s1 - 1] = c_[s1 - 1];
                } else {
                    for (int e = s0 + tid; e < s1; e += nthr)
                        d_[e] = c_[e];
                }
            }
        }
        // the line buffer must outlive the bulk copies' reads of it
        if (tid == 0)
            bulk_store_wait_read();
    } else {
        const int64_t es = a.elem_stride;
        const C *dcell = cells + (size_t)HP * G;
        if (a.store_quot) {
            // two threads per row, G/2 cells (16 bytes of shared memory) each,
            // so a warp reads 512 consecutive bytes
            constexpr int HG = G > 1 ? G / 2 : 1;
            const bool q_vec = HG == 2 && vec_ok && (gbase % 4) == 0 && (es % 4) == 0;
            for (int i = tid; i < 2 * (s1 - s0); i += nthr) {
                const int row = s0 + (i >> 1), u0 = (i & 1) * HG;
                Real q[HG];
#pragma unroll
                for (int u = 0; u < HG; u++) {
                    const C c = dcell[row * G + u0 + u];
                    q[u] = quotient<Real>(c.x, c.y, thr, offs);
                }
                const int64_t gi = gbase + row * es + u0;
                if (a.out_f64) {
                    double *o_ = reinterpret_cast<double *>(fp.out) + gi;
#pragma unroll
                    for (int u = 0; u < HG; u++)
                        if (u0 + u < nl)
                            o_[u] = quantize((double)q[u], a.quant_bits);
                } else if (q_vec) {
                    *reinterpret_cast<float2 *>(reinterpret_cast<float *>(fp.out) + gi) =
                        make_float2((float)q[0], (float)q[1 % HG]);
                } else {
                    float *o_ = reinterpret_cast<float *>(fp.out) + gi;
#pragma unroll
                    for (int u = 0; u < HG; u++)
                        if (u0 + u < nl)
                            o_[u] = (float)q[u];
                }
            }
        } else {
            C *dst = reinterpret_cast<C *>(fp.dst) + gbase;
            if (vec_ok) {
                constexpr int V = ColG<C>::V;
                const int nv = V * (s1 - s0);
                const uint4 *s_ = reinterpret_cast<const uint4 *>(dcell + (size_t)s0 * G);
                for (int i = tid; i < nv; i += nthr) {
                    const int row = s0 + i / V, h = i % V;
                    *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(dst + row * es) + 16 * h) = s_[i];
                }
            } else {
                for (int i = tid; i < (s1 - s0) * G; i += nthr) {
                    const int row = s0 + i / G, gg = i % G;
                    if (gg < nl)
                        dst[row * es + gg] = dcell[row * G + gg];
                }
            }
        }
    }
}

// Registers per thread (launches have at most 512 threads).  Float32
// sliding passes with the short chunk fit in 64, so two 512-thread CTAs (or
// four of 256) can share an SM; with the long chunk, rows (and columns in
// 16-byte groups, 128-thread CTAs) fit in 96 without spilling (five CTAs an
// SM instead of four); the other variants (columns in 32-byte groups with
// the long chunk, float64 cells, direct sums) keep 128.
template <typename Real, int K, int MODE, int LAYOUT>
struct AxisRegs {
    static constexpr int value = (sizeof(Real) == 4 && MODE == 0 && K == K64)                  ? 64
                                 : (sizeof(Real) == 4 && MODE == 0 && K == K32 && (LAYOUT == 0 || kColBytesF32 <= 16))
                                     ? 96
                                     : 128;
};

// Block index -> (line group, tile along the lines); most launches have one
// tile a line, and the indices fit 32 bits (a 64-bit division costs every
// thread dozens of instructions).
__device__ __forceinline__ void split_block(uint32_t b, int64_t ntiles, int64_t &group, int64_t &tile)
{
    if (ntiles == 1) {
        group = b;
        tile = 0;
    } else {
        const uint32_t gq = b / (uint32_t)ntiles;
        group = gq;
        tile = b - gq * (uint32_t)ntiles;
    }
}

template <typename Real, int K, int MODE, int SPLAT_DIM, int LAYOUT>
__global__ void __maxnreg__((AxisRegs<Real, K, MODE, LAYOUT>::value))
    k_axis(const AxisLaunch a, const Geometry g, const SampleView sv)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int64_t group, tile;
    split_block(blockIdx.x, a.ntiles, group, tile);
    TilePtrs fp;
    fp.src = a.src_v;
    fp.dst = a.dst_v;
    fp.out = a.out;
    fp.bin_start = sv.bin_start;
    fp.hdr = sv.hdr;
    axis_tile<Real, K, MODE, SPLAT_DIM, LAYOUT>(a, g, sv, fp, group, tile, smem_raw);
}

// Batched form: fields of identical shape and parameters (one launch
// description in kernel parameters, one TilePtrs per field); grid (bpf,
// fields): block (x, y) is block x of field y (a one-dimensional grid of
// bpf x fields blocks when there are more fields than grid rows).
template <typename Real, int K, int MODE, int SPLAT_DIM, int LAYOUT>
__global__ void __maxnreg__((AxisRegs<Real, K, MODE, LAYOUT>::value))
    k_axis_batch(const AxisLaunch a, const Geometry g, const SampleView sv, const TilePtrs *__restrict__ fields,
                 uint32_t blocks_per_field)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint32_t f = blockIdx.y, b = blockIdx.x;
    if (gridDim.x != blocks_per_field) {
        f = blockIdx.x / blocks_per_field;
        b = blockIdx.x - f * blocks_per_field;
    }
    const TilePtrs fp = fields[f];
    int64_t group, tile;
    split_block(b, a.ntiles, group, tile);
    axis_tile<Real, K, MODE, SPLAT_DIM, LAYOUT>(a, g, sv, fp, group, tile, smem_raw);
}

// Mixed batched form: one launch for fields of different grids and
// parameters (same kernel variant).  Block x works on items[x] = (field,
// block of that field's launch); the field's description is copied to shared
// memory first.  Items are ordered largest field first.
template <typename Real, int K, int MODE, int SPLAT_DIM, int LAYOUT>
__global__ void __maxnreg__((AxisRegs<Real, K, MODE, LAYOUT>::value))
    k_axis_mixed(const MixedField *__restrict__ fields, const uint2 *__restrict__ items)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) MixedField s_f;
    static_assert(sizeof(MixedField) % 4 == 0, "field copy by words");
    const uint2 it = items[blockIdx.x];
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(fields + it.x);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&s_f);
        for (int w = threadIdx.x; w < (int)(sizeof(MixedField) / 4); w += blockDim.x)
            dst[w] = src[w];
    }
    __syncthreads();
    int64_t group, tile;
    split_block(it.y, s_f.a.ntiles, group, tile);
    axis_tile<Real, K, MODE, SPLAT_DIM, LAYOUT>(s_f.a, s_f.g, s_f.sv, s_f.fp, group, tile, smem_raw);
}

// ---------------------------------------------------------------------------
// launch templates
// ---------------------------------------------------------------------------

int axis_threads(int precision, const AxisLaunch &a);

template <typename Real, int K, int MODE, int SD, int LAY>
static cudaError_t launch_one(const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st)
{
    const int prec = sizeof(Real) == 8 ? 0 : 1;
    const size_t smem = axis_smem_bytes(prec, a);
    cudaError_t e = ensure_smem_attr((const void *)k_axis<Real, K, MODE, SD, LAY>);
    if (e != cudaSuccess)
        return e;
    const int64_t groups = a.layout == 0 ? (a.nlines + a.lines_per_cta - 1) / a.lines_per_cta
                                         : a.outer_count * a.xblocks;
    const int64_t blocks = groups * a.ntiles;
    k_axis<Real, K, MODE, SD, LAY><<<(unsigned)blocks, axis_threads(prec, a), smem, st>>>(a, g, sv);
    return cudaGetLastError();
}

template <typename Real, int K, int MODE>
static cudaError_t launch_k(int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st)
{
    if (a.layout == 1)
        return launch_one<Real, K, MODE, 0, 1>(a, g, sv, st);
    switch (sd) {
    case 0: return launch_one<Real, K, MODE, 0, 0>(a, g, sv, st);
    case 1: return launch_one<Real, K, MODE, 1, 0>(a, g, sv, st);
    case 2: return launch_one<Real, K, MODE, 2, 0>(a, g, sv, st);
    default: return launch_one<Real, K, MODE, 3, 0>(a, g, sv, st);
    }
}

template <typename Real, int K, int MODE, int SD, int LAY>
static cudaError_t launch_batch_one(int op, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                                    const TilePtrs *fields, uint32_t bpf, uint32_t nitems, int *grid, cudaStream_t st)
{
    const int prec = sizeof(Real) == 8 ? 0 : 1;
    const size_t smem = axis_smem_bytes(prec, a);
    const int threads = axis_threads(prec, a);
    if (op == 1) {
        if (*grid < 1)
            return cudaSuccess;
        const uint32_t nf = bpf > 0 ? nitems / bpf : 0;
        const dim3 grid2 = nf <= 65535u && nf * bpf == nitems ? dim3(bpf, nf) : dim3((unsigned)*grid);
        k_axis_batch<Real, K, MODE, SD, LAY><<<grid2, threads, smem, st>>>(a, g, sv, fields, bpf);
        return cudaGetLastError();
    }
    cudaError_t e = ensure_smem_attr((const void *)k_axis_batch<Real, K, MODE, SD, LAY>);
    if (e != cudaSuccess)
        return e;
    *grid = (int)nitems;
    return cudaSuccess;
}

template <typename Real, int K, int MODE, int SD, int LAY>
static cudaError_t launch_mixed_one(int op, const MixedField *fields, const uint2 *items, uint32_t nitems,
                                    size_t smem, int threads, cudaStream_t st)
{
    if (op == 1) {
        if (nitems < 1)
            return cudaSuccess;
        k_axis_mixed<Real, K, MODE, SD, LAY><<<nitems, threads, smem, st>>>(fields, items);
        return cudaGetLastError();
    }
    return ensure_smem_attr((const void *)k_axis_mixed<Real, K, MODE, SD, LAY>);
}

template <typename Real, int K, int MODE>
static cudaError_t launch_mixed_k(int op, int sd, int layout, const MixedField *fields, const uint2 *items,
                                  uint32_t nitems, size_t smem, int threads, cudaStream_t st)
{
#define FBG_M(SD, LAY) launch_mixed_one<Real, K, MODE, SD, LAY>(op, fields, items, nitems, smem, threads, st)
    if (layout == 1)
        return FBG_M(0, 1);
    switch (sd) {
    case 0: return FBG_M(0, 0);
    case 1: return FBG_M(1, 0);
    case 2: return FBG_M(2, 0);
    default: return FBG_M(3, 0);
    }
#undef FBG_M
}

template <typename Real, int K, int MODE>
static cudaError_t launch_batch_k(int op, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                                  const TilePtrs *fields, uint32_t bpf, uint32_t nitems, int *grid, cudaStream_t st)
{
#define FBG_B(SD, LAY) launch_batch_one<Real, K, MODE, SD, LAY>(op, a, g, sv, fields, bpf, nitems, grid, st)
    if (a.layout == 1)
        return FBG_B(0, 1);
    switch (sd) {
    case 0: return FBG_B(0, 0);
    case 1: return FBG_B(1, 0);
    case 2: return FBG_B(2, 0);
    default: return FBG_B(3, 0);
    }
#undef FBG_B
}

}  // namespace fbg
