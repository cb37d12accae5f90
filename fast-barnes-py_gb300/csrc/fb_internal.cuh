// fb_internal.cuh -- shared definitions of the GB300 fast-Barnes kernels.
//
// Data layout in HBM (one field):
//   samples  : pts[N][dim] float64 (x fastest), val[N] float64 -- caller owned
//   grid     : [z][y][x] row-major, x fastest, exactly the reference's
//              size[::-1] layout (fastbarnes/interpolation.py:337-339)
//   workspace: FieldHeader | bin keys | sort ping-pong | tile histograms |
//              bin starts | two intermediate value/weight field pairs
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace fbg {

// Chunk length of the line-pass kernels: odd, so that 32 lanes holding
// consecutive chunks of one line hit 32 different shared-memory banks.
constexpr int K32 = 33;   // float32-compensated form
constexpr int K64 = 17;   // float64 form (8-byte words: half-warp phases)
constexpr int K9 = 9;     // float64 sliding passes whose window 2T + 1 is shorter than 17

constexpr int kMaxLineThreads = 1024;

// Per-field scalars written on the device (min/max of the values, flags).
// All fields start at zero; the minimum is kept complemented so that an
// atomic maximum on a zeroed word computes it.
struct FieldHeader {
    unsigned long long vmin_key;   // complemented ordered-integer encoding of min(val)
    unsigned long long vmax_key;   // ordered-integer encoding of max(val)
    int nan_seen;                  // any NaN in val -> offset is NaN
    int error;                     // device-side error word (0 = ok)
    int pad[2];
};

// Ordered encoding of a double so that unsigned integer order == numeric order.
__host__ __device__ inline unsigned long long dbl_to_ordered(double x)
{
    unsigned long long u;
#ifdef __CUDA_ARCH__
    u = (unsigned long long)__double_as_longlong(x);
#else
    memcpy(&u, &x, 8);
#endif
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

__host__ __device__ inline double ordered_to_dbl(unsigned long long k)
{
    unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, 8);
    return x;
#endif
}

// offset = (min + max) / 2 as in _normalize_values (interpolation.py:204-212)
__device__ inline double field_offset(const FieldHeader *h)
{
    if (h->nan_seen)
        return __longlong_as_double(0x7ff8000000000000ll);
    return (ordered_to_dbl(~h->vmin_key) + ordered_to_dbl(h->vmax_key)) / 2.0;
}

// Float32-form cell coordinate t (>= 0 expected) split into the lower cell
// index and the offset inside the cell with integer operations on the bits of
// t (float64 instructions are scarce): t = 1.m * 2^e, index = the integer
// part of the 53-bit mantissa, offset = the 32 leading bits of the rest
// rounded to float32 (the correctly rounded offset but for ties decided by
// lower bits).  Returns false (sample skipped) for negative t (but not
// -0), NaN, infinities and t >= 2^31.
__device__ __forceinline__ bool split_cell(double t, int &ci, float &cw)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(t);
    if ((b >> 63) != 0ull)
        return (b << 1) == 0ull ? (ci = 0, cw = 0.f, true) : false;
    const int e = (int)(b >> 52) - 1023;   // sign bit is 0
    if (e >= 31)
        return false;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    if (e < 0) {
        ci = 0;
        // t = m * 2^(e - 52); its top 32 bits as an integer, scaled back
        cw = e < -95 ? 0.f : (float)(uint32_t)(m >> 21) * __int_as_float((e - 31 + 127) << 23);
        return true;
    }
    const int sh = 52 - e;   // fraction bits, 22..52
    ci = (int)(m >> sh);
    const unsigned long long fr = m & ((1ull << sh) - 1ull);   // offset * 2^sh
    if (fr == 0ull) {
        cw = 0.f;
        return true;
    }
    // the fraction's 32 leading bits (leading one at bit 31), then the scale
    const int lz = __clzll((long long)fr);
    const uint32_t top = (uint32_t)((fr << lz) >> 32);
    cw = (float)top * __int_as_float((32 - lz - sh + 127) << 23);
    return true;
}

// Float32-form cell coordinate of a sample with the reference's skip rule
// kept exact at the grid's upper edge: q = p - x0 (the reference's
// difference), t = q * inv (1 / step, a product instead of the reference's
// division).  A sample whose cell lands in the last valid cell or beyond
// (index >= size - 2, about one sample in size) is redone with the
// reference's division, so that xc >= size - 1 skips it exactly when the
// reference does (interpolation.py:249-252).  Returns false for a skipped
// sample.
__device__ __forceinline__ bool split_cell_edge(double q, double step, double inv, int64_t size, int &ci, float &cw)
{
    if (!split_cell(q * inv, ci, cw))
        return false;
    if ((int64_t)ci >= size - 2) {
        const double xc = q / step;
        if (!(xc >= 0.0))
            return false;
        ci = __double2int_rz(xc);
        if ((int64_t)ci >= size - 1)
            return false;
        cw = (float)(xc - (double)ci);
    }
    return true;
}

// Geometry and parameters of one interpolation, shared by all kernels.
struct Geometry {
    int dim;
    int64_t size[3];      // x, y, z extents (1 for missing axes)
    double x0[3], step[3];
    int T[3];             // half kernel size per axis
    double alpha[3];      // tail value per axis (0 for the plain method)
    int num_iter;
    double thr;           // NaN mask level on the unscaled weight field
};

// Cell coordinates of one sample, computed once by the bin-key kernel:
// lower-corner cell (xi, yi, zi), fractional offsets inside it and the raw
// value.  The float64 form keeps the reference's float64 offsets
// xc - int(xc) (interpolation.py:251-254); the float32 form stores them as
// float32.
template <typename Real>
struct SampleRec;
template <>
struct SampleRec<double> {
    int32_t xi, yi, zi, pad;
    double xw, yw, zw;
    double val;
};
template <>
struct SampleRec<float> {
    int32_t xi, yi, zi;
    float xw, yw, zw;
    double val;
};

// One 2D field of a batch, as the batched bin-key kernel sees it.
struct BatchKeyField {
    const double *pts;
    const double *val;
    int64_t npts;
    int64_t sample_offset;   // first global sample index of the field
    uint32_t bin_offset;     // first global bin (row) of the field
    uint32_t pad;
    double x0[2], step[2];
    double inv_step[2];      // 1 / step (float32 form: a product instead of a division)
    int64_t size[2];
};
// Samples a block of the batched key pass takes (256 threads, eight each):
// the 800k samples of eight 100k-sample fields are about one wave of blocks.
constexpr int kBatchKeysPerBlock = 2048;

// Bytes of each grid row that one columns-layout CTA holds (its G adjacent
// lines interleaved): the float32 form's and the float64 form's.
constexpr int kColBytesF32 = 32;
constexpr int kColBytesF64 = 32;

// Sorted-sample view handed to the splatting first-axis kernel.
struct SampleView {
    const void *rec;              // SampleRec<Real> in sorted order (by bin, then sample)
    int64_t npts;
    const uint32_t *sorted_idx;   // sample indices in the same order
    const uint32_t *bin_start;    // nbins + 1 offsets into rec / sorted_idx
    uint32_t nbins;
    int bin_w;                    // 1D only: cells per bin
    const FieldHeader *hdr;
};

// One launch of the line-pass kernel along one axis.
//
// Rows layout (axis 0): lines are grid rows, contiguous in HBM; a CTA takes
// lines_per_cta consecutive rows, each line buffer [e] in shared memory.
// Columns layout (axes 1, 2): a CTA takes G adjacent lines (adjacent x, same
// z for axis 1 / same y for axis 2), held interleaved [e][G] in shared memory,
// so that one 32-byte row segment in HBM is one 32-byte row in shared memory.
struct AxisLaunch {
    int axis;                 // 0 = x, 1 = y, 2 = z
    int layout;               // 0 = rows, 1 = columns
    int64_t L;                // line length
    int64_t elem_stride;      // HBM distance between consecutive cells of a line
    int64_t nlines;           // rows layout: lines along this axis
    int64_t outer_count;      // columns layout: planes (z for axis 1, y for axis 2)
    int64_t outer_stride;     // columns layout: HBM distance between planes
    int64_t xblocks;          // columns layout: groups of G lines per plane
    int64_t width;            // columns layout: lines per plane (grid nx)
    int lines_per_cta;        // rows: lines per CTA; columns: G
    int64_t tile_len;         // output positions per tile (== L if untiled)
    int64_t ntiles;           // tiles per line
    int halo;                 // extra input cells on each side of a tile
    int extent_max;           // largest shared-memory extent of one line
    int line_pitch;           // shared-memory cells reserved per line (zero pads included)
    int line_pad;             // zero cells before cell 0 of a line buffer (T + 1)
    int chunks_pad;           // chunk slots per line (threads per line and field)
    int part_pitch;           // partial-sum slots per line (zero pads included)
    int part_pad;             // zero partial slots before chunk 0 (ceil(T / K))
    int passes;               // box passes run in this launch
    int T;
    double alpha;
    int scaled;               // 1: every pass is multiplied by inv_norm
    double inv_norm;          // 1/(2T+1+2alpha)
    int fill_splat;           // 1: fill by splatting samples, 0: load from src
    int store_quot;           // 1: last axis -> quotient + mask + offset
    int out_f64;              // quotient output type: 1 = float64, 0 = float32
    int plain;                // rows layout: src / dst are single-field Real lines
    double thr;               // mask level in the units of the stored weights
    const void *src_v, *src_w;
    void *dst_v, *dst_w;
    void *out;
    int quant_bits;           // float64 quotient: mantissa bits to drop (0 = none)
    // planning choices (host side only)
    int kchunk;               // chunk length: 0 = automatic, 17 or 33
    int rows_threads;         // rows layout: target threads per CTA (0 = 256)
};

// The pointers that differ between the fields of a batched axis launch (the
// rest of the launch description is shared and lives in kernel parameters).
struct TilePtrs {
    const void *src;              // input (v, w) cells (or plain lines)
    void *dst;                    // output (v, w) cells (or plain lines)
    void *out;                    // quotient output
    const uint32_t *bin_start;    // sorted-sample bin starts of the field
    const FieldHeader *hdr;       // value range of the field
};

// One field of a mixed batched launch (fields of different grids and
// parameters sharing one kernel variant), read by the CTA from memory.
struct MixedField {
    AxisLaunch a;
    Geometry g;
    SampleView sv;
    TilePtrs fp;
};

// Device status word bits (FieldHeader::error of a field, or of the first
// field of a batch): set by kernels that stop early instead of waiting on.
constexpr uint32_t FB_DEVICE_TIMEOUT = 1u;   // a pipeline wait ran out
constexpr uint32_t FB_DEVICE_BOUNDS = 2u;    // bounds-check build: an out-of-range index was skipped

// Bounds-check build (compiled with -DFB_BOUNDS_CHECK): kernels check their
// shared- and global-memory index ranges before using them; an index out of
// range is not used and FB_DEVICE_BOUNDS is recorded in the status word.
// The checks compile away otherwise.
#ifdef FB_BOUNDS_CHECK
constexpr bool kBoundsCheck = true;
#else
constexpr bool kBoundsCheck = false;
#endif

__device__ __forceinline__ bool bounds_ok(bool ok, const void *status_word)
{
    if (!kBoundsCheck)
        return true;
    if (!ok && status_word)
        atomicOr(reinterpret_cast<unsigned int *>(const_cast<void *>(status_word)), FB_DEVICE_BOUNDS);
    return ok;
}

// Every line-buffer and partial-sum index the passes of one thread use
// (chunk j, chunk length K, half width T, line extent E; HP zero cells
// before cell 0 and P cells per line slot; PF / PP the same for the partial
// sums; q = (2T + 1) / K): the sliding passes read [jK - 2T - 2, ...) (left)
// and [min(jK, E - 1) + T, ...) (right) and write their chunks at jK - T - 1
// and jK; the direct sums read [jK - T - 1, jK + K + T + 1).  True when all
// of them lie inside the buffers.
__device__ __forceinline__ bool pass_windows_in(int j, int K, int T, int E, int HP, int P, int PP, int PF, int q,
                                                bool direct)
{
    const int lo = -HP, hi = P - HP;
    const int b = j * K;
    if (direct)
        return b - T - 1 >= lo && b + K + T + 1 <= hi;
    const int left_read = max(b - 2 * T - 2, lo);
    const int right_read = min(b, E - 1) + T;
    bool ok = left_read + K + 1 <= hi && b - T - 1 >= lo && b + K <= hi && right_read >= lo &&
              right_read + 1 + K <= hi;
    ok = ok && j - q - 1 >= -PF && j + q + 1 < PP - PF;
    return ok;
}

// Launch description of the pipelined columns kernel (fb_cols.cuh),
// host-computed.
struct ColsPipe {
    int L;               // cells per line = rows of a tile
    int line_pad;        // zero rows before row 0 of a stage (multiple of 4: 128-byte aligned boxes)
    int line_pitch;      // rows per stage buffer
    int chunks_pad;      // chunk slots per line
    int part_pad, part_pitch;
    int box_rows, nboxes;
    int axis;            // 1: the lines run along y; 2: along z
    int T, passes, scaled, store_quot, out_f64, quant_bits;
    double alpha, inv_norm, thr;
    uint32_t ntiles, tiles_per_field, xblocks;
    int64_t width;           // lines per plane (grid x extent)
    int64_t elem_stride;     // HBM cells between consecutive cells of a line
    int64_t outer_stride;    // HBM cells between planes
    uint32_t stage_bytes;    // one stage buffer (multiple of 128)
    uint32_t part_bytes;     // one group's two partial-sum arrays (multiple of 128)
    int nstages, ngroups, group_threads;
    uint32_t *status;        // device status word (or null)
    TilePtrs single;         // the field's pointers when `fields` is null (one field)
};

}  // namespace fbg
