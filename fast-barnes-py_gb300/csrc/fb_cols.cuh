// fb_cols.cuh -- the column passes (y and z axes) as a persistent, pipelined
// kernel: tensor-memory-accelerator (TMA) tile loads into a ring of shared
// memory stages, completion on mbarriers, and two independent consumer
// groups per CTA, so that the HBM reads of later column groups overlap the
// box passes of the current ones.
//
// Replaces, for whole lines (no tiling along the line), the columns layout of
// k_axis / k_axis_batch (fb_axis_impl.cuh): the reference's column loop of
// _convolve_tail_2d / _convolve_tail_3d (fastbarnes/interpolation.py:411-418,
// :449-472) over _accumulate_tail_array (:484-533), with the NaN mask
// (:420-430) and the quotient (:367) on the last axis.  The pass arithmetic
// is the same code as k_axis (pass_left / pass_right / direct sums, the same
// chunk partial sums and anchors, the same quotient), so both kernels give
// bitwise identical results.
//
// Work unit ("tile"): one column group -- G adjacent lines (32 bytes of every
// grid row) of one plane of one field, all L cells of each line.  Tiles are
// dealt round robin to the persistent CTAs (one per SM).  A CTA holds NS
// stage buffers and NG consumer groups (G x chunks threads each); its k-th
// tile goes to stage k % NS and group k % NG:
//   - a tile's load is one `full` mbarrier announcing the tile's bytes and
//     the tile's TMA box loads (boxes of up to 256 rows x 32 bytes from a 4D
//     tensor map over (x, y, z, field)); rows past the grid read as zero;
//   - the group waits on `full`, runs the n passes in place in the stage and
//     stores the last pass from registers (quotient or cells).  As soon as a
//     warp has finished its last reads of the stage it counts itself off on
//     a shared counter; the last warp of the group issues the load of tile
//     k + NS into the same stage (a tile of the other group when NS = 3,
//     NG = 2), so no warp waits for another to release a stage.
// The first NS loads are issued at kernel start.  The zero pads of every
// stage (T + 1 + K rows before the line, T + K after it) and of the
// partial-sum arrays are cleared once at kernel start: loads only write rows
// [0, L), and the passes write only zeros outside them.
//
// Every mbarrier wait is bounded (about one second of %globaltimer); a wait
// that runs out records FB_DEVICE_TIMEOUT in the launch's status word and
// the group stops.  A group decides together (a barrier with an AND
// reduction), so no thread is left waiting at a group barrier.  Before the
// CTA exits, its first thread waits (again bounded) for any load it issued
// that no group consumed.
#pragma once
#include <cuda.h>

#include "fb_axis_impl.cuh"

namespace fbg {

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint32_t mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(mbar)
        : "memory");
}

// Barrier of one consumer group (named barrier `id`, `n` threads).
__device__ __forceinline__ void group_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
// Group barrier that also returns the AND of every thread's `v`.
__device__ __forceinline__ bool group_all(int id, int n, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.b32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}

// Registers per thread.  The long float32 chunk and float64 cells take 128
// (two consumer groups of up to 256 threads: lines of up to 2065 cells with
// the long chunk); the short float32 chunk fits 96 (two groups of up to 320
// threads).  The planner checks threads x registers against the register
// file and falls back to one group when two do not fit.
template <typename Real, int K, int MODE>
struct ColsRegs {
    static constexpr int value = (sizeof(Real) == 4 && K == K64) ? 96 : 128;
};

// Issues the TMA loads of global tile t into stage buffer `dst0` (row 0 of
// the line), completing on mbarrier `full`.
__device__ __forceinline__ void cols_issue_tile(const ColsPipe &p, const CUtensorMap *map, uint32_t t, uint32_t dst0,
                                                uint32_t full, int G)
{
    const uint32_t f = t / p.tiles_per_field;
    const uint32_t rr = t - f * p.tiles_per_field;
    const uint32_t o = rr / p.xblocks;
    const uint32_t xb = rr - o * p.xblocks;
    mbar_expect_tx(full, (uint32_t)p.nboxes * (uint32_t)p.box_rows * 32u);
    const int c0 = (int)xb * 2 * G;
    for (int b = 0; b < p.nboxes; b++) {
        const int row = b * p.box_rows;
        if (p.axis == 1)
            tma_load_4d(dst0 + (uint32_t)row * 32u, map, c0, row, (int)o, (int)f, full);
        else
            tma_load_4d(dst0 + (uint32_t)row * 32u, map, c0, (int)o, row, (int)f, full);
    }
}

// Stores one thread's final chunk (cells a0 .. a0 + K - 1 of its line, HBM
// cell gb + cell * elem_stride), the line's cells [0, E) only: the quotient
// (float32 or float64, NaN-masked, optionally quantised) on the last axis,
// else the cells.  Chunks wholly inside the line skip the range test.
template <typename Real, typename C, int K>
__device__ __forceinline__ void cols_store_chunk(const ColsPipe &p, const TilePtrs &fp, int64_t gb, int a0, int E,
                                                 Real thr, Real offs, const C (&o)[K])
{
    const int64_t es = p.elem_stride;
    const bool inside = a0 >= 0 && a0 + K <= E;
    if (!p.store_quot) {
        C *d = reinterpret_cast<C *>(fp.dst) + gb + (int64_t)a0 * es;
        if (inside) {
#pragma unroll
            for (int i = 0; i < K; i++, d += es)
                *d = o[i];
        } else {
#pragma unroll
            for (int i = 0; i < K; i++, d += es)
                if (a0 + i >= 0 && a0 + i < E)
                    *d = o[i];
        }
    } else if (p.out_f64) {
        double *d = reinterpret_cast<double *>(fp.out) + gb + (int64_t)a0 * es;
#pragma unroll
        for (int i = 0; i < K; i++, d += es)
            if (inside || (a0 + i >= 0 && a0 + i < E))
                *d = quantize((double)quotient<Real>(o[i].x, o[i].y, thr, offs), p.quant_bits);
    } else {
        float *d = reinterpret_cast<float *>(fp.out) + gb + (int64_t)a0 * es;
        if (inside) {
#pragma unroll
            for (int i = 0; i < K; i++, d += es)
                *d = (float)quotient<Real>(o[i].x, o[i].y, thr, offs);
        } else {
#pragma unroll
            for (int i = 0; i < K; i++, d += es)
                if (a0 + i >= 0 && a0 + i < E)
                    *d = (float)quotient<Real>(o[i].x, o[i].y, thr, offs);
        }
    }
}

template <typename Real, int K, int MODE>
__global__ void __maxnreg__((ColsRegs<Real, K, MODE>::value))
    k_cols_pipe(const __grid_constant__ CUtensorMap tmap, const ColsPipe p, const TilePtrs *__restrict__ fields)
{
    using C = typename CellOf<Real>::T;
    constexpr int G = ColG<C>::G;
    static_assert(G * sizeof(C) == 32, "a tile row is 32 bytes");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // the field's pointers and offset per group, double-buffered by tile
    // parity: a group's first thread writes them for its next tile while the
    // group still works on (and stores) the current one
    __shared__ TilePtrs s_fp[2][2];
    __shared__ double s_off[2][2];
    __shared__ Real s_par[4];   // alpha, alpha * inv_norm, inv_norm, thr in the form's precision
    __shared__ uint32_t s_issued[4], s_used[4], s_rel[4];   // per stage: loads issued, tiles consumed, warps done

    const int tid = threadIdx.x;
    const int NG = p.ngroups, NS = p.nstages, GT = p.group_threads;
    // 128-byte aligned start, offset from the shared array itself (integer
    // arithmetic on its address would hide the address space from the
    // compiler and turn every line-buffer access into a generic one)
    unsigned char *base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    C *part0 = reinterpret_cast<C *>(base + (size_t)NS * p.stage_bytes);
    uint64_t *full = reinterpret_cast<uint64_t *>(base + (size_t)NS * p.stage_bytes + (size_t)NG * p.part_bytes);
    // this CTA's tiles: blockIdx.x + k * gridDim.x, k < nlocal
    const uint32_t nlocal = blockIdx.x < p.ntiles ? (p.ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0u;

    {
        // zero pads and partial sums once; the loads never touch the pads
        uint4 *z = reinterpret_cast<uint4 *>(base);
        const uint32_t n16 = (uint32_t)(((size_t)NS * p.stage_bytes + (size_t)NG * p.part_bytes) / 16);
        for (uint32_t i = tid; i < n16; i += blockDim.x)
            z[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    if (tid == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(smem_u32(full + s), 1u);
            s_issued[s] = 0u;
            s_used[s] = 0u;
            s_rel[s] = 0u;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_par[0] = (Real)p.alpha;
        s_par[1] = (Real)(p.alpha * p.inv_norm);
        s_par[2] = (Real)p.inv_norm;
        s_par[3] = (Real)p.thr;
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
        for (uint32_t k = 0; k < (uint32_t)NS && k < nlocal; k++) {
            cols_issue_tile(p, &tmap, blockIdx.x + k * gridDim.x,
                            smem_u32(base + (size_t)k * p.stage_bytes) + (uint32_t)p.line_pad * 32u,
                            smem_u32(full + k), G);
            s_issued[k] = 1u;
        }
    }

    // ---- consumer group g ----------------------------------------------------
    const int g = tid / GT, gt = tid - g * GT;
    const int bar_id = 1 + g;
    const uint32_t nwarps = (uint32_t)(GT / 32);
    C *part = part0 + (size_t)g * (p.part_bytes / sizeof(C));
    const int j = gt / G, li = gt - j * G;
    const int T = p.T;
    const int E = p.L;
    const int nact = MODE == 1 ? (E + K - 1) / K : (E + T + 1 + K - 1) / K;
    const int PP = p.part_pitch, PF = p.part_pad, HP = p.line_pad;
    const int QS = PP * G;
    const C *pp0 = part + (size_t)PF * G + li;
    C *pw = part + (size_t)(PF + j) * G + li;
    const int q = (2 * T + 1) / K, r = (2 * T + 1) - q * K;

    // The field's pointers and offset of a tile are fetched by the group's
    // first thread one tile ahead (two dependent global reads), so that the
    // group never waits for them at its tile barrier.
    auto fetch_field = [&](uint32_t tt, uint32_t slot) {
        const uint32_t f = tt / p.tiles_per_field;
        const TilePtrs fp = fields ? fields[f] : p.single;
        s_fp[g][slot] = fp;
        s_off[g][slot] = p.store_quot ? field_offset(fp.hdr) : 0.0;
    };
    const uint32_t t_first = blockIdx.x + (uint32_t)g * gridDim.x;
    if (gt == 0 && t_first < p.ntiles)
        fetch_field(t_first, 0u);
    uint32_t k = (uint32_t)g;
    for (uint32_t t = t_first; t < p.ntiles; t += (uint32_t)NG * gridDim.x, k += NG) {
        const uint32_t s = k % (uint32_t)NS;
        const bool ready = mbar_wait(smem_u32(full + s), (k / NS) & 1u);
        const uint32_t par = (k / (uint32_t)NG) & 1u;
        if (!group_all(bar_id, GT, ready)) {
            if (gt == 0 && p.status)
                atomicOr(p.status, FB_DEVICE_TIMEOUT);
            break;
        }
        if (gt == 0 && t + (uint32_t)NG * gridDim.x < p.ntiles)
            fetch_field(t + (uint32_t)NG * gridDim.x, par ^ 1u);   // read after the next tile barrier
        C *cells = reinterpret_cast<C *>(base + (size_t)s * p.stage_bytes) + (size_t)HP * G;
        C *ln = cells + li;
        const uint32_t xb = (t % p.tiles_per_field) % p.xblocks;
        bool active = j < nact && (int64_t)xb * G + li < p.width;
        // bounds-check build: every pass window of this thread inside the stage
        if (kBoundsCheck && active)
            active = bounds_ok(pass_windows_in(j, K, T, E, HP, p.line_pitch, PP, PF, q, MODE == 1) &&
                                   HP + p.nboxes * p.box_rows <= p.line_pitch,
                               p.status);
        C o_[K];
        int a_last = 0;   // first cell of the chunk the last pass produced

        if constexpr (MODE == 1) {
            const int k0 = j * K;
            for (int pass = 0; pass < p.passes; pass++) {
                if (pass > 0)
                    group_sync(bar_id, GT);
                if (active) {
                    if (p.scaled) {
                        PassCoef<C, true> cs;
                        cs.alpha = cpair<C>(s_par[1]);
                        cs.inv = cpair<C>(s_par[2]);
                        direct_dispatch<Real, C, K, G, 0, true>(T, ln, k0, cs, o_);
                    } else {
                        PassCoef<C, false> cu;
                        cu.alpha = cpair<C>(s_par[0]);
                        cu.inv = cpair<C>((Real)1);
                        direct_dispatch<Real, C, K, G, 0, false>(T, ln, k0, cu, o_);
                    }
                }
                if (pass + 1 == p.passes)
                    break;
                const bool edge_warp = __any_sync(0xffffffffu, active && k0 + K > E);
                group_sync(bar_id, GT);
                if (active) {
                    if (!edge_warp) {
#pragma unroll
                        for (int i = 0; i < K; i++)
                            ln[(k0 + i) * G] = o_[i];
                    } else {
#pragma unroll
                        for (int i = 0; i < K; i++)
                            if (k0 + i < E)
                                ln[(k0 + i) * G] = o_[i];
                    }
                }
                fence_proxy_async_smem();
            }
            a_last = k0;
        } else {
            C own_s = czero<C>(), own_s1 = czero<C>();
            if (active) {
                const int b = j * K;
#pragma unroll
                for (int i = 0; i < K; i++)
                    o_[i] = ln[(b + i) * G];
                C X;
                chunk_sums<C, K, false>(o_, r, own_s, own_s1, X);
                pw[0] = own_s;
                pw[QS] = X;
            }
            const C *pS = pp0;
            const C *pX = pp0 + QS;
            for (int pass = 0; pass < p.passes; pass++) {
                group_sync(bar_id, GT);
                const bool left = (pass & 1) == 0;
                const bool more = pass + 1 < p.passes;
                const int a0 = left ? j * K - T - 1 : j * K;
                const bool edge_warp = __any_sync(0xffffffffu, active && (a0 < 0 || a0 + K > E));
                C X = czero<C>();
                if (active) {
                    C mid = czero<C>();
                    if (left) {
                        for (int m = 1; m < q; m++)
                            mid = cadd(mid, pS[(j - m) * G]);
                        const C A0 = cadd(cadd(pX[(j - q - 1) * G], pS[(j - q) * G]), mid);
                        const C A1 = cadd(cadd(pX[(j - q) * G], mid), own_s);
                        const int b = j * K;
                        if (p.scaled) {
                            PassCoef<C, true> cs;
                            cs.alpha = cpair<C>(s_par[1]);
                            cs.inv = cpair<C>(s_par[2]);
                            pass_left<C, K, G, true>(ln, b, T, -HP, A0, A1, cs, o_);
                        } else {
                            PassCoef<C, false> cu;
                            cu.alpha = cpair<C>(s_par[0]);
                            cu.inv = cpair<C>((Real)1);
                            pass_left<C, K, G, false>(ln, b, T, -HP, A0, A1, cu, o_);
                        }
                    } else {
                        for (int m = 1; m < q; m++)
                            mid = cadd(mid, pS[(j + m) * G]);
                        const int b = j * K - T - 1;
                        const C A0 =
                            cadd(cadd(cadd(own_s1, mid), pX[(j + q) * G]), ln[(min(j * K, E - 1) + T) * G]);
                        const C A1 = cadd(cadd(mid, pS[(j + q) * G]), pX[(j + q + 1) * G]);
                        if (p.scaled) {
                            PassCoef<C, true> cs;
                            cs.alpha = cpair<C>(s_par[1]);
                            cs.inv = cpair<C>(s_par[2]);
                            pass_right<C, K, G, true>(ln, b, T, E, A0, A1, cs, o_);
                        } else {
                            PassCoef<C, false> cu;
                            cu.alpha = cpair<C>(s_par[0]);
                            cu.inv = cpair<C>((Real)1);
                            pass_right<C, K, G, false>(ln, b, T, E, A0, A1, cu, o_);
                        }
                    }
                    if (edge_warp)
                        clip_chunk(o_, a0, E);
                    if (more) {
                        if (left)
                            chunk_sums<C, K, true>(o_, r, own_s, own_s1, X);
                        else
                            chunk_sums<C, K, false>(o_, r, own_s, own_s1, X);
                    }
                }
                if (!more) {
                    a_last = a0;
                    break;
                }
                group_sync(bar_id, GT);
                if (active) {
                    // unchecked: outputs outside [0, E) are zero and every
                    // chunk position lies in the stage's zero pads
#pragma unroll
                    for (int i = 0; i < K; i++)
                        ln[(a0 + i) * G] = o_[i];
                    pw[0] = own_s;
                    pw[QS] = X;
                }
                fence_proxy_async_smem();
            }
        }

        // ---- release the stage: the last pass has read it ---------------------
        __syncwarp();
        if ((tid & 31) == 0) {
            __threadfence_block();
            if (atomicAdd(&s_rel[s], 1u) == nwarps - 1u) {
                // the group's last warp: every read of the stage is done
                __threadfence_block();
                s_rel[s] = 0u;
                s_used[s]++;
                if (k + (uint32_t)NS < nlocal) {
                    fence_proxy_async_smem();
                    cols_issue_tile(p, &tmap, t + (uint32_t)NS * gridDim.x,
                                    smem_u32(base + (size_t)s * p.stage_bytes) + (uint32_t)HP * 32u,
                                    smem_u32(full + s), G);
                    s_issued[s]++;
                }
            }
        }

        // ---- store the last pass from registers ---------------------------------
        if (active) {
            const uint32_t rr = t % p.tiles_per_field;
            const uint32_t o = rr / p.xblocks;
            const int64_t gb = (int64_t)o * p.outer_stride + (int64_t)xb * G + li;
            cols_store_chunk<Real, C, K>(p, s_fp[g][par], gb, a_last, E, s_par[3], (Real)s_off[g][par], o_);
        }
    }
    // a group that stopped on a timeout may leave loads in flight into this
    // CTA's stages: wait (bounded) for them before the CTA exits
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < NS; s++)
            if (s_issued[s] > s_used[s])
                mbar_wait(smem_u32(full + s), (s_issued[s] - 1u) & 1u);
    }
}

// Shared memory of a launch: stages, partial sums, mbarriers, 128 bytes of
// alignment slack.
inline size_t cols_pipe_smem(const ColsPipe &p)
{
    return (size_t)p.nstages * p.stage_bytes + (size_t)p.ngroups * p.part_bytes + 8 * (size_t)p.nstages + 128;
}

template <typename Real, int K, int MODE>
cudaError_t launch_cols_pipe_t(const CUtensorMap &map, const ColsPipe &p, const TilePtrs *fields, int grid,
                               cudaStream_t st)
{
    cudaError_t e = ensure_smem_attr((const void *)k_cols_pipe<Real, K, MODE>);
    if (e != cudaSuccess)
        return e;
    const int threads = p.ngroups * p.group_threads;
    k_cols_pipe<Real, K, MODE><<<grid, threads, cols_pipe_smem(p), st>>>(map, p, fields);
    return cudaGetLastError();
}

template <typename Real, int K, int MODE>
cudaError_t cols_pipe_regs_t(int *regs)
{
    cudaFuncAttributes at;
    cudaError_t e = cudaFuncGetAttributes(&at, (const void *)k_cols_pipe<Real, K, MODE>);
    if (e == cudaSuccess)
        *regs = at.numRegs;
    return e;
}

}  // namespace fbg
