// tb_pipe.cu -- FP32 Chebyshev recurrence, pipelined form (K2 of the
// density-matrix path: the recurrence of getKPE, withSP2_deltaH.cpp:1134-1168,
// over identity columns, with the moments taken from column dot products as in
// k_cheb_f32_staged).
//
// Slab layout: chunk-major, [B/64][n][64] floats, so that a block row of one
// 64-column chunk is 1 KB contiguous and consecutive block rows are
// contiguous too.
//
// One CTA per SM loops over tiles (row group g of R block rows x one
// 64-column chunk).  A producer warp gathers each tile into a ring of
// shared-memory stages with bulk asynchronous copies (cp.async.bulk,
// completion counted in bytes on the stage's "full" mbarrier): the group's
// distinct referenced block rows of T_k as runs of consecutive rows (one copy
// per run), its own rows of T_{k-1} (one copy), its X blocks (one copy) and a
// packed index record (one copy).  Twelve consumer warps compute the tile from
// shared memory while the producer fills the next stages.  The header and
// copy runs of the next tile are loaded while the producer waits for a free
// stage, so no global load latency sits on its path.
//
// Three launch modes share the kernel:
//  - one launch per step (steps = 1);
//  - one cooperative launch per slab running all K steps.  A tile publishes
//    its step count in flags[tile] (release, after an mbarrier that every
//    consumer warp arrives on after its stores); before the producer copies
//    tile (chunk, g) of step k >= 1 it waits (acquire) until every group g'
//    whose rows g references, g itself included, has published step k in the
//    same chunk.  That covers both the T_k rows it reads and the T_{k-1} rows
//    it overwrites: the block pattern is symmetric, so the groups that read
//    rows of g at step k-1 are exactly those neighbours.  Each CTA runs its
//    tiles in step order and all CTAs are co-resident, so the oldest
//    unfinished step can always proceed.  The pipeline never drains between
//    steps;
//  - the batched form (k_cheb_f32_pipe<true, ...>, one launch per step): tiles
//    come from a list over many structures, each tile naming its row group
//    and carrying the offset of its chunk in that structure's slabs and of
//    its column sums; a group's header holds its first (structure-local)
//    block row.
//
// Column dot products <T_k,T_k> and <T_k,T_{k+1}> accumulate in FP32 over one
// block row and then as unevaluated FP32 pairs (hi, lo) across rows and warps:
// every addition is Knuth's TwoSum (s = a + b, e = (a - (s - b')) + (b - b'),
// b' = s - a), its exact rounding error collected in lo.  GB300 issues FP64 at
// about 2 operations per clock per SM, so per-row FP64 accumulation would cost
// as much as the rest of the step; the pairs keep ~44 significant bits with
// FP32 arithmetic only.  The recurrence itself and the per-row products use
// packed FP32 pair instructions (fma.f32x2 / add.f32x2: two columns per
// instruction, each rounded as the scalar operation).  Each consumer warp
// hands its pairs over in a shared array and arrives on an mbarrier; four
// consumer warps, in rotation from tile to tile, wait for all twelve and sum
// them in warp order, giving partial[k][g][col][2] as float2 (hi, lo), while
// the other warps go on with the next tile.  k_f32_finalize_pairs converts to
// FP64.
//
// Every wait is bounded: after kPipeSpin unsuccessful polls the thread raises
// a block-wide abort flag and the device error flag; every later wait in the
// CTA then returns at once, the warps run out their tile sequence skipping
// the work, other CTAs waiting on this one's flags time out the same way, and the
// producer, before it returns, waits (again bounded) for the copies it has
// issued.  The host turns the error flag into TB_ERR_TIMEOUT (1: a stage
// mbarrier wait, 2: a neighbour-flag wait ran out).
//
// Two environment variables, read at each one-launch-per-slab launch, let a
// test make a neighbour wait run out without any fault: LARGETB_TEST_WAIT_LIMIT
// (neighbour-flag polls before giving up; default 2^22) and
// LARGETB_TEST_STALL_TILE (a tile whose step flags are never published, so
// every tile that reads its rows waits for a flag that nothing sets).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "tb_f32x2.cuh"
#include "tb_internal.h"

namespace tb {

namespace {

constexpr int kPipeCols = 64;
constexpr int kPipeCW = 12;  // consumer warps; then one producer and one publisher warp
constexpr int kPipeThreads = 32 * (kPipeCW + 2);
constexpr int kPubSlots = 4;  // tiles the publisher may lag behind the consumers
constexpr int kRedWarps = 4;  // consumer warps that reduce one tile's column sums, in rotation
static_assert(kPipeCW % kRedWarps == 0 && kRedWarps * 32 == 2 * kPipeCols, "reducer split");
constexpr uint32_t kPipeSpin = 1u << 22;  // mbarrier polls
constexpr uint32_t kFlagSpin = 1u << 22;  // neighbour-flag polls (~128 ns apart)

struct PipeArgs {
    int n, nb, R, G, nchunk, stages, stage_bytes, maxU, maxBlk, B, run_stride;
    int k0, steps;     // steps k0 .. k0+steps-1 (k = 0 computes T_1 = X T_0)
    const int4 *hdr;   // per group: {nu, tb0, nbk, rec_off}, {rec_len, -, nruns, nr}
    const int4 *runs;  // run_stride per group: {first block row, rows, first slot, 0}
    const int32_t *rec;
    const int32_t *nbr_ptr, *nbr;  // neighbouring groups of each group (itself included)
    const float *x32;
    float *T0, *T1;    // step k reads T_k from (k even ? T0 : T1) and writes T_{k+1} to the other
    float2 *partial;   // [steps][G][B][2] pairs; step k writes block k - k0
    int32_t *flags;    // [G * nchunk] completed steps per tile (multi-step launch), or null
    int32_t *err;
    const PipeBatchTile *tiles;  // batched form: the tile list (slab and partial offsets per tile)
    int ntiles;
    uint32_t flag_spin;  // neighbour-flag polls before a wait gives up (kFlagSpin unless a test lowers it)
    int stall_tile;      // test knob: this tile never publishes its step flags (-1: none)
};

__device__ __forceinline__ uint32_t sm_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(sm_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(sm_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(sm_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(sm_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// global -> shared bulk copy; both addresses 16-byte aligned, bytes % 16 == 0
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            sm_addr(dst)),
        "l"(src), "r"(bytes), "r"(sm_addr(bar))
        : "memory");
}

__device__ __forceinline__ int ld_acquire(const int32_t *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int32_t *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// orders generic-proxy accesses to global memory with the bulk (async-proxy)
// copies that follow
__device__ __forceinline__ void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;\n" ::: "memory");
}

// Poll until the phase of the given parity completes; false on abort or
// after kPipeSpin polls (then the abort and device error flags are raised).
// Each lane polls on its own; lanes may leave on an abort at different polls,
// so a caller uses it only where a lane's answer governs that lane's own work.
__device__ __forceinline__ bool wait_phase(uint64_t *bar, uint32_t parity, volatile int *s_abort,
                                           int32_t *err)
{
    uint32_t n = 0;
    while (!mbar_try_wait(bar, parity)) {
        if (*s_abort) return false;
        if (++n >= kPipeSpin) {
            *s_abort = 1;
            atomicExch(err, 1);
            return false;
        }
    }
    return true;
}

// wait_phase with the warp's answer: every lane of the warp calls it and all
// get the same result, so a warp never splits over an abort.  For the
// producer (its copy issue is one warp-wide step), the publisher and the
// publisher hand-off.
__device__ __forceinline__ bool wait_phase_warp(uint64_t *bar, uint32_t parity, volatile int *s_abort,
                                                int32_t *err)
{
    return __all_sync(0xffffffffu, wait_phase(bar, parity, s_abort, err));
}

// The consumers' wait for tile i's stage (per lane, like wait_phase).  A tile
// the producer issued is always waited for (its bulk copies must land before
// the stage is refilled or the CTA exits), abort or not; a tile the producer
// never issued (*s_issued: -1 while it runs, then the count it issued) is
// given up, and so is every later one (gave_up): once a lane has passed over
// a phase that never completed, a later poll of that stage could name a
// parity that an older, completed phase had, and try_wait would report a
// never-filled stage as full.  Until then no phase was skipped, so a poll
// that succeeds is the tile's own phase.  Every lane reaches the same verdict
// (a never-issued tile never completes, an issued one always does).  The
// issue count is looked at once every 64 unsuccessful polls, keeping the
// common path to the poll alone.  Bounded by kPipeSpin polls like every wait.
__device__ __forceinline__ bool wait_full(uint64_t *bar, uint32_t parity, int i, volatile int *s_abort,
                                          volatile int *s_issued, int32_t *err, bool &gave_up)
{
    if (gave_up) return false;
    uint32_t n = 0;
    while (!mbar_try_wait(bar, parity)) {
        if ((++n & 63u) == 0u) {
            const int iss = *s_issued;
            if (iss >= 0 && i >= iss) {
                gave_up = true;
                return false;
            }
        }
        if (n >= kPipeSpin) {
            *s_abort = 1;
            atomicExch(err, 1);
            gave_up = true;
            return false;
        }
    }
    return true;
}

// Producer warp: the flag word lane q watches for tile (chunk, g): neighbour
// q of g (q < 32), or null.
__device__ __forceinline__ const int32_t *neighbour_flag(const PipeArgs &a, int chunk, int g, int q)
{
    const int p0 = a.nbr_ptr[g], p1 = a.nbr_ptr[g + 1];
    return p0 + q < p1 ? a.flags + (int64_t)chunk * a.G + a.nbr[p0 + q] : nullptr;
}

// Producer warp: wait until every neighbour tile of (chunk, g) has published
// step k.  seen: this lane's flag as read (acquire) before the stage wait, so
// that an already satisfied wait costs no further round trip.  Otherwise the
// lanes poll the neighbours in parallel with acquire loads; false on abort /
// timeout.
__device__ __forceinline__ bool wait_neighbours(const PipeArgs &a, int chunk, int g, int k, int lane, int seen,
                                                volatile int *s_abort)
{
    const int p0 = a.nbr_ptr[g], p1 = a.nbr_ptr[g + 1];
    const int32_t *fl = a.flags + (int64_t)chunk * a.G;
    if (p1 - p0 <= 32 && __all_sync(0xffffffffu, seen >= k)) return true;
    for (int base = p0; base < p1; base += 32) {
        const int q = base + lane;
        const int32_t *f = q < p1 ? fl + a.nbr[q] : nullptr;
        uint32_t n = 0;
        while (!__all_sync(0xffffffffu, f == nullptr || ld_acquire(f) >= k)) {
            if (__any_sync(0xffffffffu, *s_abort != 0)) return false;
            if (++n >= a.flag_spin) {
                if (lane == 0) {
                    *s_abort = 1;
                    atomicExch(a.err, 2);
                }
                __syncwarp();
                return false;
            }
            __nanosleep(128);
        }
    }
    return true;
}

// Tile of this CTA's i-th task.  One-launch-per-step launches sweep the
// tiles backwards on odd steps, so a step starts on the rows of T_{k+1} and
// T_k that the previous step touched last and that are still in L2.
template <bool kMulti>
__device__ __forceinline__ int tile_of_task(const PipeArgs &a, int ntiles, int i, int mine)
{
    const int t = (int)blockIdx.x + (i % mine) * (int)gridDim.x;
    const int k = a.k0 + i / mine;
    return (!kMulti && (k & 1)) ? ntiles - 1 - t : t;
}

// kBatch: tiles come from a.tiles (row groups of many structures, each
// structure its own chunk-major slabs and partial block); else tile t is
// (chunk t / G, group t % G) of one slab.  kMulti: the one-launch-per-slab
// mode (step flags, neighbour waits, the publisher warp); the per-step and
// batched instantiations carry none of that code.
template <bool kBatch, bool kMulti>
__global__ void __launch_bounds__(kPipeThreads, 1) k_cheb_f32_pipe(const PipeArgs a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    // [CW][2][32][4]: consumer warp w, lane l, column 2l + h at ((2w + h) 32 + l) 4,
    // holding (<T_k,T_k> hi, lo, <T_k,T_{k+1}> hi, lo); each 16-byte store of a
    // warp covers 512 contiguous bytes (no bank conflict)
    float *red = reinterpret_cast<float *>(smem + (size_t)a.stages * a.stage_bytes);
    uint64_t *full = reinterpret_cast<uint64_t *>(red + kPipeCW * kPipeCols * 4);
    uint64_t *empty = full + a.stages;
    uint64_t *pub = empty + a.stages;       // consumers -> publisher: tile done
    uint64_t *pubfree = pub + kPubSlots;    // publisher -> consumers: slot free again
    uint64_t *redfull = pubfree + kPubSlots;  // consumer warps -> reducers: red[] holds the tile's sums
    uint64_t *redfree = redfull + 1;          // reducers -> consumer warps: red[] read
    volatile int *s_abort = reinterpret_cast<volatile int *>(redfree + 1);
    volatile int *s_issued = s_abort + 1;  // tiles the producer issued, -1 while it runs
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < a.stages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kPipeCW);
        }
        for (int s = 0; s < kPubSlots; s++) {
            mbar_init(&pub[s], 1);
            mbar_init(&pubfree[s], 1);
        }
        mbar_init(redfull, kPipeCW);
        mbar_init(redfree, kRedWarps);
        *s_abort = 0;
        *s_issued = -1;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    const int ntiles = kBatch ? a.ntiles : a.G * a.nchunk;
    const int mine = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int total = mine * a.steps;  // this CTA's tiles over all steps, step-major
    const int oT = 0, oP = a.maxU * 4 * kPipeCols, oX = oP + a.R * 4 * kPipeCols,
              oRec = oX + a.maxBlk * 16;  // float offsets inside a stage
    const int64_t chunk_floats = (int64_t)a.n * kPipeCols;

    if (warp == kPipeCW + 1) {
        // ---------------- publisher ----------------
        // Publishes each finished tile's step count: a GPU-scope fence makes
        // the consumers' T_{k+1} stores (ordered before the slot's mbarrier
        // arrival) visible before the release store of the flag.  The fence
        // stalls only this warp.
        if constexpr (!kMulti) return;
        for (int i = 0; i < total; ++i) {
            const int s = i % kPubSlots;
            if (!wait_phase_warp(&pub[s], (uint32_t)(i / kPubSlots) & 1u, s_abort, a.err)) break;
            if (lane == 0) {
                const int k = a.k0 + i / mine;
                const int t = tile_of_task<kMulti>(a, ntiles, i, mine);
                __threadfence();
                fence_proxy_async_global();
                if (t != a.stall_tile) st_release(a.flags + t, k + 1);
                mbar_arrive(&pubfree[s]);
            }
            __syncwarp();
        }
        return;
    }

    if (warp == kPipeCW) {
        // ---------------- producer ----------------
        int i = 0;
        int4 ha = make_int4(0, 0, 0, 0), hb = ha, run = ha;
        int gnext = 0;          // group of the next tile
        int64_t cnext = 0;      // batched form: its chunk offset
        if (total > 0) {
            if constexpr (kBatch) {
                const int t0 = tile_of_task<kMulti>(a, ntiles, 0, mine);
                gnext = a.tiles[t0].g;
                cnext = a.tiles[t0].coff;
            } else {
                gnext = tile_of_task<kMulti>(a, ntiles, 0, mine) % a.G;
            }
            ha = __ldg(a.hdr + 2 * gnext);
            hb = __ldg(a.hdr + 2 * gnext + 1);
            run = __ldg(a.runs + (int64_t)gnext * a.run_stride + lane);
        }
        for (; i < total; ++i) {
            const int k = a.k0 + i / mine;
            const int t = tile_of_task<kMulti>(a, ntiles, i, mine);
            const int g = gnext;
            const int chunk = kBatch ? 0 : t / a.G;
            const int64_t coff = kBatch ? cnext : (int64_t)chunk * chunk_floats;
            const int nu = ha.x, tb0 = ha.y, nbk = ha.z, r0 = ha.w;
            const int rl = hb.x, I0 = hb.y, nruns = hb.z, nr = hb.w;
            const int4 cur = run;
            if (i + 1 < total) {  // header and runs of the next tile
                const int tn = tile_of_task<kMulti>(a, ntiles, i + 1, mine);
                if constexpr (kBatch) {
                    gnext = a.tiles[tn].g;
                    cnext = a.tiles[tn].coff;
                } else {
                    gnext = tn % a.G;
                }
                ha = __ldg(a.hdr + 2 * gnext);
                hb = __ldg(a.hdr + 2 * gnext + 1);
                run = __ldg(a.runs + (int64_t)gnext * a.run_stride + lane);
            }
            // this tile's neighbour flags, read before the stage wait
            int seen = 0x7fffffff;
            if (kMulti && k > 0) {
                const int32_t *f = neighbour_flag(a, chunk, g, lane);
                if (f) seen = ld_acquire(f);
            }
            const int s = i % a.stages;
            if (i >= a.stages && !wait_phase_warp(&empty[s], (uint32_t)((i / a.stages) - 1) & 1u, s_abort, a.err))
                break;
            if (kMulti && k > 0) {
                if (!wait_neighbours(a, chunk, g, k, lane, seen, s_abort)) break;
                fence_proxy_async_global();
            }
            const float *Tin = (k & 1) ? a.T1 : a.T0;
            const float *Tprev = (k & 1) ? a.T0 : a.T1;
            float *stg = reinterpret_cast<float *>(smem + (size_t)s * a.stage_bytes);
            if (lane == 0)
                mbar_arrive_expect_tx(&full[s], (uint32_t)nu * 1024u + (k == 0 ? 0u : (uint32_t)nr * 1024u) +
                                                    (uint32_t)nbk * 64u + (uint32_t)rl * 4u);
            __syncwarp();
            const float *srcT = Tin + coff;
            if (lane < nruns)
                bulk_g2s(stg + oT + cur.z * 4 * kPipeCols, srcT + (int64_t)cur.x * 4 * kPipeCols,
                         (uint32_t)cur.y * 1024u, &full[s]);
            for (int q = lane + 32; q < nruns; q += 32) {
                const int4 rr = __ldg(a.runs + (int64_t)g * a.run_stride + q);
                bulk_g2s(stg + oT + rr.z * 4 * kPipeCols, srcT + (int64_t)rr.x * 4 * kPipeCols,
                         (uint32_t)rr.y * 1024u, &full[s]);
            }
            if (lane == 0) {
                bulk_g2s(stg + oX, a.x32 + (int64_t)tb0 * 16, (uint32_t)nbk * 64u, &full[s]);
                bulk_g2s(stg + oRec, a.rec + r0, (uint32_t)rl * 4u, &full[s]);
                if (k > 0)
                    bulk_g2s(stg + oP, Tprev + coff + (int64_t)I0 * 4 * kPipeCols, (uint32_t)nr * 1024u, &full[s]);
            }
        }
        // the consumers wait for every tile issued (i of them) and give up the rest
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            *s_issued = i;
        }
        if (*s_abort) {
            // let the copies already issued land before the CTA exits
            for (int j = max(0, i - a.stages); j < i; j++) {
                uint32_t n = 0;
                while (!mbar_try_wait(&full[j % a.stages], (uint32_t)(j / a.stages) & 1u) && ++n < kPipeSpin) {
                }
            }
        }
        return;
    }

    // ---------------- consumers ----------------
    const int c = 2 * lane;
    bool gave_up = false;  // this warp has passed over a tile that was never issued
    // batched form: the next tile's descriptor and group header, loaded one
    // tile ahead so that their latency overlaps the current tile
    PipeBatchTile bt_next{};
    int4 hb_next = make_int4(0, 0, 0, 0);
    if (kBatch && total > 0) {
        bt_next = a.tiles[tile_of_task<kMulti>(a, ntiles, 0, mine)];
        hb_next = __ldg(a.hdr + 2 * bt_next.g + 1);
    }
    for (int i = 0; i < total; ++i) {
        const int k = a.k0 + i / mine;
        const int t = tile_of_task<kMulti>(a, ntiles, i, mine);
        const int s = i % a.stages;
        int g, I0, nr;
        int64_t coff, pbase;  // slab offset of the tile's chunk; float2 offset of its column sums
        if constexpr (kBatch) {
            const PipeBatchTile bt = bt_next;
            const int4 hb = hb_next;
            if (i + 1 < total) {
                bt_next = a.tiles[tile_of_task<kMulti>(a, ntiles, i + 1, mine)];
                hb_next = __ldg(a.hdr + 2 * bt_next.g + 1);
            }
            g = bt.g;
            coff = bt.coff;
            pbase = bt.pbase;
            I0 = hb.y;
            nr = hb.w;
        } else {
            const int chunk = t / a.G;
            g = t - chunk * a.G;
            I0 = g * a.R;
            nr = min(a.nb, I0 + a.R) - I0;
            coff = (int64_t)chunk * chunk_floats;
            pbase = (((int64_t)(k - a.k0) * a.G + g) * a.B + chunk * kPipeCols) * 2;
        }
        float *out = ((k & 1) ? a.T0 : a.T1) + coff + (int64_t)I0 * 4 * kPipeCols + c;
        // pairs (hi, lo), packed over columns (c, c+1): <T_k,T_k> in (eh, el),
        // <T_k,T_{k+1}> in (oh, ol)
        float2 eh = make_float2(0.f, 0.f), el = eh, oh = eh, ol = eh;
        if (wait_full(&full[s], (uint32_t)(i / a.stages) & 1u, i, s_abort, s_issued, a.err, gave_up)) {
            const float *stg = reinterpret_cast<const float *>(smem + (size_t)s * a.stage_bytes);
            const float *sT = stg + oT, *sP = stg + oP, *sX = stg + oX;
            const int32_t *sRp = reinterpret_cast<const int32_t *>(stg + oRec);
            const int32_t *sLc = sRp + nr + 1;
            const int32_t *sLs = sLc + sRp[nr];
            for (int r = warp; r < nr; r += kPipeCW) {
                // acc[q] = row q of the block row, columns (c, c+1)
                float2 acc[4];
#pragma unroll
                for (int q = 0; q < 4; q++) acc[q] = make_float2(0.f, 0.f);
                const int ta = sRp[r], te = sRp[r + 1];
                for (int tt = ta; tt < te; tt++) {
                    const float *tv = sT + sLc[tt] * 4 * kPipeCols + c;
                    const float4 *xb = reinterpret_cast<const float4 *>(sX + tt * 16);
                    float2 v[4];
#pragma unroll
                    for (int m = 0; m < 4; m++) v[m] = *reinterpret_cast<const float2 *>(tv + m * kPipeCols);
                    block_fma2(acc, xb, v);
                }
                const float *own = sT + sLs[r] * 4 * kPipeCols + c;
                float2 ee = make_float2(0.f, 0.f), eo = ee;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 ov = *reinterpret_cast<const float2 *>(own + q * kPipeCols);
                    float2 o = acc[q];
                    if (k > 0) o = cheb_next2(acc[q], *reinterpret_cast<const float2 *>(sP + (r * 4 + q) * kPipeCols + c));
                    *reinterpret_cast<float2 *>(out + (r * 4 + q) * kPipeCols) = o;
                    ee = __ffma2_rn(ov, ov, ee);
                    eo = __ffma2_rn(ov, o, eo);
                }
                pair_add2(eh, el, ee);
                pair_add2(oh, ol, eo);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);  // stage s may be refilled
        // Hand this warp's sums over in red[warp]; the buffer is free again once
        // the previous tile's reducers have read it.  Neither phase below can
        // complete twice before it is polled: the next phase of redfull needs
        // this tile's redfree, and the next phase of redfree needs this warp's
        // arrival on redfull.
        if (i == 0 || wait_phase(redfree, (uint32_t)(i - 1) & 1u, s_abort, a.err)) {
            float4 *rb = reinterpret_cast<float4 *>(red + ((size_t)(2 * warp) * 32 + lane) * 4);
            rb[0] = make_float4(eh.x, el.x, oh.x, ol.x);   // column c
            rb[32] = make_float4(eh.y, el.y, oh.y, ol.y);  // column c + 1
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(redfull);  // after this warp's T_{k+1} stores of the tile
        const int rw = warp - kRedWarps * (i % (kPipeCW / kRedWarps));
        if (rw >= 0 && rw < kRedWarps) {
            // this tile's reducers: (column, which) pairs summed over the
            // consumer warps in warp order
            if (wait_phase(redfull, (uint32_t)i & 1u, s_abort, a.err)) {
                // reducer lane q reads float2 q of every warp's [2][32][4] block:
                // half h = q / 64, consumer lane l, sum `which` (consecutive lanes,
                // consecutive addresses); its column is j = 2 l + h
                const int q = rw * 32 + lane, h = q >> 6, l = (q & 63) >> 1, which = q & 1, j = 2 * l + h;
                float hsum = 0.f, lsum = 0.f;
#pragma unroll
                for (int w = 0; w < kPipeCW; w++) {
                    const float2 v = *reinterpret_cast<const float2 *>(red + (size_t)w * 256 + 2 * q);
                    pair_add(hsum, lsum, v.x);
                    lsum += v.y;
                }
                a.partial[pbase + j * 2 + which] = make_float2(hsum, lsum);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(redfree);
            // the first reducer hands the tile to the publisher: it has seen every
            // consumer warp's arrival, so all stores of the tile precede this
            if (kMulti && rw == 0) {
                const int ps = i % kPubSlots;
                if (i < kPubSlots ||
                    wait_phase_warp(&pubfree[ps], (uint32_t)((i / kPubSlots) - 1) & 1u, s_abort, a.err)) {
                    if (lane == 0) mbar_arrive(&pub[ps]);
                }
            }
        }
    }
}

// Identity columns c0 .. c0+B-1 in the chunk-major layout [B/64][n][64].
__global__ void k_slab_identity_cm(float *__restrict__ T0, int n, int B, int c0)
{
    const int64_t tot = (int64_t)n * B, per = (int64_t)n * kPipeCols;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int chunk = (int)(e / per);
        const int64_t rem = e - (int64_t)chunk * per;
        const int row = (int)(rem / kPipeCols), j = (int)(rem % kPipeCols);
        T0[e] = (row == c0 + chunk * kPipeCols + j) ? 1.f : 0.f;
    }
}

// Sum of (hi, lo) pairs over groups g = 0 .. G-1 at p[g * stride], in group
// order, eight 16-byte loads in flight before their additions.
__device__ __forceinline__ void sum_group_pairs(const float4 *__restrict__ p, int64_t stride, int G, float &eh,
                                                float &el, float &oh, float &ol)
{
    int g = 0;
    for (; g + 8 <= G; g += 8) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = __ldg(p + (g + u) * stride);
#pragma unroll
        for (int u = 0; u < 8; u++) {
            pair_add(eh, el, v[u].x);
            el += v[u].y;
            pair_add(oh, ol, v[u].z);
            ol += v[u].w;
        }
    }
    for (; g < G; g++) {
        const float4 v = __ldg(p + g * stride);
        pair_add(eh, el, v.x);
        el += v.y;
        pair_add(oh, ol, v.z);
        ol += v.w;
    }
}

// Sum the per-group (hi, lo) pairs of a slab in FP32 pairs, convert once to
// FP64 and form the moments d[2k][j] = 2 <T_k,T_k>_j - 1,
// d[2k+1][j] = 2 <T_k,T_{k+1}>_j - X_jj.
__global__ void k_f32_finalize_pairs(const float2 *__restrict__ partial, int K, int rowgroups, int B, int c0,
                                     int n, const float *__restrict__ xdiag32, double *__restrict__ d, int M)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (j >= B || k >= K) return;
    const int i = c0 + j;
    if (i >= n) return;
    float eh = 0.f, el = 0.f, oh = 0.f, ol = 0.f;
    // (e, o) of column j in group g: one 16-byte load at [g][B][2] float2
    const float4 *p = reinterpret_cast<const float4 *>(partial + (int64_t)k * rowgroups * B * 2) + j;
    sum_group_pairs(p, B, rowgroups, eh, el, oh, ol);
    const double se = (double)eh + (double)el, so = (double)oh + (double)ol;
    if (2 * k <= M) d[(int64_t)(2 * k) * n + i] = 2.0 * se - 1.0;
    if (2 * k + 1 <= M) d[(int64_t)(2 * k + 1) * n + i] = 2.0 * so - (double)xdiag32[i];
}

}  // namespace

size_t cheb_f32_pipe_stage_bytes(int R, int maxU, int maxBlk, int rec_cap)
{
    const size_t b = (size_t)(maxU + R) * 4 * kPipeCols * sizeof(float) + (size_t)maxBlk * 16 * sizeof(float) +
                     (size_t)rec_cap * sizeof(int32_t);
    return (b + 127) / 128 * 128;
}

size_t cheb_f32_pipe_smem(size_t stage_bytes, int stages)
{
    return (size_t)stages * stage_bytes + (size_t)kPipeCW * kPipeCols * 4 * sizeof(float) +
           (size_t)(2 * stages + 2 * kPubSlots + 2) * sizeof(uint64_t) + 16;
}

int cheb_f32_pipe_max_rows() { return kPipeCW * 3; }

int cheb_f32_pipe_configure(size_t smem, int *ctas_per_sm, bool batch)
{
    const void *fn = batch ? (const void *)k_cheb_f32_pipe<true, false> : (const void *)k_cheb_f32_pipe<false, false>;
    const int lim = smem_optin_max(fn);
    if ((int)smem > lim) return (int)cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e != cudaSuccess) return (int)e;
    if (!batch) {
        const void *fm = (const void *)k_cheb_f32_pipe<false, true>;
        if ((e = cudaFuncSetAttribute(fm, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin_max(fm))))
            return (int)e;
    }
    *ctas_per_sm = 0;
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, kPipeThreads, smem);
}

void launch_f32_finalize_pairs(cudaStream_t st, const DevMatrix &m, const float2 *partial, int K, int rowgroups,
                               int B, int c0, double *d, int M)
{
    dim3 grid((B + 127) / 128, K);
    k_f32_finalize_pairs<<<grid, 128, 0, st>>>(partial, K, rowgroups, B, c0, m.n, m.xdiag32, d, M);
}

void launch_slab_identity_cm(cudaStream_t st, float *T0, int n, int B, int c0)
{
    const int64_t tot = (int64_t)n * B;
    const int blocks = (int)std::min<int64_t>((tot + 255) / 256, 152 * 16);
    k_slab_identity_cm<<<blocks, 256, 0, st>>>(T0, n, B, c0);
}

int launch_cheb_f32_pipe(cudaStream_t st, const DevMatrix &m, const PipePlan &pl, float *T0, float *T1, int B,
                         int k0, int steps, float2 *partial, bool multi)
{
    PipeArgs a;
    a.n = m.n;
    a.nb = m.nb;
    a.R = pl.R;
    a.G = pl.G;
    a.nchunk = B / kPipeCols;
    a.stages = pl.stages;
    a.stage_bytes = (int)pl.stage_bytes;
    a.maxU = pl.maxU;
    a.maxBlk = pl.maxBlk;
    a.B = B;
    a.run_stride = pl.run_stride;
    a.k0 = k0;
    a.steps = steps;
    a.hdr = reinterpret_cast<const int4 *>(pl.hdr);
    a.runs = reinterpret_cast<const int4 *>(pl.runs);
    a.rec = pl.rec;
    a.nbr_ptr = pl.nbr_ptr;
    a.nbr = pl.nbr;
    a.x32 = m.x32;
    a.T0 = T0;
    a.T1 = T1;
    a.partial = partial;
    a.flags = multi ? pl.flags : nullptr;
    a.err = pl.err;
    a.tiles = nullptr;
    a.ntiles = 0;
    a.flag_spin = kFlagSpin;
    a.stall_tile = -1;
    if (multi) {
        if (const char *v = std::getenv("LARGETB_TEST_WAIT_LIMIT")) {
            const unsigned long x = std::strtoul(v, nullptr, 10);
            if (x > 0 && x < kFlagSpin) a.flag_spin = (uint32_t)x;
        }
        if (const char *v = std::getenv("LARGETB_TEST_STALL_TILE")) a.stall_tile = (int)std::strtol(v, nullptr, 10);
    }
    const int ntiles = pl.G * a.nchunk;
    const int grid = std::min(ntiles, pl.nsm);
    const size_t smem = cheb_f32_pipe_smem(pl.stage_bytes, pl.stages);
    if (!multi) {
        k_cheb_f32_pipe<false, false><<<grid, kPipeThreads, smem, st>>>(a);
        return (int)cudaSuccess;
    }
    cudaError_t e = cudaMemsetAsync(pl.flags, 0, sizeof(int32_t) * (size_t)ntiles, st);
    if (e != cudaSuccess) return (int)e;
    void *args[] = {&a};
    return (int)cudaLaunchCooperativeKernel((const void *)k_cheb_f32_pipe<false, true>, dim3(grid), dim3(kPipeThreads), args,
                                            smem, st);
}

void launch_cheb_f32_pipe_batch(cudaStream_t st, const PipePlan &pl, const PipeBatchTile *tiles, int ntiles,
                                const float *x32, float *T0, float *T1, int k, float2 *partial)
{
    PipeArgs a{};
    a.R = pl.R;
    a.G = pl.G;
    a.stages = pl.stages;
    a.stage_bytes = (int)pl.stage_bytes;
    a.maxU = pl.maxU;
    a.maxBlk = pl.maxBlk;
    a.run_stride = pl.run_stride;
    a.k0 = k;
    a.steps = 1;
    a.hdr = reinterpret_cast<const int4 *>(pl.hdr);
    a.runs = reinterpret_cast<const int4 *>(pl.runs);
    a.rec = pl.rec;
    a.x32 = x32;
    a.T0 = T0;
    a.T1 = T1;
    a.partial = partial;
    a.flags = nullptr;
    a.err = pl.err;
    a.tiles = tiles;
    a.ntiles = ntiles;
    a.flag_spin = kFlagSpin;
    a.stall_tile = -1;
    const int grid = std::min(ntiles, pl.nsm);
    if (grid < 1) return;
    k_cheb_f32_pipe<true, false><<<grid, kPipeThreads, cheb_f32_pipe_smem(pl.stage_bytes, pl.stages), st>>>(a);
}

}  // namespace tb
