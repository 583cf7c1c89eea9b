// tcgen05 GEMM of the split-BF16 form (see split.cuh for the arithmetic).
//
// One persistent CTA per SM, 320 threads in three roles:
//   warp 0      TMA producer: streams 128x64 BF16 tiles of the A and B digit
//               planes (128-byte swizzle) into a 3-slot shared-memory ring;
//               a slot holds up to two consecutive 64-wide K blocks of one
//               slice pair (a "group", 64 KB);
//   warp 1      MMA issuer: allocates 512 TMEM columns, issues
//               tcgen05.mma kind::f16 (M=128, N=128, K=16), eight per group,
//               into one of two FP32 accumulators, and commits chunk
//               completion.  A blocking mbarrier wait costs the issuing
//               thread ~140 cycles, longer than the two MMAs the tensor pipe
//               keeps queued, so the issuer tests the next slot's barrier
//               without blocking in the same instruction sequence as the
//               current group's MMAs and waits only when that test failed;
//   warps 2-9   epilogue (two warps per TMEM lane quadrant, 64 columns each):
//               after every chunk of <= 1024 products per output, convert the
//               exact FP32 sums to integers and add them to int32 partial
//               sums in registers, folded into an int64 part in TMEM at the
//               end of each slice group; at the end of a tile scale by
//               2^(eA+eB-...) in FP64 and apply C = cp*C + ab*v through the
//               output's index map.
// TMEM columns: [0,128) accumulator 0, [128,256) accumulator 1,
//               [256,384) int64 low words, [384,512) int64 high words.
// Every mbarrier wait is bounded (split.cuh, ptx.cuh): on a timeout the CTA
// records an error code in *status, raises its abort flag, waits for its own
// TMA loads and MMAs to land, frees TMEM and returns.
#include <climits>
#include <mutex>
#include <type_traits>

#include "ptx.cuh"
#include "split.cuh"

namespace eg::split {

namespace {

constexpr int GROUP_KB = 2;                // K blocks per slot
constexpr int A_BYTES = kBM * kBK * 2;     // one K block of A (16 KB)
constexpr int THREADS = 320; // warp 0 TMA, warp 1 MMA, warps 2..9 epilogue
constexpr uint32_t TMEM_COLS = 512;
constexpr int AUX_BYTES = 256;
constexpr int kFinCols = 8;  // columns of the pending tile finished per chunk (C transposed through shared memory)
// When C is contiguous along the rows (one thread per row): 4 columns per chunk;
// 8 measured 10 % slower on the CCD Wabef contraction (more registers spilled).
constexpr int kFinFast = 4;
constexpr int kDirectKB = 8; // tiles of at most this many K blocks are finished at their end, from TMEM
constexpr int FIN_T = 33;    // padded row count of a warp's transposition buffer
// per epilogue warp: 64 column offsets and exponents, the transposition buffer
// of one batch, and its 32 rows' output offsets and validity
constexpr int EPI_WARP_BYTES = (kBN / 2) * (8 + 4) + kFinCols * FIN_T * 8 + 32 * (8 + 4);

// Ring geometry.  CL = 1: one CTA per 128x128 output tile; a slot holds
// [A kb0][A kb1][B kb0][B kb1] (64 KB), three slots.  CL = 2: a CTA pair
// computes a 256x128 tile with cta_group::2 MMAs (M = 256); each CTA holds its
// own 128 rows of A and half of B (64 rows), so a slot is 48 KB and four fit.
template <int CL>
struct Ring {
    static constexpr int STAGES = CL == 2 ? 4 : 3;
    static constexpr int B_ROWS = kBN / CL;
    static constexpr int B_BYTES = B_ROWS * kBK * 2; // one K block of this CTA's part of B
    static constexpr int STAGE_BYTES = GROUP_KB * (A_BYTES + B_BYTES);
    static constexpr int SMEM_BYTES = 1024 + STAGES * STAGE_BYTES + AUX_BYTES + 8 * EPI_WARP_BYTES + 64;
};
static_assert(Ring<1>::SMEM_BYTES <= 232448 && Ring<2>::SMEM_BYTES <= 232448, "shared memory per CTA");
constexpr int GROUP_M = 16; // tile rasterisation: groups of 16 row tiles share B tiles in L2
constexpr unsigned long long DRAIN_NS = 200ull * 1000 * 1000;

// Optional cycle counters per CTA (TcGemmParams::prof, 8 slots per CTA).
enum { kProfProducerWaitEmpty, kProfMmaWaitFull, kProfMmaWaitAcc, kProfEpiWaitAcc, kProfEpiFlush, kProfEpiFinal,
       kProfTotal, kProfSlots = 8 };

__device__ __forceinline__ void prof_add(const TcGemmParams &p, int slot, long long cycles) {
    if (p.prof) atomicAdd(p.prof + blockIdx.x * kProfSlots + slot, (unsigned long long)cycles);
}

// Output tile t of the schedule in units of CL row tiles (a CTA pair takes two
// vertically adjacent 128-row tiles); mt counts those units.
template <int CL>
__device__ __forceinline__ void tile_coords(const TcGemmParams &p, int t, int &b, int &mt, int &nt) {
    const int mtiles = (p.mtiles + CL - 1) / CL, gm = GROUP_M / CL;
    const int per_batch = mtiles * p.ntiles;
    b = t / per_batch;
    t -= b * per_batch;
    const int per_group = gm * p.ntiles;
    const int g = t / per_group;
    const int first_m = g * gm;
    const int gsize = min(mtiles - first_m, gm);
    const int r = t - g * per_group;
    mt = first_m + r % gsize;
    nt = r / gsize;
}

// Everything one role needs about a tile, for both the single-contraction and
// the grouped form.
struct TileJob {
    int mt, nt;
    int zA, zB;  // digit plane of slice 0 for A / B
    int kbeg;    // first K block (of this pass) of the K slice
    int nkb;     // K blocks
    int tid;     // linear output tile index (single-contraction form); -1: rows past the
                 // last tile (the odd half of a CTA pair's tile), nothing to store
    int64_t M, N;
    const ModeGroup *mg, *ng;
    const int *eA, *eB; // exponents of rows / columns of this (item, batch)
    double *C;          // output base of this (item, batch)
    const CUtensorMap *mapA, *mapB; // per-item maps (grouped launches), else null
};

// Tile t of the schedule, as seen by CTA `rank` of its pair (0 when CL = 1).
template <bool GROUPED, int CL>
__device__ __forceinline__ TileJob resolve(const TcGemmParams &p, const TcItem *items, const int4 *work, int t,
                                           int rank) {
    TileJob j;
    if (!GROUPED) {
        int b, mu;
        const int ks = t % p.ksplit;
        t /= p.ksplit;
        tile_coords<CL>(p, t, b, mu, j.nt);
        j.mt = mu * CL + rank;
        j.zA = b * p.S;
        j.zB = b * p.S;
        j.kbeg = ks * p.kslice;
        j.nkb = min(p.kslice, p.nkb - j.kbeg);
        j.tid = j.mt < p.mtiles ? (b * p.mtiles + j.mt) * p.ntiles + j.nt : -1;
        j.M = p.M;
        j.N = p.N;
        j.mg = &p.mg;
        j.ng = &p.ng;
        j.eA = p.eA + (int64_t)b * p.Mp;
        j.eB = p.eB + (int64_t)b * p.Np;
        int64_t oa, ob, oc;
        group_offsets(p.bg, b, oa, ob, oc);
        j.C = p.C + oc;
        j.mapA = j.mapB = nullptr;
    } else {
        const int4 w = work[t];
        const TcItem &it = items[w.x];
        const int b = w.y;
        j.mt = w.z;
        j.nt = w.w;
        if (p.item_maps) { // planes numbered within the item
            j.mapA = p.item_maps + 2 * w.x;
            j.mapB = j.mapA + 1;
            j.zA = j.zB = b * p.S;
        } else {
            j.mapA = j.mapB = nullptr;
            j.zA = it.zA + b * p.S;
            j.zB = it.zB + b * p.S;
        }
        j.kbeg = 0;
        j.nkb = it.nkb;
        j.tid = 0;
        j.M = it.M;
        j.N = it.N;
        j.mg = &it.mg;
        j.ng = &it.ng;
        j.eA = p.eA + it.eAoff + (int64_t)b * it.Mp;
        j.eB = p.eB + it.eBoff + (int64_t)b * it.Np;
        int64_t oa, ob, oc;
        group_offsets(it.bg, b, oa, ob, oc);
        j.C = it.C + oc;
    }
    return j;
}

// K blocks of schedule entry t.
template <bool GROUPED>
__device__ __forceinline__ int entry_nkb(const TcGemmParams &p, const TcItem *items, const int4 *work, int t) {
    if (GROUPED) return items[work[t].x].nkb;
    const int kbeg = (t % p.ksplit) * p.kslice;
    return min(p.kslice, p.nkb - kbeg);
}

// The eight MMAs of one group (two K blocks at A/B descriptors a0, b0; the
// second block sits A_BYTES / the slot's B block size further on) and, in the
// same instruction sequence, a test of whether phase `parity` of the barrier at
// `next_bar` has completed.  The test's result is read after the MMAs are
// issued, so its latency overlaps their execution.
#define EG_MMA_GROUP_ASM(CG)                                                                                           \
    "{\n .reg .pred p, q;\n .reg .b64 a, b;\n setp.ne.b32 q, %4, 0;\n"                                              \
    " mbarrier.test_wait.parity.shared::cta.b64 p, [%5], %6;\n"                                                        \
    " tcgen05.mma.cta_group::" CG ".kind::f16 [%1], %2, %3, %7, q;\n"                                                  \
    " tcgen05.mma.cta_group::" CG ".kind::f16 [%1], %8, %9, %7, 1;\n"                                                  \
    " tcgen05.mma.cta_group::" CG ".kind::f16 [%1], %10, %11, %7, 1;\n"                                                \
    " tcgen05.mma.cta_group::" CG ".kind::f16 [%1], %12, %13, %7, 1;\n"                                                \
    " add.s64 a, %2, %14;\n add.s64 b, %3, %15;\n"                                                                     \
    " tcgen05.mma.cta_group::" CG ".kind::f16 [%1], a, b, %7, 1;\n"                                                    \
    " add.s64 a, %8, %14;\n add.s64 b, %9, %15;\n"                                                                     \
    " tcgen05.mma.cta_group::" CG ".kind::f16 [%1], a, b, %7, 1;\n"                                                    \
    " add.s64 a, %10, %14;\n add.s64 b, %11, %15;\n"                                                                   \
    " tcgen05.mma.cta_group::" CG ".kind::f16 [%1], a, b, %7, 1;\n"                                                    \
    " add.s64 a, %12, %14;\n add.s64 b, %13, %15;\n"                                                                   \
    " tcgen05.mma.cta_group::" CG ".kind::f16 [%1], a, b, %7, 1;\n"                                                    \
    " selp.u32 %0, 1, 0, p;\n}\n"

template <int CL>
__device__ __forceinline__ bool mma_group(uint32_t d, uint64_t a0, uint64_t b0, uint32_t idesc, uint32_t accumulate,
                                          uint32_t next_bar, uint32_t parity) {
    static_assert(GROUP_KB == 2, "two K blocks per group");
    constexpr uint64_t kStep = 32 >> 4; // 16 BF16 along K
    constexpr uint64_t aBlk = A_BYTES >> 4, bBlk = Ring<CL>::B_BYTES >> 4;
    uint32_t ok;
#define EG_MMA_GROUP_OPERANDS                                                                                          \
    : "=r"(ok)                                                                                                         \
    : "r"(d), "l"(a0), "l"(b0), "r"(accumulate), "r"(next_bar), "r"(parity), "r"(idesc), "l"(a0 + kStep),             \
      "l"(b0 + kStep), "l"(a0 + 2 * kStep), "l"(b0 + 2 * kStep), "l"(a0 + 3 * kStep), "l"(b0 + 3 * kStep), "l"(aBlk), \
      "l"(bBlk)                                                                                                        \
    : "memory"
    if constexpr (CL == 1)
        asm volatile(EG_MMA_GROUP_ASM("1") EG_MMA_GROUP_OPERANDS);
    else
        asm volatile(EG_MMA_GROUP_ASM("2") EG_MMA_GROUP_OPERANDS);
#undef EG_MMA_GROUP_OPERANDS
    return ok != 0;
}
#undef EG_MMA_GROUP_ASM

// Records `code` and stops this CTA's roles; in a CTA pair also the peer's
// (peer_flag: shared::cluster address of its abort flag, 0 without a peer).
__device__ __forceinline__ void raise_abort(const TcGemmParams &p, volatile int *abort_flag, int code,
                                            uint32_t peer_flag = 0) {
    atomicCAS(p.status, 0, code);
    *abort_flag = 1;
    if (peer_flag) ptx::st_cluster_u32(peer_flag, 1u);
}

// 10 warps: two of the four SM sub-partitions hold three warps, so the
// 16K-register file of a sub-partition caps a thread at 168 registers.
//
// CL = 2 (launched as clusters of two CTAs): the pair computes 256x128 tiles.
// Both CTAs run a TMA producer that loads its own 128 rows of A and its half of
// B into its own ring, completing on the even CTA's "full" barrier (which
// expects both CTAs' bytes); the even CTA's MMA issuer alone issues
// cta_group::2 MMAs (M = 256) that read both CTAs' shared memory and write
// each CTA's 128 rows into that CTA's tensor memory, and commits to the
// "empty" and "accumulator full" barriers of both CTAs; both CTAs' epilogue
// warps release an accumulator on the even CTA's barrier (16 arrivals).
template <bool GROUPED, int CL>
__global__ void __launch_bounds__(THREADS, 1)
    k_tc_split_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    const __grid_constant__ TcGemmParams p, const TcItem *items, const int4 *work,
                    int ntiles_total) {
    static_assert(CL == 1 || (CL == 2 && !GROUPED), "CTA pairs serve single contractions");
    using R = Ring<CL>;
    constexpr int STAGES = R::STAGES, STAGE_BYTES = R::STAGE_BYTES;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + STAGES * STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *accf = empty + STAGES;
    uint64_t *acce = accf + 2;
    uint64_t *done = acce + 2;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    // per-epilogue-warp copies of the tile's column offsets and exponents, so
    // the epilogue warps never wait on one another
    int64_t *colOffAll = (int64_t *)(smem + STAGES * STAGE_BYTES + AUX_BYTES);
    int *colExpAll = (int *)(colOffAll + 4 * kBN);             // 8 warps x 64 columns each
    double *finTAll = (double *)(colExpAll + 4 * kBN);         // 8 warps x kFinCols x FIN_T
    int64_t *rowOffAll = (int64_t *)(finTAll + 8 * kFinCols * FIN_T); // 8 warps x 32 rows
    int *rowOkAll = (int *)(rowOffAll + 8 * 32);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rank = CL == 2 ? (int)ptx::cluster_ctarank() : 0;
    // shared::cluster addresses: the even CTA's barriers, and the peer's abort flag
    const uint32_t full_lead = CL == 2 ? ptx::mapa(ptx::smem_u32(full), 0) : 0;
    const uint32_t acce_lead = CL == 2 ? ptx::mapa(ptx::smem_u32(acce), 0) : 0;
    const uint32_t peer_flag = CL == 2 ? ptx::mapa(ptx::smem_u32((const void *)abort_flag), rank ^ 1) : 0;
    const long long t_start = p.prof ? clock64() : 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; i++) {
            ptx::mbar_init(&full[i], 1);
            ptx::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; i++) {
            ptx::mbar_init(&accf[i], 1);
            ptx::mbar_init(&acce[i], 8 * CL);
        }
        ptx::mbar_init(done, 1);
        *abort_flag = 0;
        ptx::fence_mbar_init();
    }
    if (warp == 1) {
        ptx::tmem_alloc<CL>(tmem_slot, TMEM_COLS);
        ptx::tmem_relinquish<CL>();
    }
    ptx::tc_fence_before();
    __syncthreads();
    if (CL == 2) ptx::cluster_sync(); // the peer's barriers are initialised before any remote arrival
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // schedule index and stride of this CTA (of its pair when CL = 2)
    const int cta0 = blockIdx.x / CL, ctas = gridDim.x / CL;

    const int total_tiles =
        GROUPED ? ntiles_total : p.nbatch * ((p.mtiles + CL - 1) / CL) * p.ntiles * p.ksplit;

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            ptx::tma_prefetch_desc(&tmA);
            ptx::tma_prefetch_desc(&tmB);
            int stage = 0;
            uint32_t phase = 0;
            int issued = 0; // slots that have received a group (they fill in order 0, 1, 2, ...)
            bool ok = true;
            for (int tile = cta0; tile < total_tiles && ok; tile += ctas) {
                const TileJob job = resolve<GROUPED, CL>(p, items, work, tile, rank);
                const int arow = job.mt * kBM, brow = job.nt * kBN + rank * R::B_ROWS;
                const void *mA = &tmA, *mB = &tmB;
                if (GROUPED && job.mapA) {
                    mA = job.mapA;
                    mB = job.mapB;
                    if (tile + ctas < total_tiles) { // the next tile's maps, while this one runs
                        const CUtensorMap *nm = p.item_maps + 2 * work[tile + ctas].x;
                        ptx::tma_prefetch_desc(nm);
                        ptx::tma_prefetch_desc(nm + 1);
                    }
                    if (tile == cta0) {
                        ptx::tma_prefetch_desc(mA);
                        ptx::tma_prefetch_desc(mB);
                    }
                }
                for (int d = p.d0; d < p.d1 && ok; d++) {
                    for (int s = 0; s <= d && ok; s++) {
                        const int t = d - s;
                        for (int kb = 0; kb < job.nkb; kb += GROUP_KB) {
                            const long long t0 = p.prof ? clock64() : 0;
                            const bool got = ptx::mbar_wait(&empty[stage], phase ^ 1, p.timeout_ns, abort_flag);
                            if (p.prof) prof_add(p, kProfProducerWaitEmpty, clock64() - t0);
                            if (!got) {
                                raise_abort(p, abort_flag, 1, peer_flag);
                                ok = false;
                                break;
                            }
                            if (rank == 0) ptx::mbar_arrive_expect_tx(&full[stage], (uint32_t)(CL * STAGE_BYTES));
                            uint8_t *sa = smem + stage * STAGE_BYTES;
#pragma unroll
                            for (int h = 0; h < GROUP_KB; h++) {
                                const int kc = (p.kb0 + job.kbeg + kb + h) * kBK;
                                uint8_t *sb = sa + GROUP_KB * A_BYTES + h * R::B_BYTES;
                                if (CL == 1) {
                                    ptx::tma_load_3d(sa + h * A_BYTES, mA, &full[stage], kc, arow, job.zA + s);
                                    ptx::tma_load_3d(sb, mB, &full[stage], kc, brow, job.zB + t);
                                } else {
                                    const uint32_t fb = full_lead + (uint32_t)(stage * 8);
                                    ptx::tma_load_3d_pair(sa + h * A_BYTES, &tmA, fb, kc, arow, job.zA + s);
                                    ptx::tma_load_3d_pair(sb, &tmB, fb, kc, brow, job.zB + t);
                                }
                            }
                            if (issued < STAGES) issued++;
                            if (++stage == STAGES) {
                                stage = 0;
                                phase ^= 1;
                            }
                        }
                    }
                }
            }
            // Slot i last received a group in the current round of the ring if
            // i < stage, else in the previous one.  In a pair the even CTA's
            // barriers count both CTAs' loads.
            if (rank == 0)
                for (int i = 0; i < issued; i++)
                    if (!ptx::mbar_wait(&full[i], i < stage ? phase : phase ^ 1, DRAIN_NS, nullptr))
                        raise_abort(p, abort_flag, 4, peer_flag);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer (the even CTA of a pair)
        if (lane == 0 && rank == 0) {
            const uint32_t idesc = ptx::idesc_bf16_f32(kBM * CL, kBN);
            const uint32_t smem_base = ptx::smem_u32(smem), full_base = ptx::smem_u32(full);
            // Descriptors of the slots, fixed for the whole kernel: the issue loop
            // below is unrolled over the slots so that none is recomputed.
            uint64_t da[STAGES], db[STAGES];
#pragma unroll
            for (int i = 0; i < STAGES; i++) {
                da[i] = ptx::smem_desc_sw128(smem_base + i * STAGE_BYTES);
                db[i] = ptx::smem_desc_sw128(smem_base + i * STAGE_BYTES + GROUP_KB * A_BYTES);
            }
            // The barriers a commit arrives on: this CTA's, and in a pair the peer's too.
            auto commit = [&](uint64_t *bar) {
                if (CL == 1) {
                    ptx::mma_commit(bar);
                } else {
                    const uint32_t a = ptx::smem_u32(bar);
                    ptx::mma_commit_pair(a);
                    ptx::mma_commit_pair(ptx::mapa(a, 1));
                }
            };
            uint32_t phase = 0;
            int abuf = 0;
            uint32_t aphase = 0;
            bool ready = false; // the look-ahead test saw the next slot full
            uint32_t dt = tmem;
            // Position in the group sequence: tile, slice group d, pair s, group g
            // of the pair (gpp groups per pair), groups in the open chunk.
            int tile = cta0, d = p.d0, s = 0, g = 0, in_chunk = 0;
            int gpp = tile < total_tiles ? entry_nkb<GROUPED>(p, items, work, tile) / GROUP_KB : 0;
            auto close_chunk = [&]() {
                commit(&accf[abuf]);
                abuf ^= 1;
                if (abuf == 0) aphase ^= 1;
                in_chunk = 0;
            };
            // One group in ring slot ST; false when the sequence ended or a wait gave up.
            auto step = [&](auto slot) -> bool {
                constexpr int ST = decltype(slot)::value;
                if (in_chunk == 0) {
                    const long long ta = p.prof ? clock64() : 0;
                    const bool got_acc = ptx::mbar_wait(&acce[abuf], aphase ^ 1, p.timeout_ns, abort_flag);
                    if (p.prof) prof_add(p, kProfMmaWaitAcc, clock64() - ta);
                    if (!got_acc) {
                        raise_abort(p, abort_flag, 2, peer_flag);
                        return false;
                    }
                    dt = tmem + (uint32_t)(abuf * kBN);
                }
                if (!ready) {
                    const long long tf = p.prof ? clock64() : 0;
                    const bool got_full = ptx::mbar_wait(&full[ST], phase, p.timeout_ns, abort_flag);
                    if (p.prof) prof_add(p, kProfMmaWaitFull, clock64() - tf);
                    if (!got_full) {
                        raise_abort(p, abort_flag, 2, peer_flag);
                        return false;
                    }
                }
                ptx::tc_fence_after();
                const uint32_t nphase = ST == STAGES - 1 ? phase ^ 1 : phase;
                ready = mma_group<CL>(dt, da[ST], db[ST], idesc, in_chunk > 0 ? 1u : 0u,
                                      full_base + (uint32_t)(((ST + 1) % STAGES) * 8), nphase);
                commit(&empty[ST]);
                phase = nphase;
                if (++in_chunk == kChunkKB / GROUP_KB) close_chunk();
                if (++g == gpp) {
                    g = 0;
                    if (++s > d) {
                        s = 0;
                        if (in_chunk > 0) close_chunk(); // the slice group ends inside a chunk
                        if (++d == p.d1) {
                            d = p.d0;
                            tile += ctas;
                            if (tile >= total_tiles) return false;
                            gpp = entry_nkb<GROUPED>(p, items, work, tile) / GROUP_KB;
                        }
                    }
                }
                return true;
            };
            // one pass over the ring's slots
            auto ring = [&]() -> bool {
                if (!step(std::integral_constant<int, 0>{})) return false;
                if (!step(std::integral_constant<int, 1>{})) return false;
                if (!step(std::integral_constant<int, 2>{})) return false;
                if constexpr (STAGES == 4) {
                    if (!step(std::integral_constant<int, 3>{})) return false;
                }
                return true;
            };
            static_assert(STAGES == 3 || STAGES == 4, "the issue loop is unrolled over three or four slots");
            if (gpp > 0)
                while (ring()) {
                }
            // All issued MMAs must complete before TMEM is released.
            if (CL == 1)
                ptx::mma_commit(done);
            else
                ptx::mma_commit_pair(ptx::smem_u32(done));
            if (!ptx::mbar_wait(done, 0, DRAIN_NS, nullptr)) raise_abort(p, abort_flag, 5, peer_flag);
        }
    } else {
        // ------------------------------------------------ epilogue (warps 2..9)
        // Two warps per TMEM lane quadrant; each owns 64 of the tile's 128 columns.
        const int ew = warp - 2;              // 0..7
        const int q = warp & 3;               // TMEM lane quadrant this warp may access
        const int col0 = (ew >> 2) * (kBN / 2);
        const int row = q * 32 + lane;        // tile row owned by this thread
        const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16);
        int64_t *colOff = colOffAll + ew * (kBN / 2);
        int *colExp = colExpAll + ew * (kBN / 2);
        double *finT = finTAll + ew * (kFinCols * FIN_T);
        int64_t *rowOffW = rowOffAll + ew * 32;
        int *rowOkW = rowOkAll + ew * 32;
        int abuf = 0;
        uint32_t aphase = 0;
        bool ok = true;
        const bool plain_store = p.zero && p.cp == 0.0;
        const bool cp_one = p.cp == 1.0; // both tests once here: FP64 compares run on the slow FP64 pipe
        // The previous ("pending") tile: its int64 sums wait in this CTA's scratch
        // (column-major, so the warp's stores and loads of it are contiguous) and
        // are finished kFinCols columns at a time after each flush of the next
        // tile, so the FP64 epilogue never holds the accumulators the MMA issuer
        // is waiting for.  When C is contiguous along the rows, one thread per
        // row reads and writes C directly (consecutive lanes, consecutive rows);
        // otherwise a batch is converted with one thread per row and transposed
        // through shared memory so that the read-modify-write of C runs along a
        // row.  colOff / colExp / rowOffW / rowOkW describe the pending tile.
        long long *const rbc = p.rbuf + (size_t)blockIdx.x * kBM * kBN;
        bool pend = false, pend_row_ok = false;
        bool pend_rows_fast = false; // C is contiguous along the rows: one thread per row stays coalesced
        const long long *pend_src = rbc; // the pending tile's sums (scratch, or the K slices' accumulator)
        int pend_done = 0, pend_rowExp = 0;
        double *pend_C = nullptr;
        auto finalize_cols = [&](int upto) {
            if (pend && pend_rows_fast) {
                if (pend_row_ok) {
                    const int64_t rowOff = rowOffW[lane];
                    for (int c0 = pend_done; c0 < upto; c0 += kFinFast) {
                        long long Rv[kFinFast];
                        double old[kFinFast];
#pragma unroll
                        for (int i = 0; i < kFinFast; i++) Rv[i] = __ldcg(pend_src + (size_t)(col0 + c0 + i) * kBM + row);
                        if (!plain_store) {
#pragma unroll
                            for (int i = 0; i < kFinFast; i++)
                                old[i] = colExp[c0 + i] != INT_MAX ? pend_C[rowOff + colOff[c0 + i]] : 0.0;
                        }
#pragma unroll
                        for (int i = 0; i < kFinFast; i++) {
                            const int ce = colExp[c0 + i];
                            if (ce == INT_MAX) continue;
                            long long R = Rv[i];
                            if (p.ab_neg) R = -R;
                            double v;
                            if (pend_rowExp == INT_MIN || ce == INT_MIN)
                                v = __longlong_as_double(0x7ff8000000000000ll);
                            else
                                v = int_times_pow2_rn(R, pend_rowExp + ce + p.shift_const);
                            if (!p.ab_pow2) v *= p.ab;
                            pend_C[rowOff + colOff[c0 + i]] =
                                plain_store ? v : (cp_one ? old[i] + v : fma(p.cp, old[i], v));
                        }
                    }
                }
            } else if (pend) {
                for (int c0 = pend_done; c0 < upto; c0 += kFinCols) {
                    // Both global reads of the batch -- the old C values (lanes kFinCols*r ..
                    // kFinCols*r + kFinCols-1 take the batch's columns of row r) and the sums
                    // (one thread per row) -- are issued before either is used, so their
                    // latencies overlap instead of adding up.
                    double old[kFinCols];
                    if (!plain_store) {
#pragma unroll
                        for (int k = 0; k < kFinCols; k++) {
                            const int e = k * 32 + lane, r = e / kFinCols, c = e % kFinCols;
                            old[k] = (rowOkW[r] && colExp[c0 + c] != INT_MAX) ? pend_C[rowOffW[r] + colOff[c0 + c]] : 0.0;
                        }
                    }
                    long long Rv[kFinCols];
#pragma unroll
                    for (int i = 0; i < kFinCols; i++)
                        Rv[i] = (pend_row_ok && colExp[c0 + i] != INT_MAX)
                                    ? __ldcg(pend_src + (size_t)(col0 + c0 + i) * kBM + row)
                                    : 0ll;
#pragma unroll
                    for (int i = 0; i < kFinCols; i++) {
                        const int ce = colExp[c0 + i];
                        double v = 0.0;
                        if (pend_row_ok && ce != INT_MAX) {
                            long long R = Rv[i];
                            if (p.ab_neg) R = -R;
                            if (pend_rowExp == INT_MIN || ce == INT_MIN)
                                v = __longlong_as_double(0x7ff8000000000000ll);
                            else
                                v = int_times_pow2_rn(R, pend_rowExp + ce + p.shift_const);
                            if (!p.ab_pow2) v *= p.ab;
                        }
                        finT[i * FIN_T + lane] = v;
                    }
                    __syncwarp();
#pragma unroll
                    for (int k = 0; k < kFinCols; k++) {
                        const int e = k * 32 + lane, r = e / kFinCols, c = e % kFinCols;
                        if (rowOkW[r] && colExp[c0 + c] != INT_MAX) {
                            const double v = finT[c * FIN_T + r];
                            pend_C[rowOffW[r] + colOff[c0 + c]] =
                                plain_store ? v : (cp_one ? old[k] + v : fma(p.cp, old[k], v));
                        }
                    }
                    __syncwarp();
                }
            }
            pend_done = upto;
        };
        for (int tile = cta0; tile < total_tiles && ok; tile += ctas) {
            // Only the K block count is held through the chunks; the rest of the
            // tile's description is resolved at its end (registers are scarce here).
            const int nkb = entry_nkb<GROUPED>(p, items, work, tile);
            // Running sum of this thread's 64 outputs, R = H + L: L (int32, registers)
            // takes every chunk, H (int64, TMEM columns 256..511) is written only when
            // L is folded in -- at the end of each slice group (Horner step R *= 256)
            // and every 64 chunks (|L| < 64 * 2^24 = 2^30).  Keeping the per-chunk
            // work free of TMEM stores matters: a tcgen05.st from the epilogue warps
            // that share the MMA issuer's sub-partition stalls the issue.
            int32_t L[kBN / 2];
#pragma unroll
            for (int i = 0; i < kBN / 2; i++) L[i] = 0;
            bool hvalid = false; // H holds a part of the sum (else it reads as 0)
            int since_fold = 0;
            for (int d = p.d0; d < p.d1 && ok; d++) {
                const int kbs = (d + 1) * nkb;
                for (int c0 = 0; c0 < kbs; c0 += kChunkKB) {
                    const long long tw = (p.prof && ew == 0 && lane == 0) ? clock64() : 0;
                    bool w = ptx::mbar_wait(&accf[abuf], aphase, p.timeout_ns, abort_flag);
                    const long long tw1 = (p.prof && ew == 0 && lane == 0) ? clock64() : 0;
                    if (p.prof && ew == 0 && lane == 0) prof_add(p, kProfEpiWaitAcc, tw1 - tw);
                    w = __all_sync(0xffffffffu, w);
                    if (!w) {
                        if (lane == 0) raise_abort(p, abort_flag, 3, peer_flag);
                        ok = false;
                        break;
                    }
                    ptx::tc_fence_after();
#pragma unroll
                    for (int cc = 0; cc < kBN / 32; cc++) {
                        uint32_t acc[16];
                        ptx::tmem_ld16(tl + (uint32_t)(abuf * kBN + col0 + cc * 16), acc);
                        ptx::tmem_wait_ld();
#pragma unroll
                        for (int i = 0; i < 16; i++) L[cc * 16 + i] += __float2int_rn(__uint_as_float(acc[i]));
                    }
                    ptx::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) {
                        if (CL == 1)
                            ptx::mbar_arrive(&acce[abuf]);
                        else
                            ptx::mbar_arrive_cluster_relaxed(acce_lead + (uint32_t)(abuf * 8));
                    }
                    abuf ^= 1;
                    if (abuf == 0) aphase ^= 1;
                    // Fold L into H every 64 chunks and at the end of each slice group,
                    // with the Horner step R *= 256 before the next one; after the last
                    // slice group H holds the tile's sums and L is free.
                    const bool group_end = c0 + kChunkKB >= kbs;
                    const bool shift = group_end && d + 1 < p.d1;
                    if (++since_fold == 64 || group_end) {
#pragma unroll
                        for (int cc = 0; cc < kBN / 16; cc++) {
                            const uint32_t col = (uint32_t)(col0 + cc * 8);
                            uint32_t lo[8], hi[8];
                            if (hvalid) {
                                ptx::tmem_ld8(tl + 256u + col, lo);
                                ptx::tmem_ld8(tl + 384u + col, hi);
                                ptx::tmem_wait_ld();
                            }
#pragma unroll
                            for (int i = 0; i < 8; i++) {
                                long long H = hvalid ? (long long)(((unsigned long long)hi[i] << 32) | lo[i]) : 0ll;
                                H += L[cc * 8 + i];
                                if (shift) H *= 256;
                                lo[i] = (uint32_t)((unsigned long long)H);
                                hi[i] = (uint32_t)((unsigned long long)H >> 32);
                                L[cc * 8 + i] = 0;
                            }
                            ptx::tmem_st8(tl + 256u + col, lo);
                            ptx::tmem_st8(tl + 384u + col, hi);
                            ptx::tmem_wait_st();
                        }
                        hvalid = true;
                        since_fold = 0;
                    }
                    if (p.prof && ew == 0 && lane == 0) prof_add(p, kProfEpiFlush, clock64() - tw1);
                    // a slice of the pending tile while the MMAs run
                    if (pend_done < kBN / 2) finalize_cols(pend_done + (pend_rows_fast ? kFinFast : kFinCols));
                }
            }
            if (!ok) break;
            // end of tile: finish the pending tile, park this tile's sums in the
            // scratch, and make this tile the pending one
            const long long tfin = (p.prof && ew == 0 && lane == 0) ? clock64() : 0;
            finalize_cols(kBN / 2);
            __syncwarp();
            const TileJob job = resolve<GROUPED, CL>(p, items, work, tile, rank);
            if (!GROUPED && job.tid < 0) {
                // the odd half of a pair's last row of tiles: rows past the output
                ptx::tc_fence_before();
                pend = false;
                continue;
            }
            const int64_t m = (int64_t)job.mt * kBM + row;
            const bool row_ok = m < job.M;
            int64_t rowOff = 0;
            int rowExp = 0;
            if (row_ok) {
                int64_t oa, ob;
                group_offsets32(*job.mg, (uint32_t)m, oa, ob, rowOff);
                rowExp = job.eA[m];
            }
            // Short-K tiles (few chunks: the deferred finishing would run longer than
            // the next tile's MMAs) are finished here, straight from TMEM.
            const bool direct = p.ksplit == 1 && nkb <= kDirectKB;
            // K slices add their sums into the tile's accumulator; only the last
            // one to arrive at this warp's region finishes it
            long long *const dst = p.ksplit > 1 ? p.racc + (size_t)job.tid * kBM * kBN : rbc;
#pragma unroll 1
            for (int cc = 0; cc < kBN / 32 && !direct; cc++) {
                const uint32_t col = (uint32_t)(col0 + cc * 16);
                uint32_t lo[16], hi[16];
                ptx::tmem_ld16(tl + 256u + col, lo);
                ptx::tmem_ld16(tl + 384u + col, hi);
                ptx::tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const unsigned long long R = ((unsigned long long)hi[i] << 32) | lo[i];
                    long long *q = dst + (size_t)(col0 + cc * 16 + i) * kBM + row;
                    if (p.ksplit > 1)
                        atomicAdd((unsigned long long *)q, R); // two's complement: exact for signed sums
                    else
                        *q = (long long)R;
                }
            }
            ptx::tc_fence_before();
            bool finish = true;
            if (p.ksplit > 1) {
                __threadfence();
                __syncwarp();
                int last = 0;
                if (lane == 0) last = atomicAdd(p.rcnt + job.tid * 8 + ew, 1) == p.ksplit - 1;
                finish = __shfl_sync(0xffffffffu, last, 0) != 0;
                if (finish) __threadfence();
            }
            for (int i = lane; i < kBN / 2; i += 32) {
                const int64_t n = (int64_t)job.nt * kBN + col0 + i;
                int64_t oa, ob, oc = 0;
                int ex = INT_MAX; // marks a column beyond N
                if (n < job.N) {
                    group_offsets32(*job.ng, (uint32_t)n, oa, ob, oc);
                    ex = job.eB[n];
                }
                colOff[i] = oc;
                colExp[i] = ex;
            }
            __syncwarp();
            rowOffW[lane] = rowOff;
            rowOkW[lane] = row_ok ? 1 : 0;
            __syncwarp();
            if (direct) {
                // the same conversion and stores as finalize_cols, the sums read from TMEM
                const bool rows_fast = job.mg->n > 0 && job.mg->s[2][job.mg->n - 1] == 1;
                double *const Cj = job.C;
                if constexpr (GROUPED) {
                    // grouped tiles (mostly partial, written once with C_prefactor 0): one
                    // column at a time measured faster than loading C ahead
#pragma unroll 1
                    for (int cc = 0; cc < kBN / 32; cc++) {
                        uint32_t lo[16], hi[16];
                        ptx::tmem_ld16(tl + 256u + (uint32_t)(col0 + cc * 16), lo);
                        ptx::tmem_ld16(tl + 384u + (uint32_t)(col0 + cc * 16), hi);
                        ptx::tmem_wait_ld();
#pragma unroll
                        for (int b = 0; b < 16; b += kFinCols) {
                            const int c0 = cc * 16 + b;
                            double v[kFinCols];
#pragma unroll
                            for (int i = 0; i < kFinCols; i++) {
                                const int ce = colExp[c0 + i];
                                v[i] = 0.0;
                                if (row_ok && ce != INT_MAX) {
                                    long long R = (long long)(((unsigned long long)hi[b + i] << 32) | lo[b + i]);
                                    if (p.ab_neg) R = -R;
                                    if (rowExp == INT_MIN || ce == INT_MIN)
                                        v[i] = __longlong_as_double(0x7ff8000000000000ll);
                                    else
                                        v[i] = int_times_pow2_rn(R, rowExp + ce + p.shift_const);
                                    if (!p.ab_pow2) v[i] *= p.ab;
                                }
                            }
                            if (rows_fast) {
                                if (row_ok) {
#pragma unroll
                                    for (int i = 0; i < kFinCols; i++) {
                                        if (colExp[c0 + i] == INT_MAX) continue;
                                        double *const cp_ = Cj + rowOff + colOff[c0 + i];
                                        *cp_ = plain_store ? v[i] : (cp_one ? *cp_ + v[i] : fma(p.cp, *cp_, v[i]));
                                    }
                                }
                            } else {
#pragma unroll
                                for (int i = 0; i < kFinCols; i++) finT[i * FIN_T + lane] = v[i];
                                __syncwarp();
                                // lanes kFinCols*r .. kFinCols*r + kFinCols-1 take the batch's columns of row r
#pragma unroll
                                for (int k = 0; k < kFinCols; k++) {
                                    const int e = k * 32 + lane, r = e / kFinCols, c = e % kFinCols;
                                    if (rowOkW[r] && colExp[c0 + c] != INT_MAX) {
                                        const double w = finT[c * FIN_T + r];
                                        double *const cp_ = Cj + rowOffW[r] + colOff[c0 + c];
                                        *cp_ = plain_store ? w : (cp_one ? *cp_ + w : fma(p.cp, *cp_, w));
                                    }
                                }
                                __syncwarp();
                            }
                        }
                    }
                } else {
#pragma unroll 1
                    for (int cc = 0; cc < kBN / 32; cc++) {
                        // per batch, C's old values are loaded first, all at once (a load after
                        // each store would wait a full memory round trip per column, since the
                        // stores may alias later loads), then converted sums are added and stored
                        constexpr int NB = 16 / kFinCols; // batches per block
                        uint32_t lo[16], hi[16];
                        ptx::tmem_ld16(tl + 256u + (uint32_t)(col0 + cc * 16), lo);
                        ptx::tmem_ld16(tl + 384u + (uint32_t)(col0 + cc * 16), hi);
                        ptx::tmem_wait_ld();
#pragma unroll
                        for (int bb = 0; bb < NB; bb++) {
                            const int b = bb * kFinCols;
                            const int c0 = cc * 16 + b;
                            double old[kFinCols];
#pragma unroll
                            for (int i = 0; i < kFinCols; i++) old[i] = 0.0;
                            if (!plain_store) {
#pragma unroll
                                for (int i = 0; i < kFinCols; i++) {
                                    if (rows_fast) {
                                        if (row_ok && colExp[c0 + i] != INT_MAX) old[i] = Cj[rowOff + colOff[c0 + i]];
                                    } else {
                                        // lanes kFinCols*r .. kFinCols*r + kFinCols-1 take the batch's columns of row r
                                        const int e = i * 32 + lane, r = e / kFinCols, c = e % kFinCols;
                                        if (rowOkW[r] && colExp[c0 + c] != INT_MAX) old[i] = Cj[rowOffW[r] + colOff[c0 + c]];
                                    }
                                }
                            }
                            double v[kFinCols];
#pragma unroll
                            for (int i = 0; i < kFinCols; i++) {
                                const int ce = colExp[c0 + i];
                                v[i] = 0.0;
                                if (row_ok && ce != INT_MAX) {
                                    long long R = (long long)(((unsigned long long)hi[b + i] << 32) | lo[b + i]);
                                    if (p.ab_neg) R = -R;
                                    if (rowExp == INT_MIN || ce == INT_MIN)
                                        v[i] = __longlong_as_double(0x7ff8000000000000ll);
                                    else
                                        v[i] = int_times_pow2_rn(R, rowExp + ce + p.shift_const);
                                    if (!p.ab_pow2) v[i] *= p.ab;
                                }
                            }
                            if (rows_fast) {
                                if (row_ok) {
#pragma unroll
                                    for (int i = 0; i < kFinCols; i++) {
                                        if (colExp[c0 + i] == INT_MAX) continue;
                                        Cj[rowOff + colOff[c0 + i]] =
                                            plain_store ? v[i] : (cp_one ? old[i] + v[i] : fma(p.cp, old[i], v[i]));
                                    }
                                }
                            } else {
#pragma unroll
                                for (int i = 0; i < kFinCols; i++) finT[i * FIN_T + lane] = v[i];
                                __syncwarp();
#pragma unroll
                                for (int k = 0; k < kFinCols; k++) {
                                    const int e = k * 32 + lane, r = e / kFinCols, c = e % kFinCols;
                                    if (rowOkW[r] && colExp[c0 + c] != INT_MAX) {
                                        const double w = finT[c * FIN_T + r];
                                        Cj[rowOffW[r] + colOff[c0 + c]] =
                                            plain_store ? w : (cp_one ? old[k] + w : fma(p.cp, old[k], w));
                                    }
                                }
                                __syncwarp();
                            }
                        }
                    }
                }
                ptx::tc_fence_before();
                finish = false; // nothing left pending
            }
            pend = finish;
            pend_src = dst;
            pend_done = 0;
            pend_row_ok = row_ok;
            pend_rows_fast = job.mg->n > 0 && job.mg->s[2][job.mg->n - 1] == 1;
            pend_rowExp = rowExp;
            pend_C = job.C;
            if (p.prof && ew == 0 && lane == 0) prof_add(p, kProfEpiFinal, clock64() - tfin);
        }
        if (ok) finalize_cols(kBN / 2);
    }

    __syncthreads();
    // A CTA of a pair leaves only when the peer is done too: the even CTA's MMAs
    // read the odd CTA's shared memory, and both CTAs arrive on each other's barriers.
    if (CL == 2) ptx::cluster_sync();
    if (p.prof && threadIdx.x == 0) prof_add(p, kProfTotal, clock64() - t_start);
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc<CL>(tmem, TMEM_COLS);
    }
}

} // namespace

eg_status ensure_tc_attributes() {
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        err = cudaFuncSetAttribute(k_tc_split_gemm<false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   Ring<1>::SMEM_BYTES);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_tc_split_gemm<true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       Ring<1>::SMEM_BYTES);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_tc_split_gemm<false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       Ring<2>::SMEM_BYTES);
    });
    if (err != cudaSuccess) return cuda_fail(err, "cudaFuncSetAttribute(k_tc_split_gemm)");
    return EG_SUCCESS;
}

namespace {
cudaLaunchConfig_t pair_config(int grid, cudaStream_t s, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = Ring<2>::SMEM_BYTES;
    cfg.stream = s;
    attr->id = cudaLaunchAttributeClusterDimension;
    attr->val.clusterDim.x = 2;
    attr->val.clusterDim.y = 1;
    attr->val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}
} // namespace

int tc_pair_clusters() {
    static std::once_flag once;
    static int n = 0;
    std::call_once(once, [] {
        // CTA pairs only on request: on the CCD shapes they measure slower than
        // single-CTA tiles (the epilogue, not operand delivery, bounds the kernel)
        const char *env = std::getenv("EINSUMS_GB300_TC_PAIRS");
        if (!env || env[0] != '1') return;
        if (ensure_tc_attributes() != EG_SUCCESS) return;
        cudaLaunchAttribute attr;
        cudaLaunchConfig_t cfg = pair_config(num_sms(), nullptr, &attr);
        int c = 0;
        if (cudaOccupancyMaxActiveClusters(&c, (void *)k_tc_split_gemm<false, 2>, &cfg) == cudaSuccess) n = c;
        cudaGetLastError();
    });
    return n;
}

eg_status launch_tc_gemm(const CUtensorMap &tmA, const CUtensorMap &tmB, const TcGemmParams &p, cudaStream_t s) {
    eg_status st = ensure_tc_attributes();
    if (st != EG_SUCCESS) return st;
    if (p.pair) {
        const int clusters = tc_pair_clusters();
        if (clusters < 1) return fail(EG_ERROR_CUDA, "k_tc_split_gemm: CTA pairs are not available");
        const int total = p.nbatch * ((p.mtiles + 1) / 2) * p.ntiles * p.ksplit;
        if (total <= 0) return EG_SUCCESS;
        const int grid = 2 * (total < clusters ? total : clusters);
        cudaLaunchAttribute attr;
        cudaLaunchConfig_t cfg = pair_config(grid, s, &attr);
        {
            LaunchScope ls_("k_tc_split_gemm", s);
            const TcItem *no_items = nullptr;
            const int4 *no_work = nullptr;
            EG_CUDA(cudaLaunchKernelEx(&cfg, k_tc_split_gemm<false, 2>, tmA, tmB, p, no_items, no_work, 0));
        }
        EG_CHECK_LAUNCH("k_tc_split_gemm");
        return EG_SUCCESS;
    }
    const int total = p.nbatch * p.mtiles * p.ntiles * p.ksplit;
    if (total <= 0) return EG_SUCCESS;
    const int grid = total < num_sms() ? total : num_sms();
    {
        LaunchScope ls_("k_tc_split_gemm", s);
        k_tc_split_gemm<false, 1><<<grid, THREADS, Ring<1>::SMEM_BYTES, s>>>(tmA, tmB, p, nullptr, nullptr, 0);
    }
    EG_CHECK_LAUNCH("k_tc_split_gemm");
    return EG_SUCCESS;
}

eg_status launch_tc_gemm_grouped(const CUtensorMap &tmA, const CUtensorMap &tmB, const TcGemmParams &p,
                                 const TcItem *items, const int4 *work, int ntiles_total, cudaStream_t s) {
    eg_status st = ensure_tc_attributes();
    if (st != EG_SUCCESS) return st;
    if (ntiles_total <= 0) return EG_SUCCESS;
    const int grid = ntiles_total < num_sms() ? ntiles_total : num_sms();
    {
        LaunchScope ls_("k_tc_split_gemm_grouped", s);
        k_tc_split_gemm<true, 1><<<grid, THREADS, Ring<1>::SMEM_BYTES, s>>>(tmA, tmB, p, items, work, ntiles_total);
    }
    EG_CHECK_LAUNCH("k_tc_split_gemm_grouped");
    return EG_SUCCESS;
}

} // namespace eg::split

extern "C" eg_status eg_tc_pair_clusters(int32_t *clusters) {
    if (!clusters) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "eg_tc_pair_clusters: NULL output");
    *clusters = eg::split::tc_pair_clusters();
    return EG_SUCCESS;
}
