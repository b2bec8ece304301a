// V-list M2L of the mixed-precision path on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// Per operator o (level, lattice offset) the V-list pairs form a dense contraction
//     L[tgt_j] += K_o . M[src_j]        K_o: 4p^3 x 4p^3,  j = pairs of the operator
// computed as D[128 rows x 128 pairs] (FP32, in TMEM) += A[128 x K] . B[K x 128 pairs].  FP32
// accuracy comes from a three-product split, A = A_hi + A_lo, B = B_hi + B_lo, D accumulating
// A_hi.B_hi + A_hi.B_lo + A_lo.B_hi (the dropped A_lo.B_lo is below FP32 rounding), in one of two
// operand forms: scaled FP16 (the default: operator rows and multipole columns scaled by powers
// of two, kind::f16 MMAs with K = 16) or TF32 (IBIM_TC_FP16=0: kind::tf32, K = 8).
//
// One CTA takes one chunk of up to 128 pairs of an operator against up to four 128-row tiles of
// the operator (four FP32 accumulators of 128 x 128 = all 512 TMEM columns), so each gathered
// multipole is read once per chunk rather than once per row tile.  Operands sit in shared memory
// in the canonical no-swizzle K-major layout (8-row x 16-byte core matrices; K-direction
// core-matrix stride 128 B, row-group stride 256 B), 8 K-elements per stage, five stage buffers.
// The operator tiles are pre-packed in that layout and arrive by bulk asynchronous copies; the
// multipole rows are gathered by cp.async.  Warp roles (copy issue, MMA issue, gather) meet only
// on mbarriers; every wait is bounded and reports through an error flag instead of hanging.  The
// epilogue reads the accumulators with tcgen05.ld (each warp its 32 TMEM lanes) and adds them
// into the target nodes' local expansions.

#include <cstdint>
#include <cstdlib>
#include <type_traits>

#include <cuda_fp16.h>

#include "fmm_common.cuh"

namespace ibim {

namespace {

constexpr int TC_M = 128, TC_KS = 8;               // rows per tile, K elements per stage
constexpr int TC_THREADS = 256;
constexpr int TC_TILE_BYTES = TC_M * TC_KS * 4;    // 4 KB per operator tile and stage
constexpr long TC_WAIT_LIMIT = 1L << 20;           // bounded mbarrier polling

// FP16 operand form: K elements per stage (a stage row is 32 bytes in both forms)
constexpr int TC_KS16 = 16;

// Shape of the contraction for N pairs per chunk (MMA N) against RT row tiles of 128 operator
// rows, CPS CTAs resident per SM: RT N TMEM columns per CTA (all 512 for CPS 1); a stage holds RT
// operator tiles (hi, lo) and the N multipole rows (hi, lo).
template <int N, int RT_ = 512 / N, int CPS = 1> struct TcShape {
    static constexpr int RT = RT_;
    static_assert(RT * N * CPS <= 512, "TMEM columns of the resident CTAs");
    static constexpr int BT = N * TC_KS * 4;                           // multipole tile bytes
    static constexpr int STAGE = 2 * RT * TC_TILE_BYTES + 2 * BT;       // 40 KB (N 128, RT 4)
    static constexpr int NST = ((CPS == 1 ? 200 : 96) * 1024) / STAGE;  // 5 (RT 4) or 4 (RT 2, CPS 2)
    static constexpr int SMEM = NST * STAGE;
    // stages of multipole copies a gathering thread keeps in flight before it signals the oldest:
    // one (a deeper lag makes a stage's signal wait for a later stage's buffer, i.e. for an older
    // stage's MMAs; lag 1 against NST - 2 measured 2.63 against 2.67 ms a launch in the one-CTA
    // form of four row tiles, equal in the default form)
    static constexpr int LAG = 1;
    // D FP32, A and B TF32, both K-major, M = 128, N.
    static constexpr uint32_t IDESC =
        (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
    // D FP32, A and B FP16 (kind::f16), both K-major, M = 128, N.
    static constexpr uint32_t IDESC16 =
        (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor, no swizzle, K-major.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void *g, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(saddr), "l"(g), "r"(src_bytes));
}

// Wait for the mbarrier phase with the given parity; false when the bound is exceeded.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (long it = 0; it < TC_WAIT_LIMIT; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Byte offset of element (row, 4 * kchunk) of a 128 x 8 tile in the canonical no-swizzle
// K-major layout: core matrix (row / 8, kchunk) at ((row / 8) * 2 + kchunk) * 128, row % 8 at 16 B.
// Descriptor strides: 128 B between the two core matrices along K, 256 B between row groups.
__device__ __forceinline__ uint32_t tile_off(int row, int kchunk) {
    return (uint32_t)((((row >> 3) << 1) + kchunk) * 128 + (row & 7) * 16);
}

// One CTA: one chunk of <= N V pairs of a single operator x up to RT row tiles of 128
// operator rows.  Stage st holds K elements [8 st, 8 st + 8) of A_hi, A_lo (per row tile, pre-packed
// as contiguous 4 KB blocks in the shared-memory layout) and of B_hi, B_lo in buffer st % TC_NST.
// Warp-specialised: warp 0 (one thread) issues the operator bulk copies, warp 1 (one thread)
// issues the MMAs, warps 2-7 gather the multipole rows with cp.async.
// Per stage buffer: full_a (bulk copies, transaction count), full_b (the 192 gathering threads,
// each after its own copies of the stage have landed and been fenced to the async proxy), empty
// (tcgen05.commit of the stage's MMAs).  No CTA-wide barrier inside the K loop; every wait is
// bounded and an expired wait aborts the CTA through a shared flag and the error word.
constexpr int TC_BPROD = 192;

template <int N, bool H16, int RT = 512 / N, int CPS = 1>
__global__ void __launch_bounds__(TC_THREADS, CPS)
    k_m2l_tc(int n4, int kpad, int mtiles, const int *__restrict__ chunks, const int *__restrict__ vsrc,
                const int *__restrict__ vtgt, const void *__restrict__ a_hi_, const void *__restrict__ a_lo_,
                const void *__restrict__ b_hi_, const void *__restrict__ b_lo_, const float *__restrict__ rscale,
                const float *__restrict__ cscale, float *local, int *err, const int *__restrict__ chunk_mol,
                const int *__restrict__ mol_active, const MolImg *__restrict__ mol_img) {
    // a merged plan (batch.cu): chunks of molecules that have stopped iterating are skipped whole,
    // the others read their molecule's own operator images
    if (chunk_mol) {
        const int m = chunk_mol[blockIdx.x];
        if (!mol_active[m]) return;
        a_hi_ = mol_img[m].tc_hi;
        a_lo_ = mol_img[m].tc_lo;
        rscale = mol_img[m].tc_rsc;
    }
    using SH = TcShape<N, RT, CPS>;
    constexpr int TC_RT = SH::RT, TC_NST = SH::NST, TC_LAG = SH::LAG;
    constexpr int KS = H16 ? TC_KS16 : TC_KS, ES = H16 ? 2 : 4;  // K elements per stage, bytes per element
    const char *a_hi = static_cast<const char *>(a_hi_), *a_lo = static_cast<const char *>(a_lo_);
    const char *b_hi = static_cast<const char *>(b_hi_), *b_lo = static_cast<const char *>(b_lo_);
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t full_a[TC_NST], full_b[TC_NST], empty_bar[TC_NST], acc_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int src_s[N], tgt_s[N];
    __shared__ float csc_s[N];
    __shared__ volatile int abort_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int op = chunks[3 * blockIdx.x], b = chunks[3 * blockIdx.x + 1], cnt = chunks[3 * blockIdx.x + 2];
    const int tile0 = blockIdx.y * TC_RT;
    const int rt = min(TC_RT, mtiles - tile0);
    const int nstage = kpad / KS;
    // MMA width of this chunk: its pairs rounded up to 16 (the last chunk of an operator is
    // partial), set in the instruction descriptor's N field; gathers and epilogue stop there too
    const int neff = max(16, (cnt + 15) & ~15);
    constexpr uint32_t NMASK = 0x3Fu << 17;
    const uint32_t idesc16 = (SH::IDESC16 & ~NMASK) | ((uint32_t)(neff >> 3) << 17);
    const uint32_t idesc32 = (SH::IDESC & ~NMASK) | ((uint32_t)(neff >> 3) << 17);
    constexpr int kStageBytes = SH::STAGE;
    for (int i = tid; i < N; i += TC_THREADS) {
        src_s[i] = i < cnt ? vsrc[b + i] : -1;
        tgt_s[i] = i < cnt ? vtgt[b + i] : -1;
        if (H16) csc_s[i] = i < cnt ? cscale[src_s[i]] : 0.f;
    }
    if (tid == 0) {
        abort_s = 0;
        for (int i = 0; i < TC_NST; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_a[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_b[i])), "r"(TC_BPROD));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty_bar[i])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_bar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(TC_RT * N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem_d = tmem_base;
    const long atile0 = ((long)op * mtiles + tile0) * nstage;

    if (warp == 0) {
        if (lane == 0) {  // operator tiles: bulk copies
            int issued = -1;
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % TC_NST;
                if (st >= TC_NST &&
                    !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((st / TC_NST) - 1) & 1))) {
                    abort_s = 1;
                    break;
                }
                if (abort_s) break;
                unsigned char *base = tc_smem + buf * kStageBytes;
                const uint32_t fb = smem_u32(&full_a[buf]);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb),
                             "r"(2 * rt * TC_TILE_BYTES)
                             : "memory");
                for (int t = 0; t < rt; ++t) {
                    const long g = (atile0 + (long)t * nstage + st) * TC_TILE_BYTES;
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                            smem_u32(base + t * TC_TILE_BYTES)),
                        "l"(a_hi + g), "r"(TC_TILE_BYTES), "r"(fb)
                        : "memory");
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                            smem_u32(base + (rt + t) * TC_TILE_BYTES)),
                        "l"(a_lo + g), "r"(TC_TILE_BYTES), "r"(fb)
                        : "memory");
                }
                issued = st;
            }
            // every issued copy lands before the CTA may exit (the last use of each buffer)
            for (int s2 = max(0, issued - TC_NST + 1); s2 <= issued; ++s2)
                if (!mbar_wait(smem_u32(&full_a[s2 % TC_NST]), (uint32_t)((s2 / TC_NST) & 1))) abort_s = 1;
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issue
            int last = -1;
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % TC_NST;
                const uint32_t par = (uint32_t)((st / TC_NST) & 1);
                if (!mbar_wait(smem_u32(&full_a[buf]), par) || !mbar_wait(smem_u32(&full_b[buf]), par) || abort_s) {
                    abort_s = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t base = smem_u32(tc_smem + buf * kStageBytes);
                const uint64_t bh = make_desc(base + (2 * rt) * TC_TILE_BYTES, 128, 256);
                const uint64_t bl = make_desc(base + (2 * rt) * TC_TILE_BYTES + SH::BT, 128, 256);
                for (int t = 0; t < rt; ++t) {
                    const uint64_t ah = make_desc(base + t * TC_TILE_BYTES, 128, 256);
                    const uint64_t al = make_desc(base + (rt + t) * TC_TILE_BYTES, 128, 256);
                    const uint32_t d = tmem_d + (uint32_t)(t * N);
                    if (H16) {
                        mma_f16(d, ah, bh, idesc16, st > 0 ? 1u : 0u);
                        mma_f16(d, ah, bl, idesc16, 1u);
                        mma_f16(d, al, bh, idesc16, 1u);
                    } else {
                        mma_tf32(d, ah, bh, idesc32, st > 0 ? 1u : 0u);
                        mma_tf32(d, ah, bl, idesc32, 1u);
                        mma_tf32(d, al, bh, idesc32, 1u);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&empty_bar[buf]))
                             : "memory");
                last = st;
            }
            if (last == nstage - 1) {
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&acc_bar))
                             : "memory");
            } else {
                abort_s = 1;
                if (last >= 0) mbar_wait(smem_u32(&empty_bar[last % TC_NST]), (uint32_t)((last / TC_NST) & 1));
            }
        }
    } else {  // multipole rows: cp.async by 192 threads
        // each thread fills the same (tile, row, 16-byte piece) slots of every stage: up to
        // ceil(4 N / 192) of them, addressed once here; a stage only adds its K offset.  (Arrivals
        // made by the hardware on copy completion, cp.async.mbarrier.arrive.noinc with the proxy
        // fence in the MMA thread, measured slower here: 2.38 -> 2.49 ms a launch.)
        const int t = tid - 64;
        constexpr int MAXS = (4 * N + TC_BPROD - 1) / TC_BPROD;
        uint32_t soff[MAXS], sbytes[MAXS];
        const char *gsrc[MAXS];
        int nsl = 0;
#pragma unroll
        for (int q = 0; q < MAXS; ++q) {
            const int i = t + q * TC_BPROD;
            soff[q] = 0;
            sbytes[q] = 0;
            gsrc[q] = b_hi;
            if (i < 4 * neff) {
                const int tile = i / (2 * neff), row = (i >> 1) % neff, c = i & 1;
                const int sn = src_s[row];
                soff[q] = 2 * rt * TC_TILE_BYTES + tile * SH::BT + tile_off(row, c);
                sbytes[q] = sn >= 0 ? 16u : 0u;
                gsrc[q] = (tile == 0 ? b_hi : b_lo) + (sn >= 0 ? (long)sn * kpad * ES + 16 * c : 0);
                nsl = q + 1;
            }
        }
        int issued = -1;
        for (int st = 0; st < nstage; ++st) {
            const int buf = st % TC_NST;
            if (st >= TC_NST && !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((st / TC_NST) - 1) & 1))) {
                abort_s = 1;
                break;
            }
            if (abort_s) break;
            const uint32_t base = smem_u32(tc_smem + buf * kStageBytes);
            const long koff = (long)st * KS * ES;
#pragma unroll
            for (int q = 0; q < MAXS; ++q)
                if (q < nsl) cp_async16(base + soff[q], sbytes[q] ? gsrc[q] + koff : gsrc[q], sbytes[q]);
            asm volatile("cp.async.commit_group;");
            issued = st;
            if (st >= TC_LAG) {
                asm volatile("cp.async.wait_group %0;" ::"n"(TC_LAG) : "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_b[(st - TC_LAG) % TC_NST]))
                             : "memory");
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int s2 = max(0, issued - TC_LAG + 1); s2 <= issued; ++s2)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_b[s2 % TC_NST])) : "memory");
    }
    __syncthreads();
    bool ok = !abort_s;
    if (ok) ok = mbar_wait(smem_u32(&acc_bar), 0u);
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (!ok && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (ok) {
        // Each warp turns its 32 rows x 16 pairs through a 2 KB tile of the (now idle) stage
        // buffers, so that a thread adds 4 consecutive rows of one target's local expansion with
        // one vector atomic: a quarter of the atomic instructions.  4p^3 is a multiple of 4, so a
        // group of 4 rows is all below n4 or all above, and every group is 16-byte aligned.
        const int lg = warp & 3;
        float *tp = reinterpret_cast<float *>(tc_smem) + warp * 512;  // [16 pairs][32 rows]
        for (int tt = warp >> 2; tt < rt; tt += 2) {
            const int rowb = (tile0 + tt) * TC_M + 32 * lg;  // the warp's first row
            const float rs = H16 ? rscale[(long)op * mtiles * TC_M + rowb + lane] : 1.f;  // < mtiles * 128
            const uint32_t taddr = tmem_d + ((uint32_t)(32 * lg) << 16) + (uint32_t)(tt * N);
#pragma unroll 1
            for (int c0 = 0; c0 < neff; c0 += 16) {
                uint32_t v[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15}, [%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(taddr + (uint32_t)c0));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int q = 0; q < 16; ++q)
                    tp[q * 32 + lane] = H16 ? __uint_as_float(v[q]) * rs * csc_s[c0 + q] : __uint_as_float(v[q]);
                __syncwarp();
#pragma unroll
                for (int hq = 0; hq < 4; ++hq) {
                    const int j = lane + 32 * hq;            // float4 j: pair j / 8, rows 4 (j % 8) .. + 3
                    const int q = j >> 3, r = rowb + 4 * (j & 7);
                    const int tg = tgt_s[c0 + q];
                    if (tg >= 0 && r < n4) {
                        const float4 x = *reinterpret_cast<const float4 *>(tp + q * 32 + 4 * (j & 7));
                        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(local + (long)tg * n4 + r),
                                     "f"(x.x), "f"(x.y), "f"(x.z), "f"(x.w)
                                     : "memory");
                    }
                }
                __syncwarp();
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(TC_RT * N));
}

// Persistent form of the scaled FP16 contraction: one CTA per SM walks work units u = blockIdx.x,
// blockIdx.x + gridDim.x, ... (unit = chunk u / 2 against row tiles 2 (u % 2), + 1), so the
// copies and gathers of the next unit stream while the current one's MMAs run, and its
// accumulators (two slots of 2 x N TMEM columns) drain while the next unit's MMAs fill the other
// slot.  Roles: warp 0 (one thread) bulk-copies the operator tiles, warp 1 (one thread) issues
// the MMAs, the next TCP_BPROD / 32 warps gather the multipole rows, the last four drain the
// accumulators (warp w reads TMEM lanes 32 (w % 4) .. + 31).  The stage ring (NST buffers of 2 row tiles) runs across
// unit boundaries; every wait is bounded and an expired wait aborts the CTA through a shared
// flag and the error word, after the copies and MMAs already issued have completed.
constexpr int TCP_BPROD = 256, TCP_EPI = 128, TCP_THREADS = 64 + TCP_BPROD + TCP_EPI, TCP_RT = 2;
constexpr int TCP_EPI_WARP0 = (64 + TCP_BPROD) / 32;  // first epilogue warp
constexpr int TCP_STAGE = 2 * TCP_RT * TC_TILE_BYTES + 2 * 128 * TC_KS * 4;  // 24 KB
constexpr int TCP_NST = 8, TCP_LAG = 4;
constexpr int TCP_SMEM = TCP_NST * TCP_STAGE;                               // 192 KB

__global__ void __launch_bounds__(TCP_THREADS, 1)
    k_m2l_tc_persist(int n4, int kpad, int mtiles, int nunits, const int *__restrict__ chunks,
                     const int *__restrict__ vsrc, const int *__restrict__ vtgt, const void *__restrict__ a_hi_,
                     const void *__restrict__ a_lo_, const void *__restrict__ b_hi_, const void *__restrict__ b_lo_,
                     const float *__restrict__ rscale, const float *__restrict__ cscale, float *local, int *err) {
    constexpr int N = 128, KS = TC_KS16, ES = 2, BT = N * TC_KS * 4;
    const char *a_hi = static_cast<const char *>(a_hi_), *a_lo = static_cast<const char *>(a_lo_);
    const char *b_hi = static_cast<const char *>(b_hi_), *b_lo = static_cast<const char *>(b_lo_);
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t full_a[TCP_NST], full_b[TCP_NST], empty_bar[TCP_NST];
    __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_s;
    __shared__ int tgt_e[2][128];    // per accumulator slot: target node of each pair column
    __shared__ float csc_e[2][128];  // and the column scale of its source
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nstage = kpad / KS;
    const int npair = (mtiles + TCP_RT - 1) / TCP_RT;  // row-tile pairs per chunk
    // units of this CTA: u = blockIdx.x + i gridDim.x, i < nmine
    const int nmine = blockIdx.x < nunits ? (nunits - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (tid == 0) {
        abort_s = 0;
        for (int i = 0; i < TCP_NST; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_a[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_b[i])), "r"(TCP_BPROD));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty_bar[i])));
        }
        for (int i = 0; i < 2; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acc_empty[i])), "r"(TCP_EPI / 32));
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem_d = tmem_base;
    auto unit_of = [&](int i, int &op, int &b, int &cnt, int &tile0, int &rt) {
        const int u = blockIdx.x + i * gridDim.x, c = u / npair;
        op = chunks[3 * c];
        b = chunks[3 * c + 1];
        cnt = chunks[3 * c + 2];
        tile0 = (u % npair) * TCP_RT;
        rt = min(TCP_RT, mtiles - tile0);
    };

    if (warp == 0) {
        if (lane == 0) {  // operator tiles: bulk copies, stage g = i nstage + st
            long issued = -1;
            for (int i = 0; i < nmine && !abort_s; ++i) {
                int op, b, cnt, tile0, rt;
                unit_of(i, op, b, cnt, tile0, rt);
                const long atile0 = ((long)op * mtiles + tile0) * nstage;
                for (int st = 0; st < nstage; ++st) {
                    const long g = (long)i * nstage + st;
                    const int buf = (int)(g % TCP_NST);
                    if (g >= TCP_NST &&
                        !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((g / TCP_NST) - 1) & 1))) {
                        abort_s = 1;
                        break;
                    }
                    if (abort_s) break;
                    unsigned char *base = tc_smem + buf * TCP_STAGE;
                    const uint32_t fb = smem_u32(&full_a[buf]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb),
                                 "r"(2 * rt * TC_TILE_BYTES)
                                 : "memory");
                    for (int t = 0; t < rt; ++t) {
                        const long ga = (atile0 + (long)t * nstage + st) * TC_TILE_BYTES;
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
                            "[%3];" ::"r"(smem_u32(base + t * TC_TILE_BYTES)),
                            "l"(a_hi + ga), "r"(TC_TILE_BYTES), "r"(fb)
                            : "memory");
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
                            "[%3];" ::"r"(smem_u32(base + (TCP_RT + t) * TC_TILE_BYTES)),
                            "l"(a_lo + ga), "r"(TC_TILE_BYTES), "r"(fb)
                            : "memory");
                    }
                    issued = g;
                }
            }
            // every issued copy lands before the CTA may exit
            for (long g2 = issued - TCP_NST + 1 < 0 ? 0 : issued - TCP_NST + 1; g2 <= issued; ++g2)
                if (!mbar_wait(smem_u32(&full_a[g2 % TCP_NST]), (uint32_t)((g2 / TCP_NST) & 1))) abort_s = 1;
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issue
            long last = -1;
            for (int i = 0; i < nmine && !abort_s; ++i) {
                int op, b, cnt, tile0, rt;
                unit_of(i, op, b, cnt, tile0, rt);
                const int neff = max(16, (cnt + 15) & ~15);
                constexpr uint32_t NMASK = 0x3Fu << 17;
                const uint32_t idesc = (TcShape<128>::IDESC16 & ~NMASK) | ((uint32_t)(neff >> 3) << 17);
                const int slot = i & 1;
                // the epilogue has drained this slot's previous unit (i - 2)
                if (i >= 2 && !mbar_wait(smem_u32(&acc_empty[slot]), (uint32_t)(((i >> 1) - 1) & 1))) {
                    abort_s = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                bool ok = true;
                for (int st = 0; st < nstage; ++st) {
                    const long g = (long)i * nstage + st;
                    const int buf = (int)(g % TCP_NST);
                    const uint32_t par = (uint32_t)((g / TCP_NST) & 1);
                    if (!mbar_wait(smem_u32(&full_a[buf]), par) || !mbar_wait(smem_u32(&full_b[buf]), par) ||
                        abort_s) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t base = smem_u32(tc_smem + buf * TCP_STAGE);
                    const uint64_t bh = make_desc(base + (2 * TCP_RT) * TC_TILE_BYTES, 128, 256);
                    const uint64_t bl = make_desc(base + (2 * TCP_RT) * TC_TILE_BYTES + BT, 128, 256);
                    for (int t = 0; t < rt; ++t) {
                        const uint64_t ah = make_desc(base + t * TC_TILE_BYTES, 128, 256);
                        const uint64_t al = make_desc(base + (TCP_RT + t) * TC_TILE_BYTES, 128, 256);
                        const uint32_t d = tmem_d + (uint32_t)(slot * TCP_RT * N + t * N);
                        mma_f16(d, ah, bh, idesc, st > 0 ? 1u : 0u);
                        mma_f16(d, ah, bl, idesc, 1u);
                        mma_f16(d, al, bh, idesc, 1u);
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(&empty_bar[buf]))
                                 : "memory");
                    last = g;
                }
                if (!ok) {
                    abort_s = 1;
                    break;
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&acc_full[slot]))
                             : "memory");
            }
            // every MMA issued completes before TMEM is released (also after an abort)
            if (last >= 0 && !mbar_wait(smem_u32(&empty_bar[last % TCP_NST]), (uint32_t)((last / TCP_NST) & 1)))
                abort_s = 1;
        }
    } else if (warp < TCP_EPI_WARP0) {  // multipole rows: cp.async by TCP_BPROD threads
        const int t = tid - 64;
        long issued = -1;
        for (int i = 0; i < nmine && !abort_s; ++i) {
            int op, b, cnt, tile0, rt;
            unit_of(i, op, b, cnt, tile0, rt);
            const int neff = max(16, (cnt + 15) & ~15);
            // this thread's pieces of a stage (2 tiles x neff rows x 2 halves of 16 B), fixed per unit
            constexpr int MAXP = (4 * 128 + TCP_BPROD - 1) / TCP_BPROD;
            const char *srcp[MAXP];
            uint32_t dsto[MAXP];
            int np = 0;
            for (int q = t; q < 4 * neff && np < MAXP; q += TCP_BPROD, ++np) {
                const int tile = q / (2 * neff), row = (q >> 1) % neff, c = q & 1;
                dsto[np] = (uint32_t)(2 * TCP_RT * TC_TILE_BYTES + tile * BT) + tile_off(row, c);
                const int sn = row < cnt ? vsrc[b + row] : -1;
                const char *B = tile == 0 ? b_hi : b_lo;
                srcp[np] = sn >= 0 ? B + (long)sn * kpad * ES + 16 * c : nullptr;
            }
            for (int st = 0; st < nstage; ++st) {
                const long g = (long)i * nstage + st;
                const int buf = (int)(g % TCP_NST);
                if (g >= TCP_NST && !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((g / TCP_NST) - 1) & 1))) {
                    abort_s = 1;
                    break;
                }
                if (abort_s) break;
                const uint32_t base = smem_u32(tc_smem + buf * TCP_STAGE);
                for (int j = 0; j < np; ++j)
                    cp_async16(base + dsto[j], srcp[j] ? (const void *)(srcp[j] + (long)st * KS * ES) : (const void *)b_hi,
                               srcp[j] ? 16u : 0u);
                asm volatile("cp.async.commit_group;");
                issued = g;
                if (g >= TCP_LAG) {
                    asm volatile("cp.async.wait_group %0;" ::"n"(TCP_LAG) : "memory");
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                     smem_u32(&full_b[(g - TCP_LAG) % TCP_NST]))
                                 : "memory");
                }
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (long g2 = issued - TCP_LAG + 1 < 0 ? 0 : issued - TCP_LAG + 1; g2 <= issued; ++g2)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_b[g2 % TCP_NST])) : "memory");
    } else {  // epilogue: the last four warps, TMEM lanes 32 (warp % 4) .. + 31
        // decisions stay warp-uniform (tcgen05.ld is a warp-collective instruction), and every
        // epilogue warp passes the same number of named barriers: after an abort the remaining
        // units are skipped, not left
        const int lg = warp & 3;
        for (int i = 0; i < nmine; ++i) {
            int op, b, cnt, tile0, rt;
            unit_of(i, op, b, cnt, tile0, rt);
            const int neff = max(16, (cnt + 15) & ~15);
            const int slot = i & 1;
            {  // this unit's column table, then a barrier among the four epilogue warps (id 1)
                const int e = tid - 32 * TCP_EPI_WARP0;
                tgt_e[slot][e] = e < cnt ? __ldg(vtgt + b + e) : -1;
                csc_e[slot][e] = e < cnt ? __ldg(cscale + __ldg(vsrc + b + e)) : 0.f;
                asm volatile("bar.sync 1, %0;" ::"n"(TCP_EPI) : "memory");
            }
            bool go = __shfl_sync(0xffffffffu, (int)abort_s, 0) == 0;
            if (go) go = __all_sync(0xffffffffu, mbar_wait(smem_u32(&acc_full[slot]), (uint32_t)((i >> 1) & 1)));
            if (!go) {
                abort_s = 1;
                continue;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            for (int tt = 0; tt < rt; ++tt) {
                const int row = (tile0 + tt) * TC_M + 32 * lg + lane;
                const float rs = rscale[(long)op * mtiles * TC_M + row];  // row < mtiles * 128
                const uint32_t taddr = tmem_d + ((uint32_t)(32 * lg) << 16) + (uint32_t)(slot * TCP_RT * N + tt * N);
#pragma unroll 1
                for (int c0 = 0; c0 < neff; c0 += 16) {
                    uint32_t v[16];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                        "%12, %13, %14, %15}, [%16];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                          "=r"(v[14]), "=r"(v[15])
                        : "r"(taddr + (uint32_t)c0));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (row < n4) {
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            const int tg = tgt_e[slot][c0 + q];
                            if (tg >= 0)
                                atomicAdd(local + (long)tg * n4 + row, __uint_as_float(v[q]) * rs * csc_e[slot][c0 + q]);
                        }
                    }
                }
            }
            // this slot may be overwritten once every epilogue warp has read it
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[slot])) : "memory");
        }
    }
    __syncthreads();
    if (abort_s && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(512));
}

// ---------------------------------------------------------------------------------------------
// CTA-pair form (tcgen05 cta_group::2).  A cluster of two CTAs on two SMs takes one chunk of up to
// 256 pairs of an operator against four operator row tiles.  Each MMA is M = 256 (128 operator
// rows from each CTA's shared memory) x N = 256 pairs (the multipole rows of 128 pairs from each
// CTA) x K = 8, issued by the even CTA; each CTA's TMEM receives its own 128 rows for all 256
// pairs, two row tiles filling its 512 columns.  Per SM and stage this moves 16 KB of operator
// tiles and 8 KB of multipole rows for the MMA work that the one-CTA form feeds with 32 KB + 8 KB.
// The even CTA holds operator row tiles 0 and 2 of its group of four, the odd CTA tiles 1 and 3.
// Barriers: each CTA keeps the one-CTA form's full_a / full_b / empty; the odd CTA's relay thread
// waits on its own full barriers and arrives remotely on the even CTA's peer_full; the even CTA's
// MMA thread waits on all three and multicasts its commits to both CTAs' empty and accumulator
// barriers.  Every wait is bounded; an abort in either CTA is written into the other's flag
// before the epilogue, and both CTAs meet at cluster barriers only on paths every thread takes.
// ---------------------------------------------------------------------------------------------
constexpr int TC2_N = 256, TC2_HALF = 128, TC2_PT = 2;  // pairs per chunk, per CTA; row tiles per CTA
constexpr int TC2_STAGE = 2 * TC2_PT * TC_TILE_BYTES + 2 * TC_TILE_BYTES;  // 16 KB operator + 8 KB multipoles
constexpr int TC2_NST = 8, TC2_LAG = 2;  // (copy lag 2, 4 and 6 measured 5.35, 5.39 and 6.13 ms)
constexpr int TC2_SMEM = TC2_NST * TC2_STAGE;  // 192 KB
// D FP32, A and B TF32, K-major, N = 256, M = 256 (the pair)
constexpr uint32_t TC2_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC2_N >> 3) << 17) | ((256u >> 4) << 24);

__device__ __forceinline__ uint32_t cluster_addr(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void mma_tf32_pair(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(TC2_IDESC), "r"(accumulate));
}

__device__ __forceinline__ void commit_pair(uint32_t mbar) {
    const uint16_t both = 3;
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(mbar),
        "h"(both)
        : "memory");
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(TC_THREADS, 1)
    k_m2l_tc2(int n4, int kpad, int mtiles, const int *__restrict__ chunks, const int *__restrict__ vsrc,
              const int *__restrict__ vtgt, const float *__restrict__ a_hi, const float *__restrict__ a_lo,
              const float *__restrict__ b_hi, const float *__restrict__ b_lo, float *local, int *err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t full_a[TC2_NST], full_b[TC2_NST], empty_bar[TC2_NST], peer_full[TC2_NST], acc_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int src_s[TC2_HALF], tgt_s[TC2_N];
    __shared__ volatile int abort_s;
    uint32_t rank;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int chunk = blockIdx.x >> 1;
    const int op = chunks[3 * chunk], b = chunks[3 * chunk + 1], cnt = chunks[3 * chunk + 2];
    const int tile_base = blockIdx.y * 2 * TC2_PT;               // first operator row tile of the group
    const int pt = min(TC2_PT, (mtiles - tile_base + 1) / 2);    // row tiles of the pair in use
    const int nstage = kpad / TC_KS;
    for (int i = tid; i < TC2_N; i += TC_THREADS) tgt_s[i] = i < cnt ? vtgt[b + i] : -1;
    for (int i = tid; i < TC2_HALF; i += TC_THREADS) {
        const int j = (int)rank * TC2_HALF + i;
        src_s[i] = j < cnt ? vsrc[b + j] : -1;
    }
    if (tid == 0) {
        abort_s = 0;
        for (int i = 0; i < TC2_NST; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_a[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_b[i])), "r"(TC_BPROD));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty_bar[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&peer_full[i])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_bar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {  // collective over the pair: both CTAs allocate, and receive the same columns
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(TC2_PT * TC2_N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    cluster_sync_all();  // both CTAs' barriers initialised and TMEM allocated
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem_d = tmem_base;
    auto has_tile = [&](int T) { return tile_base + 2 * T + (int)rank < mtiles; };

    if (warp == 0) {
        if (lane == 0) {  // this CTA's operator tiles: bulk copies
            int issued = -1;
            int nbytes = 0;
            for (int T = 0; T < pt; ++T)
                if (has_tile(T)) nbytes += 2 * TC_TILE_BYTES;
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % TC2_NST;
                if (st >= TC2_NST &&
                    !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((st / TC2_NST) - 1) & 1))) {
                    abort_s = 1;
                    break;
                }
                if (abort_s) break;
                unsigned char *base = tc_smem + buf * TC2_STAGE;
                const uint32_t fb = smem_u32(&full_a[buf]);
                if (nbytes == 0) {
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(fb) : "memory");
                } else {
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(nbytes)
                                 : "memory");
                    for (int T = 0; T < pt; ++T) {
                        if (!has_tile(T)) continue;
                        const int tile = tile_base + 2 * T + (int)rank;
                        const long g = (((long)op * mtiles + tile) * nstage + st) * (TC_TILE_BYTES / 4);
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                                smem_u32(base + T * TC_TILE_BYTES)),
                            "l"(a_hi + g), "r"(TC_TILE_BYTES), "r"(fb)
                            : "memory");
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                                smem_u32(base + (TC2_PT + T) * TC_TILE_BYTES)),
                            "l"(a_lo + g), "r"(TC_TILE_BYTES), "r"(fb)
                            : "memory");
                    }
                }
                issued = st;
            }
            for (int s2 = max(0, issued - TC2_NST + 1); s2 <= issued; ++s2)
                if (!mbar_wait(smem_u32(&full_a[s2 % TC2_NST]), (uint32_t)((s2 / TC2_NST) & 1))) abort_s = 1;
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {  // MMA issue for the pair
            int last = -1;
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % TC2_NST;
                const uint32_t par = (uint32_t)((st / TC2_NST) & 1);
                if (!mbar_wait(smem_u32(&full_a[buf]), par) || !mbar_wait(smem_u32(&full_b[buf]), par) ||
                    !mbar_wait(smem_u32(&peer_full[buf]), par) || abort_s) {
                    abort_s = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t base = smem_u32(tc_smem + buf * TC2_STAGE);
                const uint64_t bh = make_desc(base + (2 * TC2_PT) * TC_TILE_BYTES, 128, 256);
                const uint64_t bl = make_desc(base + (2 * TC2_PT + 1) * TC_TILE_BYTES, 128, 256);
                for (int T = 0; T < pt; ++T) {
                    const uint64_t ah = make_desc(base + T * TC_TILE_BYTES, 128, 256);
                    const uint64_t al = make_desc(base + (TC2_PT + T) * TC_TILE_BYTES, 128, 256);
                    const uint32_t d = tmem_d + (uint32_t)(T * TC2_N);
                    mma_tf32_pair(d, ah, bh, st > 0 ? 1u : 0u);
                    mma_tf32_pair(d, ah, bl, 1u);
                    mma_tf32_pair(d, al, bh, 1u);
                }
                commit_pair(smem_u32(&empty_bar[buf]));
                last = st;
            }
            // the accumulator barriers of both CTAs always receive a commit: it tracks every MMA
            // issued above, so after it neither CTA's shared memory is read any more
            commit_pair(smem_u32(&acc_bar));
            if (last != nstage - 1) abort_s = 1;
        } else if (lane == 0) {  // odd CTA: relay its full stages to the even CTA
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % TC2_NST;
                const uint32_t par = (uint32_t)((st / TC2_NST) & 1);
                if (!mbar_wait(smem_u32(&full_a[buf]), par) || !mbar_wait(smem_u32(&full_b[buf]), par) || abort_s) {
                    abort_s = 1;
                    break;
                }
                asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(
                                 cluster_addr(smem_u32(&peer_full[buf]), 0))
                             : "memory");
            }
        }
    } else {  // this CTA's 128 multipole rows: cp.async by 192 threads
        const int t = tid - 64;
        int issued = -1;
        for (int st = 0; st < nstage; ++st) {
            const int buf = st % TC2_NST;
            if (st >= TC2_NST &&
                !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((st / TC2_NST) - 1) & 1))) {
                abort_s = 1;
                break;
            }
            if (abort_s) break;
            unsigned char *base = tc_smem + buf * TC2_STAGE + 2 * TC2_PT * TC_TILE_BYTES;
            const int k0 = st * TC_KS;
            for (int i = t; i < 4 * TC2_HALF; i += TC_BPROD) {  // 2 tiles x 128 rows x 2 pieces of 16 B
                const int tile = i / (2 * TC2_HALF), row = (i >> 1) % TC2_HALF, c = i & 1;
                const uint32_t dst = smem_u32(base + tile * TC_TILE_BYTES + tile_off(row, c));
                const int sn = src_s[row];
                const float *B = tile == 0 ? b_hi : b_lo;
                cp_async16(dst, sn >= 0 ? (const void *)(B + (long)sn * kpad + k0 + 4 * c) : (const void *)B,
                           sn >= 0 ? 16u : 0u);
            }
            asm volatile("cp.async.commit_group;");
            issued = st;
            if (st >= TC2_LAG) {
                asm volatile("cp.async.wait_group %0;" ::"n"(TC2_LAG) : "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                 smem_u32(&full_b[(st - TC2_LAG) % TC2_NST]))
                             : "memory");
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int s2 = max(0, issued - TC2_LAG + 1); s2 <= issued; ++s2)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_b[s2 % TC2_NST])) : "memory");
    }
    __syncthreads();
    // every MMA of the pair is complete once the accumulator barrier flips (the even CTA commits
    // to it on every path); an abort on either side is copied into the other CTA's flag
    if (tid == 0) {
        const bool acc = mbar_wait(smem_u32(&acc_bar), 0u);
        if (!acc || abort_s) {
            abort_s = 1;
            asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(cluster_addr(smem_u32((const void *)&abort_s), rank ^ 1u)),
                         "r"(1u)
                         : "memory");
        }
    }
    cluster_sync_all();
    const bool ok = !abort_s;
    if (!ok && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (ok) {
        const int lg = warp & 3;
        for (int T = warp >> 2; T < pt; T += 2) {
            if (!has_tile(T)) continue;
            const int row = (tile_base + 2 * T + (int)rank) * TC_M + 32 * lg + lane;
            const uint32_t taddr = tmem_d + ((uint32_t)(32 * lg) << 16) + (uint32_t)(T * TC2_N);
#pragma unroll 1
            for (int c0 = 0; c0 < TC2_N; c0 += 16) {
                uint32_t v[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15}, [%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(taddr + (uint32_t)c0));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (row < n4) {
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int tg = tgt_s[c0 + q];
                        if (tg >= 0) atomicAdd(local + (long)tg * n4 + row, __uint_as_float(v[q]));
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    cluster_sync_all();  // neither CTA leaves while the other may still use the pair's TMEM
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(TC2_PT * TC2_N));
}

// ---------------------------------------------------------------------------------------------
// CTA-pair form of the scaled FP16 contraction.  One tcgen05.mma.cta_group::2 of M = 256 x N x
// K = 16 reads, on each SM, only that CTA's 128 operator rows and its half of the N multipole
// rows, where the one-CTA form reads 128 rows of both operands for half the work: per SM the
// MMAs' shared-memory operand reads fall from 16 to 8 bytes per 1,024 flops, and the copies into
// shared memory from 7.6 to 5.1.  The one-CTA form is bound by that bandwidth (its tensor pipe's
// operand reads run at 1.27x the pipe's active fraction, the copies at 0.92x).  A cluster of two
// CTAs takes one chunk of up to 256 pairs against PT row-tile pairs: pair T holds row tile
// tile_base + 2T in the even CTA and tile_base + 2T + 1 in the odd one; the chunk's MMA width N
// is its pair count rounded up to 16, each CTA gathering N / 2 multipole rows.  Barriers as in
// the TF32 pair kernel (k_m2l_tc2): the odd CTA's relay thread passes its full stages to the
// even CTA (a relaxed arrive: the release form's cluster-scope fence on every stage made the kernel
// 3.62 instead of 2.62 ms a launch), whose MMA thread multicasts its commits to both CTAs; every
// wait is bounded, and both CTAs meet at cluster barriers only on paths every thread takes.  The
// epilogue applies the FP16 form's row and column scales.  Measured on the 2,000-atom protein:
// 2.56 ms a launch (one row-tile pair per CTA, two CTAs per SM) against 2.34 ms for two CTAs of
// two row tiles per SM, so it is a launch form the tuning table may pick (6, 7), not the default.
// ---------------------------------------------------------------------------------------------
template <int PT> struct Tc2hShape {
    static constexpr int STAGE = (2 * PT + 2) * TC_TILE_BYTES;  // operator hi/lo per row tile + multipole hi/lo
    static constexpr int NST = PT == 1 ? 6 : 8;                 // 96 KB (two CTAs per SM) or 192 KB
    static constexpr int SMEM = NST * STAGE;
    static constexpr int LAG = 1;  // copy lag (lags 2, 3, 4 and 5: 2.60, 2.61, 2.68 and 3.39 ms against 2.56)
};

__device__ __forceinline__ void mma_f16_pair(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

template <int PT>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(TC_THREADS, PT == 1 ? 2 : 1)
    k_m2l_tc2h(int n4, int kpad, int mtiles, const int *__restrict__ chunks, const int *__restrict__ vsrc,
               const int *__restrict__ vtgt, const char *__restrict__ a_hi, const char *__restrict__ a_lo,
               const char *__restrict__ b_hi, const char *__restrict__ b_lo, const float *__restrict__ rscale,
               const float *__restrict__ cscale, float *local, int *err) {
    using SH = Tc2hShape<PT>;
    constexpr int NST = SH::NST, LAG = SH::LAG, STAGE = SH::STAGE;
    constexpr int KS = TC_KS16, ES = 2;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t full_a[NST], full_b[NST], empty_bar[NST], peer_full[NST], acc_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int src_s[TC2_HALF], tgt_s[TC2_N];
    __shared__ float csc_s[TC2_N];
    __shared__ volatile int abort_s;
    uint32_t rank;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int chunk = blockIdx.x >> 1;
    const int op = chunks[3 * chunk], b = chunks[3 * chunk + 1], cnt = chunks[3 * chunk + 2];
    const int neff = max(16, (cnt + 15) & ~15), half = neff >> 1;  // MMA width; rows per CTA
    const int tile_base = blockIdx.y * 2 * PT;
    const int pt = min(PT, (mtiles - tile_base + 1) / 2);
    const int nstage = kpad / KS;
    constexpr uint32_t IDESC0 = (1u << 4) | (0u << 7) | (0u << 10) | ((256u >> 4) << 24);
    const uint32_t idesc = IDESC0 | ((uint32_t)(neff >> 3) << 17);
    for (int i = tid; i < TC2_N; i += TC_THREADS) {
        tgt_s[i] = i < cnt ? vtgt[b + i] : -1;
        csc_s[i] = i < cnt ? cscale[vsrc[b + i]] : 0.f;
    }
    for (int i = tid; i < TC2_HALF; i += TC_THREADS) {
        const int j = (int)rank * half + i;
        src_s[i] = (i < half && j < cnt) ? vsrc[b + j] : -1;
    }
    if (tid == 0) {
        abort_s = 0;
        for (int i = 0; i < NST; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_a[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_b[i])), "r"(TC_BPROD));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty_bar[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&peer_full[i])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_bar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {  // collective over the pair: both CTAs allocate, and receive the same columns
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(PT * TC2_N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    cluster_sync_all();  // both CTAs' barriers initialised and TMEM allocated
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem_d = tmem_base;
    auto has_tile = [&](int T) { return tile_base + 2 * T + (int)rank < mtiles; };

    if (warp == 0) {
        if (lane == 0) {  // this CTA's operator tiles: bulk copies
            int issued = -1;
            int nbytes = 0;
            for (int T = 0; T < pt; ++T)
                if (has_tile(T)) nbytes += 2 * TC_TILE_BYTES;
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % NST;
                if (st >= NST && !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((st / NST) - 1) & 1))) {
                    abort_s = 1;
                    break;
                }
                if (abort_s) break;
                unsigned char *base = tc_smem + buf * STAGE;
                const uint32_t fb = smem_u32(&full_a[buf]);
                if (nbytes == 0) {
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(fb) : "memory");
                } else {
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(nbytes)
                                 : "memory");
                    for (int T = 0; T < pt; ++T) {
                        if (!has_tile(T)) continue;
                        const int tile = tile_base + 2 * T + (int)rank;
                        const long g = (((long)op * mtiles + tile) * nstage + st) * TC_TILE_BYTES;
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                                smem_u32(base + T * TC_TILE_BYTES)),
                            "l"(a_hi + g), "r"(TC_TILE_BYTES), "r"(fb)
                            : "memory");
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                                smem_u32(base + (PT + T) * TC_TILE_BYTES)),
                            "l"(a_lo + g), "r"(TC_TILE_BYTES), "r"(fb)
                            : "memory");
                    }
                }
                issued = st;
            }
            for (int s2 = max(0, issued - NST + 1); s2 <= issued; ++s2)
                if (!mbar_wait(smem_u32(&full_a[s2 % NST]), (uint32_t)((s2 / NST) & 1))) abort_s = 1;
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {  // MMA issue for the pair
            int last = -1;
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % NST;
                const uint32_t par = (uint32_t)((st / NST) & 1);
                if (!mbar_wait(smem_u32(&full_a[buf]), par) || !mbar_wait(smem_u32(&full_b[buf]), par) ||
                    !mbar_wait(smem_u32(&peer_full[buf]), par) || abort_s) {
                    abort_s = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t base = smem_u32(tc_smem + buf * STAGE);
                const uint64_t bh = make_desc(base + (2 * PT) * TC_TILE_BYTES, 128, 256);
                const uint64_t bl = make_desc(base + (2 * PT + 1) * TC_TILE_BYTES, 128, 256);
                for (int T = 0; T < pt; ++T) {
                    const uint64_t ah = make_desc(base + T * TC_TILE_BYTES, 128, 256);
                    const uint64_t al = make_desc(base + (PT + T) * TC_TILE_BYTES, 128, 256);
                    const uint32_t d = tmem_d + (uint32_t)(T * TC2_N);
                    mma_f16_pair(d, ah, bh, idesc, st > 0 ? 1u : 0u);
                    mma_f16_pair(d, ah, bl, idesc, 1u);
                    mma_f16_pair(d, al, bh, idesc, 1u);
                }
                commit_pair(smem_u32(&empty_bar[buf]));
                last = st;
            }
            // the accumulator barriers of both CTAs always receive a commit: it tracks every MMA
            // issued above, so after it neither CTA's shared memory is read any more
            commit_pair(smem_u32(&acc_bar));
            if (last != nstage - 1) abort_s = 1;
        } else if (lane == 0) {  // odd CTA: relay its full stages to the even CTA
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % NST;
                const uint32_t par = (uint32_t)((st / NST) & 1);
                if (!mbar_wait(smem_u32(&full_a[buf]), par) || !mbar_wait(smem_u32(&full_b[buf]), par) || abort_s) {
                    abort_s = 1;
                    break;
                }
                // relaxed: the data this stage holds is already in this CTA's shared memory (the
                // waits above acquired its completion) and is read there by this SM's tensor core
                asm volatile("mbarrier.arrive.relaxed.cluster.shared::cluster.b64 _, [%0];" ::"r"(
                                 cluster_addr(smem_u32(&peer_full[buf]), 0))
                             : "memory");
            }
        }
    } else {  // this CTA's half of the multipole rows: cp.async by 192 threads, slots addressed once
        const int t = tid - 64;
        constexpr int MAXS = (4 * TC2_HALF + TC_BPROD - 1) / TC_BPROD;
        uint32_t soff[MAXS], sbytes[MAXS];
        const char *gsrc[MAXS];
        int nsl = 0;
#pragma unroll
        for (int q = 0; q < MAXS; ++q) {
            const int i = t + q * TC_BPROD;
            soff[q] = 0;
            sbytes[q] = 0;
            gsrc[q] = b_hi;
            if (i < 4 * half) {
                const int tile = i / (2 * half), row = (i >> 1) % half, c = i & 1;
                const int sn = src_s[row];
                soff[q] = (2 * PT + tile) * TC_TILE_BYTES + tile_off(row, c);
                sbytes[q] = sn >= 0 ? 16u : 0u;
                gsrc[q] = (tile == 0 ? b_hi : b_lo) + (sn >= 0 ? (long)sn * kpad * ES + 16 * c : 0);
                nsl = q + 1;
            }
        }
        int issued = -1;
        for (int st = 0; st < nstage; ++st) {
            const int buf = st % NST;
            if (st >= NST && !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((st / NST) - 1) & 1))) {
                abort_s = 1;
                break;
            }
            if (abort_s) break;
            const uint32_t base = smem_u32(tc_smem + buf * STAGE);
            const long koff = (long)st * KS * ES;
#pragma unroll
            for (int q = 0; q < MAXS; ++q)
                if (q < nsl) cp_async16(base + soff[q], sbytes[q] ? gsrc[q] + koff : gsrc[q], sbytes[q]);
            asm volatile("cp.async.commit_group;");
            issued = st;
            if (st >= LAG) {
                asm volatile("cp.async.wait_group %0;" ::"n"(LAG) : "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_b[(st - LAG) % NST]))
                             : "memory");
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int s2 = max(0, issued - LAG + 1); s2 <= issued; ++s2)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_b[s2 % NST])) : "memory");
    }
    __syncthreads();
    // every MMA of the pair is complete once the accumulator barrier flips (the even CTA commits
    // to it on every path); an abort on either side is copied into the other CTA's flag
    if (tid == 0) {
        const bool acc = mbar_wait(smem_u32(&acc_bar), 0u);
        if (!acc || abort_s) {
            abort_s = 1;
            asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(cluster_addr(smem_u32((const void *)&abort_s), rank ^ 1u)),
                         "r"(1u)
                         : "memory");
        }
    }
    cluster_sync_all();
    const bool ok = !abort_s;
    if (!ok && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (ok) {
        // warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows); the two warp groups take
        // alternate 16-column blocks of each accumulator
        const int lg = warp & 3, grp = warp >> 2, nb = neff >> 4;
        for (int u = grp; u < pt * nb; u += 2) {
            const int T = u / nb, c0 = (u % nb) * 16;
            if (!has_tile(T)) continue;  // uniform over the CTA
            const int row = (tile_base + 2 * T + (int)rank) * TC_M + 32 * lg + lane;
            const float rs = rscale[(long)op * mtiles * TC_M + row];  // row < mtiles * 128
            const uint32_t taddr = tmem_d + ((uint32_t)(32 * lg) << 16) + (uint32_t)(T * TC2_N + c0);
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < n4) {
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int tg = tgt_s[c0 + q];
                    if (tg >= 0) atomicAdd(local + (long)tg * n4 + row, __uint_as_float(v[q]) * rs * csc_s[c0 + q]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    cluster_sync_all();  // neither CTA leaves while the other may still use the pair's TMEM
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(PT * TC2_N));
}

// hi = x rounded to TF32 (10 explicit mantissa bits, to nearest even), lo = x - hi.
__device__ __forceinline__ float tf32_round(float x) {
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x0fffu + ((u >> 13) & 1u);
    u &= 0xffffe000u;
    return __uint_as_float(u);
}

// Operators (column-major n4 x n4 per op, FP32) -> hi / lo tiles in the shared-memory layout,
// [op][row tile of 128][stage of 8 K][1024 floats]; float f of a tile holds row
// (f / 64) * 8 + (f % 32) / 4 and K element ((f / 32) % 2) * 4 + f % 4 (core matrices of 8 rows
// x 4 K, two per row group along K).  Rows and K beyond n4 are zero.
__global__ void k_pack_ops_tc(int n4, int mtiles, int kpad, int nops, const float *__restrict__ ops, float *a_hi,
                              float *a_lo) {
    const int nstage = kpad / TC_KS;
    const long total = (long)nops * mtiles * nstage * (TC_TILE_BYTES / 4);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int f = (int)(i % (TC_TILE_BYTES / 4));
        const long tix = i / (TC_TILE_BYTES / 4);
        const int st = (int)(tix % nstage);
        const int t = (int)((tix / nstage) % mtiles);
        const int op = (int)(tix / ((long)nstage * mtiles));
        const int cm = f >> 5;  // core matrix: row group cm / 2, K half cm % 2
        const int row = t * TC_M + (cm >> 1) * 8 + ((f & 31) >> 2);
        const int k = st * TC_KS + (cm & 1) * 4 + (f & 3);
        float x = 0.f;
        if (row < n4 && k < n4) x = ops[(long)op * n4 * n4 + (long)k * n4 + row];
        const float h = tf32_round(x);
        a_hi[i] = h;
        a_lo[i] = x - h;
    }
}

// Multipoles [node][n4] -> [node][kpad] hi / lo (padding zero).
__global__ void k_split_mult_tc(long nnodes, int n4, int kpad, const float *__restrict__ m, float *hi, float *lo) {
    const long total = nnodes * kpad;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i % kpad);
        const long node = i / kpad;
        const float x = k < n4 ? m[node * n4 + k] : 0.f;
        const float h = tf32_round(x);
        hi[i] = h;
        lo[i] = x - h;
    }
}


// Scaled FP16 operand form.  Each operator row r is divided by a power of two s_r with
// max_k |A_rk| / s_r in [2^13, 2^14), each multipole column (source node) j likewise by t_j, and
// a scaled value x is split into hi = fp16(x) and lo = fp16(x - hi), 11 significant bits each;
// D accumulates A_hi.B_hi + A_hi.B_lo + A_lo.B_hi in FP32 (kind::f16, K = 16 per MMA; products
// below 2^28, sums below 2^37) and the epilogue multiplies by s_r t_j.  Placing the maximum at
// 2^14 keeps lo in the FP16 normal range down to 2^-17 of the row or column maximum, so a split
// value carries about 22 bits, as the TF32 split does, while a stage of 32 bytes per row holds
// 16 K elements instead of 8: half the operand bytes per flop.

// Power-of-two scale s with m / s in [2^13, 2^14) (2^-14 for m == 0).
__device__ __forceinline__ float h16_scale(float m) {
    if (!(m > 0.f)) return ldexpf(1.f, -14);
    int e;
    frexpf(m, &e);  // m = f 2^e, f in [0.5, 1)
    return ldexpf(1.f, e - 14);
}

// An operator entry as (hi, lo): FP32 operators have lo = 0, float-float ones carry both words.
__device__ __forceinline__ float2 op_word(const float *__restrict__ ops, long i) { return make_float2(ops[i], 0.f); }
__device__ __forceinline__ float2 op_word(const float2 *__restrict__ ops, long i) { return ops[i]; }

// Row scales s_r of the operators (FP32 or float-float, column-major n4 x n4 per op):
// rscale[op][mtiles * 128].
template <class OW>
__global__ void k_scale_ops_h16(int n4, int mtiles, int nops, const OW *__restrict__ ops, float *rscale) {
    const int mpad = mtiles * TC_M;
    const long total = (long)nops * mpad;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int r = (int)(i % mpad), op = (int)(i / mpad);
        float m = 0.f;
        if (r < n4) {
            const long c0 = (long)op * n4 * n4 + r;
            for (int k = 0; k < n4; ++k) {
                const float2 x = op_word(ops, c0 + (long)k * n4);
                m = fmaxf(m, fabsf(x.x) + fabsf(x.y));
            }
        }
        rscale[i] = h16_scale(m);
    }
}

__device__ __forceinline__ void split_h16(float x, uint16_t &hi, uint16_t &lo) {
    const __half h = __float2half_rn(x);
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(__float2half_rn(x - __half2float(h)));
}

// The same for a scaled (hi, lo) word pair: hi from the high word, lo from the rest.
__device__ __forceinline__ void split_h16(float2 x, uint16_t &hi, uint16_t &lo) {
    const __half h = __float2half_rn(x.x);
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(__float2half_rn((x.x - __half2float(h)) + x.y));
}

// FP32 operators -> scaled FP16 hi / lo tiles [op][row tile][stage of 16 K][4 KB] in the
// shared-memory layout (tile_off with 8 K elements of 2 bytes per 16-byte row piece).  One thread
// per (op, row, group of 8 K elements): 8 coalesced column reads, one 16-byte store per word.
template <class OW>
__global__ void k_pack_ops_h16(int n4, int mtiles, int kpad, int nops, const OW *__restrict__ ops,
                               const float *__restrict__ rscale, uint4 *a_hi, uint4 *a_lo) {
    const int nstage = kpad / TC_KS16, mpad = mtiles * TC_M, ngrp = kpad / 8;
    const long total = (long)nops * ngrp * mpad;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int r = (int)(i % mpad);
        const long rest = i / mpad;
        const int grp = (int)(rest % ngrp), op = (int)(rest / ngrp);
        const float inv = 1.f / rscale[(long)op * mpad + r];  // a power of two: exact
        uint32_t wh[4], wl[4];
        for (int q = 0; q < 8; q += 2) {
            uint16_t h0, l0, h1, l1;
            const int k = grp * 8 + q;
            float2 x0 = make_float2(0.f, 0.f), x1 = make_float2(0.f, 0.f);
            if (r < n4 && k < n4) x0 = op_word(ops, (long)op * n4 * n4 + (long)k * n4 + r);
            if (r < n4 && k + 1 < n4) x1 = op_word(ops, (long)op * n4 * n4 + (long)(k + 1) * n4 + r);
            x0.x *= inv;  // powers of two: exact
            x0.y *= inv;
            x1.x *= inv;
            x1.y *= inv;
            split_h16(x0, h0, l0);
            split_h16(x1, h1, l1);
            wh[q >> 1] = (uint32_t)h0 | ((uint32_t)h1 << 16);
            wl[q >> 1] = (uint32_t)l0 | ((uint32_t)l1 << 16);
        }
        const int t = r / TC_M, row = r % TC_M, st = grp / 2, half = grp & 1;
        const long tile = ((long)op * mtiles + t) * nstage + st;
        const long idx = (tile * TC_TILE_BYTES + tile_off(row, half)) / 16;
        a_hi[idx] = make_uint4(wh[0], wh[1], wh[2], wh[3]);
        a_lo[idx] = make_uint4(wl[0], wl[1], wl[2], wl[3]);
    }
}

// Multipoles [node][n4] (FP32) -> scaled FP16 hi / lo [node][kpad] and the column scales t_j.
// One warp per node.
__global__ void k_split_mult_h16(long nnodes, int n4, int kpad, const float *__restrict__ m, uint16_t *hi,
                                 uint16_t *lo, float *cscale) {
    const int lane = threadIdx.x & 31;
    const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
    const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
    for (long node = warp; node < nnodes; node += nwarps) {
        const float *x = m + node * n4;
        float mx = 0.f;
        for (int k = lane; k < n4; k += 32) mx = fmaxf(mx, fabsf(x[k]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const float sc = h16_scale(mx), inv = 1.f / sc;
        if (lane == 0) cscale[node] = sc;
        for (int k = lane; k < kpad; k += 32) {
            uint16_t h, l;
            split_h16(k < n4 ? x[k] * inv : 0.f, h, l);
            hi[node * kpad + k] = h;
            lo[node * kpad + k] = l;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// FP64-class V-list M2L for the refinement residual: integer digit slices on the tensor cores.
//
// The Ozaki scheme (Ozaki, Ogita, Oishi, Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication", Numer. Algorithms 59, 2012),
// in its fixed-point form: each operator row r is scaled by a power of two s_r >= max |A_r.|,
// each multipole column j by t_j >= max |B_.j|, and the scaled values (in [-1, 1]) are cut into
// S signed digits of D = 42 / S bits (balanced base-2^D digits of rint(A_rk / s_r 2^42)),
//     A_rk / s_r = sum_i a_i(r,k) 2^(-D(i+1)) + e,   |a_0| <= 2^D, |a_i>0| <= 2^(D-1), |e| <= 2^-43.
// Digit i is stored as a_i 2^(-D i) (a power-of-two multiple of a small integer: exact in BF16),
// so the product of operator digit i and multipole digit l carries its weight 2^(-D(i+l))
// and the MMAs of one group k = i + l accumulate G_k 2^(-D k), G_k = sum_{i+l=k} sum_K a_i b_l.
// Groups 0, 1 and 2 get one TMEM accumulator each and stay exact in the FP32 accumulation:
// |G_k| <= 1.25 2^(2D) K < 2^24 (S = 6, D = 7: K <= 800; S = 7, D = 6: K <= 3200).  Groups
// 3 .. S-1 share a fourth accumulator, rounded at 2^-24 of a value 2^(-3D) below group 0
// (~2^-45 of s_r t_j per step of 16 K elements).  The epilogue combines the four in int64 fixed
// point, assembles the double times s_r t_j 2^(-2D) from its bits (integer instructions: the
// FP64 pipe is narrow) and adds it into the FP64 locals.  Digit pairs with i + l >= S are
// dropped: the result differs from the FP64 product by about 2^-40 of s_r t_j per term (~1e-11
// relative), far below the FP32 operator the refinement corrects.  S = 6 (7-bit digits, 21
// digit MMAs a step) where K allows it (orders up to 5), else S = 7 (6-bit digits, 28 MMAs).
//
// One CTA: one chunk of <= 128 pairs x one 128-row tile; accumulator g (g = 0..3) in TMEM
// columns [128 g, 128 g + 128).  Stage st holds K elements [16 st, 16 st + 16): the S operator
// digit tiles (128 x 16 BF16, 4 KB each, pre-packed contiguously: one bulk copy) and the S
// multipole digit tiles (128 x 16 BF16, gathered by cp.async).  Warp-specialised like k_m2l_tc:
// one thread issues the bulk copies, one the MMAs, six warps gather; they meet on mbarriers only.
// ---------------------------------------------------------------------------------------------

constexpr int OZ_M = 128, OZ_N = 128, OZ_KS = 16, OZ_ACC = 4;
constexpr int OZ_THREADS = 256, OZ_BPROD = 192;
constexpr int OZ_ATILE = OZ_M * OZ_KS * 2;                 // 4 KB
constexpr int OZ_BTILE = OZ_N * OZ_KS * 2;                 // 4 KB
constexpr int OZ_K7 = 800;                                  // largest K for 7-bit digits (S = 6)
static_assert(OZ_N * OZ_ACC <= 512, "TMEM columns");

template <int S> struct OzShape {
    static constexpr int D = 42 / S;                        // bits per digit
    static_assert(S * D == 42, "42-bit cut");
    static constexpr int STAGE = S * (OZ_ATILE + OZ_BTILE);  // 48 KB (S 6), 56 KB (S 7)
    static constexpr int NST = (200 * 1024) / STAGE;        // 4 or 3 stage buffers
    static constexpr int LAG = 1;                           // copy lag (NST - 2: 14.49 against 14.24 ms)
    static constexpr int SMEM = NST * STAGE;
};

// D FP32, A and B BF16, both K-major, M = 128; N in bits 17-22 per chunk.
constexpr uint32_t kIdescOz = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_M >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// BF16 bits of a float whose significand has at most 8 bits (exact: the low 16 bits are zero).
__device__ __forceinline__ uint16_t bf16_bits_exact(float v) {
    return (uint16_t)(__float_as_uint(v) >> 16);
}

// rint(v 2^s), rounding half to even, from the bits of v by integer arithmetic (no FP64 pipe);
// |v 2^s| < 2^62.  The same value as __double2ll_rn(ldexp(v, s)).
__device__ __forceinline__ long long scaled_rint_bits(double v, int s) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int E = (int)((u >> 52) & 0x7ff);
    unsigned long long M = u & 0xfffffffffffffULL;
    if (E != 0) M |= 1ULL << 52;                       // v = M 2^(max(E, 1) - 1075)
    const int sh = (E == 0 ? 1 : E) - 1075 + s;
    long long m;
    if (sh >= 0) {
        m = (long long)(M << sh);
    } else {
        const int k = -sh;
        if (k > 63) {
            m = 0;
        } else {
            const unsigned long long q = M >> k, rem = M & ((1ULL << k) - 1), half = 1ULL << (k - 1);
            m = (long long)(q + ((rem > half || (rem == half && (q & 1ULL))) ? 1ULL : 0ULL));
        }
    }
    return (u >> 63) ? -m : m;
}

// Balanced base-2^D digits of m = rint(x 2^42), |x| <= 1, stored scaled: dig[i] = a_i 2^(-D i)
// with x = sum_i a_i 2^(-D(i+1)) up to 2^-43 (a_i in [-2^(D-1), 2^(D-1)) for i >= 1,
// |a_0| <= 2^D).
template <int S>
__device__ __forceinline__ void oz_digits_of(long long m, uint16_t *dig) {
    constexpr int D = OzShape<S>::D;
    constexpr long long H = 1LL << (D - 1), MASK = (1LL << D) - 1;
#pragma unroll
    for (int i = S - 1; i > 0; --i) {
        const long long a = ((m + H) & MASK) - H;
        dig[i] = bf16_bits_exact((float)(int)a * __int_as_float((127 - D * i) << 23));  // a 2^(-D i)
        m = (m - a) >> D;  // exact: m - a is a multiple of 2^D
    }
    dig[0] = bf16_bits_exact((float)(int)m);
}

// Digits of ldexp(v, -e) (|v| < 2^e): the cut of the operator or multipole value v under its
// power-of-two scale 2^e.
template <int S>
__device__ __forceinline__ void oz_digits(double v, int e, uint16_t *dig) {
    oz_digits_of<S>(scaled_rint_bits(v, 42 - e), dig);
}

// trunc(v 2^s) toward zero from the bits of a float, |v 2^s| < 2^62.
__device__ __forceinline__ long long scaled_trunc_bits_f32(float v, int s) {
    const unsigned u = __float_as_uint(v);
    const int E = (int)((u >> 23) & 0xff);
    unsigned long long M = u & 0x7fffffu;
    if (E != 0) M |= 0x800000u;  // v = M 2^(max(E, 1) - 150)
    const int sh = (E == 0 ? 1 : E) - 150 + s;
    long long m = 0;
    if (sh >= 0)
        m = (long long)(M << sh);
    else if (sh > -24)
        m = (long long)(M >> -sh);
    return (u >> 31) ? -m : m;
}

// Digits of (h + l) 2^-e for a float-float value: rint from a 2^-16 fixed point of the exact sum
// (only the rounding of a value within 2^-16 of a half-way point can differ from the exact rint,
// by one unit of 2^-42, below the cut's own 2^-43).
template <int S>
__device__ __forceinline__ void oz_digits(float2 v, int e, uint16_t *dig) {
    const long long f = scaled_trunc_bits_f32(v.x, 58 - e) + scaled_trunc_bits_f32(v.y, 58 - e);
    oz_digits_of<S>((f + (1LL << 15)) >> 16, dig);
}

// Power-of-two scale >= m (1 for m == 0), returned as its exponent.
__device__ __forceinline__ int oz_scale_exp(double m) {
    if (!(m > 0.0)) return 0;
    int e;
    frexp(m, &e);  // m = f 2^e, f in [0.5, 1)
    return e;
}

// Exponent of the power-of-two scale of one operator row (n4 entries, stride n4): FP64 entries
// by the maximum of |x|'s bit patterns (for non-negative doubles their order is the integer
// order), float-float entries by the maximum of |hi| + |lo|.
__device__ __forceinline__ int row_scale_exp(const double *__restrict__ col0, int n4) {
    unsigned long long mb = 0;
    for (int k = 0; k < n4; ++k)
        mb = max(mb, (unsigned long long)__double_as_longlong(col0[(long)k * n4]) & 0x7fffffffffffffffULL);
    return oz_scale_exp(__longlong_as_double((long long)mb));
}
__device__ __forceinline__ int row_scale_exp(const float2 *__restrict__ col0, int n4) {
    float m = 0.f;
    for (int k = 0; k < n4; ++k) {
        const float2 x = col0[(long)k * n4];
        m = fmaxf(m, fabsf(x.x) + fabsf(x.y));
    }
    if (!(m > 0.f)) return 0;
    int e;
    frexpf(m, &e);  // m = f 2^e, f in [0.5, 1)
    return e;
}

// Row scales of the operators (FP64 or float-float, column-major n4 x n4 per op):
// sig[op][mtiles * 128] = s_r 2^(-2D) with s_r the power of two >= max_k |A_rk|, and the exponent
// of s_r.  One thread per (op, row); neighbouring threads read neighbouring rows of a column.
template <class OW>
__global__ void k_scale_ops_oz(int n4, int mtiles, int nops, int scale_exp, const OW *__restrict__ ops, double *sig,
                               int *sexp) {
    const int mpad = mtiles * OZ_M;
    const long total = (long)nops * mpad;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int r = (int)(i % mpad), op = (int)(i / mpad);
        const int e = r < n4 ? row_scale_exp(ops + (long)op * n4 * n4 + r, n4) : 0;
        sig[i] = ldexp(1.0, e - scale_exp);
        sexp[i] = e;
    }
}

// Operators (FP64 or float-float) -> digit tiles [op][row tile][stage][digit][4 KB] in the
// shared-memory layout (tile_off with 16 K elements of 2 bytes per row).  One thread per (op, row,
// group of 8 K elements): 8 reads, then one 16-byte store per digit.
// With H16 (float-float operators), the same pass also writes the scaled FP16 hi / lo tiles of
// the mixed contraction (k_pack_ops_h16's values and layout) from the row scales rscale: the
// operators are read once for both images.
template <int S, class OW, bool H16 = false>
__global__ void k_pack_ops_oz(int n4, int mtiles, int kpad, int nops, const OW *__restrict__ ops,
                              const int *__restrict__ sexp, uint4 *a, const float *__restrict__ rscale = nullptr,
                              uint4 *a_hi = nullptr, uint4 *a_lo = nullptr) {
    static_assert(!H16 || std::is_same<OW, float2>::value, "FP16 images from float-float operators");
    static_assert(OZ_M == TC_M && OZ_KS == TC_KS16 && OZ_ATILE == TC_TILE_BYTES, "one tile layout");
    const int nstage = kpad / OZ_KS, mpad = mtiles * OZ_M, ngrp = kpad / 8;
    const long total = (long)nops * ngrp * mpad;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int r = (int)(i % mpad);  // rows fastest: coalesced column reads
        const long rest = i / mpad;
        const int grp = (int)(rest % ngrp), op = (int)(rest / ngrp);
        const int e = sexp[(long)op * mpad + r];
        float inv = 1.f;
        if constexpr (H16) inv = 1.f / rscale[(long)op * mpad + r];  // a power of two: exact
        uint32_t w[S][4], wh[4], wl[4];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int k = grp * 8 + q;
            const OW v = (r < n4 && k < n4) ? ops[(long)op * n4 * n4 + (long)k * n4 + r] : OW{};
            uint16_t dig[S];
            oz_digits<S>(v, e, dig);
#pragma unroll
            for (int d = 0; d < S; ++d) {
                if (q & 1) w[d][q >> 1] |= (uint32_t)dig[d] << 16;
                else w[d][q >> 1] = dig[d];
            }
            if constexpr (H16) {
                float2 x = op_word(&v, 0);
                x.x *= inv;  // powers of two: exact
                x.y *= inv;
                uint16_t h, l;
                split_h16(x, h, l);
                if (q & 1) {
                    wh[q >> 1] |= (uint32_t)h << 16;
                    wl[q >> 1] |= (uint32_t)l << 16;
                } else {
                    wh[q >> 1] = h;
                    wl[q >> 1] = l;
                }
            }
        }
        const int t = r / OZ_M, row = r % OZ_M, st = grp / 2, half = grp & 1;
        const long tile = ((long)op * mtiles + t) * nstage + st, tbase = tile * S;
        const uint32_t off = tile_off(row, half);  // byte offset of the 16-byte piece
#pragma unroll
        for (int d = 0; d < S; ++d)
            a[((tbase + d) * OZ_ATILE + off) / 16] = make_uint4(w[d][0], w[d][1], w[d][2], w[d][3]);
        if constexpr (H16) {
            const long idx = (tile * TC_TILE_BYTES + off) / 16;
            a_hi[idx] = make_uint4(wh[0], wh[1], wh[2], wh[3]);
            a_lo[idx] = make_uint4(wl[0], wl[1], wl[2], wl[3]);
        }
    }
}

// Row scales of both images from one read of the float-float operators: the FP16 form's s_r
// (k_scale_ops_h16) and the digit form's exponent and s_r 2^(-2D) (k_scale_ops_oz), both from
// max_k (|hi| + |lo|).
__global__ void k_scale_ops_ff2(int n4, int mtiles, int nops, int scale_exp, const float2 *__restrict__ ops,
                                float *rscale, double *sig, int *sexp) {
    const int mpad = mtiles * OZ_M;
    const long total = (long)nops * mpad;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int r = (int)(i % mpad), op = (int)(i / mpad);
        float m = 0.f;
        if (r < n4) {
            const float2 *col0 = ops + (long)op * n4 * n4 + r;
            for (int k = 0; k < n4; ++k) {
                const float2 x = col0[(long)k * n4];
                m = fmaxf(m, fabsf(x.x) + fabsf(x.y));
            }
        }
        int e = 0;
        if (m > 0.f) frexpf(m, &e);  // m = f 2^e, f in [0.5, 1)
        rscale[i] = h16_scale(m);
        sig[i] = ldexp(1.0, e - scale_exp);
        sexp[i] = e;
    }
}

// Multipoles (FP64 [node][n4]) -> digits [node][stage][digit][16] and column scales tau = t_j.
// One warp per node.
template <int S>
__global__ void k_split_mult_oz(long nnodes, int n4, int kpad, const double *__restrict__ mult, uint16_t *b,
                                double *tau) {
    const int lane = threadIdx.x & 31;
    const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
    const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
    const int nstage = kpad / OZ_KS;
    for (long node = warp; node < nnodes; node += nwarps) {
        const double *m = mult + node * n4;
        double mx = 0.0;
        for (int k = lane; k < n4; k += 32) mx = fmax(mx, fabs(m[k]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const int e = oz_scale_exp(mx);
        if (lane == 0) tau[node] = ldexp(1.0, e);
        for (int k = lane; k < kpad; k += 32) {
            const double v = k < n4 ? m[k] : 0.0;
            uint16_t dig[S];
            oz_digits<S>(v, e, dig);
            const long base = ((node * nstage + k / OZ_KS) * S) * OZ_KS + (k % OZ_KS);
#pragma unroll
            for (int d = 0; d < S; ++d) b[base + (long)d * OZ_KS] = dig[d];
        }
    }
}

// Exponent e of a positive power of two 2^e (normal range), from its bits.
__device__ __forceinline__ int exp_of_pow2(double p) {
    return (int)((__double_as_longlong(p) >> 52) & 0x7ff) - 1023;
}

// The double nearest T 2^e (ties to even) for an integer 0 < |T| < 2^63, assembled from T's bits
// by integer instructions while the result is a normal number, else by an FP64 multiply.
__device__ __forceinline__ double pow2_scaled_ll(long long T, const int e0) {
    unsigned long long a = (unsigned long long)(T < 0 ? -T : T);
    int e = e0;
    int msb = 63 - __clzll((long long)a);
    if (msb > 52) {  // round the low bits away
        const int sh = msb - 52;
        const unsigned long long rem = a & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
        a >>= sh;
        if (rem > half || (rem == half && (a & 1ULL))) ++a;
        e += sh;
        if (a >> 53) {  // the rounding carried into bit 53: a = 2^53
            a >>= 1;
            ++e;
        }
        msb = 52;
    }
    const int E = msb + e + 1023;  // biased exponent of the result
    if (E < 1 || E > 2046) return ldexp((double)T, e0);  // subnormal or overflowing result
    const unsigned long long mant = ((a << (63 - msb)) & 0x7fffffffffffffffULL) >> 11;
    const unsigned long long bits = ((unsigned long long)(T < 0) << 63) | ((unsigned long long)E << 52) | mant;
    return __longlong_as_double((long long)bits);
}

// rint(x 2^s) of an FP32 value, |x 2^s| < 2^62, from its bits (ties away from zero; subnormal
// x, below 2^-126, count as zero).
__device__ __forceinline__ long long f32_fixed(float x, int s) {
    const unsigned u = __float_as_uint(x);
    const int E = (int)((u >> 23) & 0xff);
    if (E == 0) return 0;
    const long long m = (long long)((u & 0x7fffffu) | 0x800000u);  // x = m 2^(E - 150)
    const int sh = E - 150 + s;
    long long r;
    if (sh >= 0) r = m << sh;
    else if (sh < -25) r = 0;
    else r = (m + (1LL << (-sh - 1))) >> -sh;
    return (u >> 31) ? -r : r;
}

template <int S>
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_m2l_oz(int n4, int kpad, int mtiles, const int *__restrict__ chunks, const int *__restrict__ vsrc,
             const int *__restrict__ vtgt, const uint16_t *__restrict__ a, const double *__restrict__ sig,
             const uint16_t *__restrict__ bdig, const double *__restrict__ tau, double *local, int *err,
             const int *__restrict__ chunk_mol, const int *__restrict__ mol_active,
             const MolImg *__restrict__ mol_img) {
    // a merged plan (batch.cu): chunks of molecules that have stopped iterating are skipped whole,
    // the others read their molecule's own digit images
    if (chunk_mol) {
        const int m = chunk_mol[blockIdx.x];
        if (!mol_active[m]) return;
        a = mol_img[m].oz_a;
        sig = mol_img[m].oz_sig;
    }
    using SH = OzShape<S>;
    constexpr int NST = SH::NST, LAG = SH::LAG, STAGE = SH::STAGE;
    extern __shared__ __align__(1024) unsigned char oz_smem[];
    __shared__ __align__(8) uint64_t full_a[NST], full_b[NST], empty_bar[NST], acc_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int src_s[OZ_N], tgt_s[OZ_N];
    __shared__ int tau_e[OZ_N];
    __shared__ volatile int abort_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int op = chunks[3 * blockIdx.x], b = chunks[3 * blockIdx.x + 1], cnt = chunks[3 * blockIdx.x + 2];
    const int t = blockIdx.y;
    const int nstage = kpad / OZ_KS;
    // MMA width of this chunk: its pairs rounded up to 16; gathers and epilogue stop there too
    const int neff = max(16, (cnt + 15) & ~15);
    const uint32_t idesc = kIdescOz | ((uint32_t)(neff >> 3) << 17);
    if (tid < OZ_N) {
        const int sn = tid < cnt ? vsrc[b + tid] : -1;
        src_s[tid] = sn;
        tgt_s[tid] = tid < cnt ? vtgt[b + tid] : -1;
        tau_e[tid] = sn >= 0 ? exp_of_pow2(tau[sn]) : 0;
    }
    if (tid == 0) {
        abort_s = 0;
        for (int i = 0; i < NST; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_a[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full_b[i])), "r"(OZ_BPROD));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty_bar[i])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_bar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem_d = tmem_base;
    const long atile0 = ((long)op * mtiles + t) * nstage;

    if (warp == 0) {
        if (lane == 0) {  // operator digit tiles: one bulk copy per stage
            int issued = -1;
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % NST;
                if (st >= NST && !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((st / NST) - 1) & 1))) {
                    abort_s = 1;
                    break;
                }
                if (abort_s) break;
                const uint32_t fb = smem_u32(&full_a[buf]);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(S * OZ_ATILE)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        smem_u32(oz_smem + buf * STAGE)),
                    "l"(a + (atile0 + st) * (long)(S * OZ_ATILE / 2)), "r"(S * OZ_ATILE), "r"(fb)
                    : "memory");
                issued = st;
            }
            for (int s2 = max(0, issued - NST + 1); s2 <= issued; ++s2)
                if (!mbar_wait(smem_u32(&full_a[s2 % NST]), (uint32_t)((s2 / NST) & 1))) abort_s = 1;
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issue: S (S + 1) / 2 digit-pair MMAs per stage into 4 accumulators
            int last = -1;
            for (int st = 0; st < nstage; ++st) {
                const int buf = st % NST;
                const uint32_t par = (uint32_t)((st / NST) & 1);
                if (!mbar_wait(smem_u32(&full_a[buf]), par) || !mbar_wait(smem_u32(&full_b[buf]), par) || abort_s) {
                    abort_s = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t base = smem_u32(oz_smem + buf * STAGE);
#pragma unroll
                for (int k = 0; k < S; ++k) {
                    const int g = min(k, OZ_ACC - 1);
#pragma unroll
                    for (int i = 0; i <= k; ++i) {
                        const uint64_t ad = make_desc(base + i * OZ_ATILE, 128, 256);
                        const uint64_t bd = make_desc(base + S * OZ_ATILE + (k - i) * OZ_BTILE, 128, 256);
                        // the first MMA into each accumulator overwrites it
                        const bool first = st == 0 && i == 0 && k <= OZ_ACC - 1;
                        mma_bf16(tmem_d + (uint32_t)(g * OZ_N), ad, bd, idesc, first ? 0u : 1u);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&empty_bar[buf]))
                             : "memory");
                last = st;
            }
            if (last == nstage - 1) {
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&acc_bar))
                             : "memory");
            } else {
                abort_s = 1;
                if (last >= 0) mbar_wait(smem_u32(&empty_bar[last % NST]), (uint32_t)((last / NST) & 1));
            }
        }
    } else {  // multipole digits: neff rows x S digits x 2 pieces of 16 B per stage, 192 threads
        const int tq = tid - 64;
        int issued = -1;
        for (int st = 0; st < nstage; ++st) {
            const int buf = st % NST;
            if (st >= NST && !mbar_wait(smem_u32(&empty_bar[buf]), (uint32_t)(((st / NST) - 1) & 1))) {
                abort_s = 1;
                break;
            }
            if (abort_s) break;
            unsigned char *base = oz_smem + buf * STAGE;
            for (int i = tq; i < neff * S * 2; i += OZ_BPROD) {
                const int row = i / (S * 2), rem = i % (S * 2), d = rem >> 1, c = rem & 1;
                const uint32_t dst = smem_u32(base + S * OZ_ATILE + d * OZ_BTILE + tile_off(row, c));
                const int sn = src_s[row];
                const uint16_t *g = sn >= 0 ? bdig + (((long)sn * nstage + st) * S + d) * OZ_KS + 8 * c : bdig;
                cp_async16(dst, g, sn >= 0 ? 16u : 0u);
            }
            asm volatile("cp.async.commit_group;");
            issued = st;
            if (st >= LAG) {
                asm volatile("cp.async.wait_group %0;" ::"n"(LAG) : "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_b[(st - LAG) % NST]))
                             : "memory");
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int s2 = max(0, issued - LAG + 1); s2 <= issued; ++s2)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full_b[s2 % NST])) : "memory");
    }
    __syncthreads();
    bool ok = !abort_s;
    if (ok) ok = mbar_wait(smem_u32(&acc_bar), 0u);
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (!ok && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (ok) {
        // warp w: TMEM lanes 32 (w % 4) .. + 31 = rows, pair columns [64 (w / 4), + 64) below neff.
        // Integer epilogue (the FP64 pipe is narrow): T = (G_0 2^(2D) + G_1 2^D + G_2) 2^F +
        // rint(M 2^(2D+F)) in int64 with F = 24 (|G_0 2^(2D)| < 2^38, so |T| < 2^62; M kept to
        // 2^-(2D+24) of a group-0 unit, far below the cut's own error), then the double nearest
        // T 2^(e_r + e_j - 4D - F) is assembled from T's bits; s_r = 2^e_r and t_j = 2^e_j.
        constexpr int D = SH::D;
        const int lg = warp & 3, h = warp >> 2;
        const int row = t * OZ_M + 32 * lg + lane;
        const int erow = row < n4 ? exp_of_pow2(sig[(long)op * mtiles * OZ_M + row]) + 2 * D : 0;
#pragma unroll 1
        for (int c0 = 64 * h; c0 < min(64 * h + 64, neff); c0 += 16) {
            uint32_t v[OZ_ACC][16];
#pragma unroll
            for (int g = 0; g < OZ_ACC; ++g)
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15}, [%16];"
                    : "=r"(v[g][0]), "=r"(v[g][1]), "=r"(v[g][2]), "=r"(v[g][3]), "=r"(v[g][4]), "=r"(v[g][5]),
                      "=r"(v[g][6]), "=r"(v[g][7]), "=r"(v[g][8]), "=r"(v[g][9]), "=r"(v[g][10]), "=r"(v[g][11]),
                      "=r"(v[g][12]), "=r"(v[g][13]), "=r"(v[g][14]), "=r"(v[g][15])
                    : "r"(tmem_d + ((uint32_t)(32 * lg) << 16) + (uint32_t)(g * OZ_N + c0)));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < n4) {
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int tg = tgt_s[c0 + q];
                    constexpr int F = 24;
                    const long long g0 = __float2int_rn(__uint_as_float(v[0][q]));
                    const long long g1 = __float2int_rn(__uint_as_float(v[1][q]) * (float)(1 << D));
                    const long long g2 = __float2int_rn(__uint_as_float(v[2][q]) * (float)(1 << (2 * D)));
                    const long long T = (((g0 << (2 * D)) + (g1 << D) + g2) << F) +
                                        f32_fixed(__uint_as_float(v[3][q]), 2 * D + F);
                    if (tg >= 0 && T != 0)
                        atomicAdd(local + (long)tg * n4 + row,
                                  pow2_scaled_ll(T, erow + tau_e[c0 + q] - 4 * D - F));
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(512));
}

}  // namespace

bool m2l_tc_supported() {
    int dev = 0, major = 0, minor = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    return major == 10 && minor == 3;
}

// The CTA-pair kernel is opt-in (IBIM_TC_PAIR=1): on the 2,000-atom protein it takes 5.35 ms a
// launch against the one-CTA kernel's 3.9 ms.  Its 256-pair chunks fill 71 % of their slots
// against 83 %; the rest of the gap is not explained yet (ncu, 150-atom protein: tensor pipe
// active 30 %, 5 long-scoreboard stalls per issued instruction).
bool m2l_tc_pair() {
    static const bool on = [] {
        const char *v = std::getenv("IBIM_TC_PAIR");
        return v && v[0] == '1';
    }();
    return on;
}

// Operand form of the mixed path's tensor-core M2L: scaled FP16 hi / lo (default) or TF32 hi / lo
// (IBIM_TC_FP16=0, or the CTA-pair kernel).
static bool tc_fp16() {
    static const bool on = [] {
        const char *v = std::getenv("IBIM_TC_FP16");
        return !(v && v[0] == '0');
    }();
    return on && !m2l_tc_pair();
}

bool m2l_tc_fp16_form() { return tc_fp16(); }

// Launch form of the contraction (the plan's tuning, tuning.cpp): two CTAs of two row tiles per SM
// (2: one CTA's prologue and epilogue overlap the other's MMAs; 2.32 ms a launch on the 2,000-atom
// protein), one CTA of four row tiles per SM (4; 2.50 ms) or, FP16 form only, persistent (0: one
// CTA per SM walking units of two row tiles with double-buffered accumulators; 2.94 ms).

// Shapes and device buffers of the contraction's images (operators, multipoles, scales).
static void tc_alloc(Plan &P) {
    P.tc_h16 = tc_fp16();
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R;
    const int ks = P.tc_h16 ? TC_KS16 : TC_KS;
    P.tc_kpad = (n4 + ks - 1) / ks * ks;
    P.tc_mpad = (n4 + TC_M - 1) / TC_M * TC_M;
    // image sizes in floats (an FP16 image takes half the words)
    const size_t na = (size_t)std::max(1, P.nops) * P.tc_mpad * P.tc_kpad / (P.tc_h16 ? 2 : 1);
    const size_t nb = (size_t)P.tree.nnodes * P.tc_kpad / (P.tc_h16 ? 2 : 1);
    P.tc_a_hi.alloc(na, s);
    P.tc_a_lo.alloc(na, s);
    if (P.tc_h16) {
        P.tc_rsc.alloc((size_t)std::max(1, P.nops) * P.tc_mpad, s);
        P.tc_csc.alloc((size_t)P.tree.nnodes, s);
    }
    P.tc_b_hi.alloc(nb, s);
    P.tc_b_lo.alloc(nb, s);
    if (!P.tc_err.ptr) {
        P.tc_err.alloc(1, s);
        P.tc_err.zero();
    }
    // the contraction kernels' shared memory (above the 48 KB default)
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc<M2L_CHTC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   TcShape<M2L_CHTC>::SMEM));
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc<M2L_CHTC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   TcShape<M2L_CHTC>::SMEM));
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc<M2L_CHTC, false, 2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   TcShape<M2L_CHTC, 2, 2>::SMEM));
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, TCP_SMEM));
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc<M2L_CHTC, true, 2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   TcShape<M2L_CHTC, 2, 2>::SMEM));
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize, TC2_SMEM));
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc2h<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, Tc2hShape<1>::SMEM));
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc2h<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, Tc2hShape<2>::SMEM));
}

void m2l_tc_pack(Plan &P, const float2 *ff) {
    tc_alloc(P);
    if (!P.tc_h16) ff = nullptr;
    IBIM_REQUIRE(P.ops32.ptr || ff || P.nops == 0, "tensor-core images need the operators");
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R;
    const int mt = P.tc_mpad / TC_M;
    if (P.tc_h16) {
        if (P.nops > 0) {
            const long rows = (long)P.nops * P.tc_mpad, pieces = rows * (P.tc_kpad / 8);
            const int gs = (int)std::min<long>((rows + 255) / 256, 32L * P.ctx->num_sms);
            const int gp = (int)std::min<long>((pieces + 255) / 256, 64L * P.ctx->num_sms);
            uint4 *ah = reinterpret_cast<uint4 *>(P.tc_a_hi.ptr), *al = reinterpret_cast<uint4 *>(P.tc_a_lo.ptr);
            if (ff) {  // from the float-float operators of the FP64-class images
                (count_launch(), k_scale_ops_h16<float2><<<gs, 256, 0, s>>>(n4, mt, P.nops, ff, P.tc_rsc.ptr));
                (count_launch(), k_pack_ops_h16<float2><<<gp, 256, 0, s>>>(n4, mt, P.tc_kpad, P.nops, ff, P.tc_rsc.ptr,
                                                                           ah, al));
            } else {
                (count_launch(), k_scale_ops_h16<float><<<gs, 256, 0, s>>>(n4, mt, P.nops, P.ops32.ptr, P.tc_rsc.ptr));
                (count_launch(), k_pack_ops_h16<float><<<gp, 256, 0, s>>>(n4, mt, P.tc_kpad, P.nops, P.ops32.ptr,
                                                                          P.tc_rsc.ptr, ah, al));
            }
        }
    } else if (P.nops > 0) {
        (count_launch(), k_pack_ops_tc<<<8 * P.ctx->num_sms, 256, 0, s>>>(n4, mt, P.tc_kpad, P.nops, P.ops32.ptr,
                                                                      P.tc_a_hi.ptr, P.tc_a_lo.ptr));
    }
    IBIM_CHECK_LAUNCH();
}

// V-list M2L on the tensor cores; mult32 -> local32 (accumulating): chunks of 128 pairs against
// two row tiles per CTA, two CTAs per SM (or four row tiles, one CTA per SM).  (Chunks of 256 pairs against two row tiles, k_m2l_tc<256>, measured 5.0 ms
// against 3.9 ms on the 2,000-atom protein: the operator traffic falls but the chunks fill worse.)
void m2l_tc_run(Plan &P, TargetSet &S) {
    constexpr int N = M2L_CHTC;
    if (S.nchunks_tc == 0) return;
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R;
    if (P.tc_h16)
        (count_launch(), k_split_mult_h16<<<4 * P.ctx->num_sms, 256, 0, s>>>(
                             P.tree.nnodes, n4, P.tc_kpad, P.mult32.ptr, reinterpret_cast<uint16_t *>(P.tc_b_hi.ptr),
                             reinterpret_cast<uint16_t *>(P.tc_b_lo.ptr), P.tc_csc.ptr));
    else
        (count_launch(), k_split_mult_tc<<<4 * P.ctx->num_sms, 256, 0, s>>>(P.tree.nnodes, n4, P.tc_kpad, P.mult32.ptr,
                                                                            P.tc_b_hi.ptr, P.tc_b_lo.ptr));
    const int mt = P.tc_mpad / TC_M;
    IBIM_REQUIRE(!S.chunk_mol_tc.ptr || (P.mol_img.ptr && P.mol_active.ptr), "merged plan without its image table");
    ProfScope ps_(PROF_M2L_V, 2.0 * n4 * (double)n4 * S.nvpairs,
                  4.0 * 2.0 * ((double)P.tc_mpad * P.tc_kpad * P.nops + (double)P.tc_kpad * S.nvpairs));
    if (!P.tc_h16 && m2l_tc_pair() && !P.batched) {
        if (S.nchunks_tc2 == 0) return;
        const dim3 grid2(2 * S.nchunks_tc2, (mt + 2 * TC2_PT - 1) / (2 * TC2_PT));
        (count_launch(), k_m2l_tc2<<<grid2, TC_THREADS, TC2_SMEM, s>>>(
                             n4, P.tc_kpad, mt, S.v_chunk_tc2.ptr, S.v_src.ptr, S.v_tgt.ptr, P.tc_a_hi.ptr,
                             P.tc_a_lo.ptr, P.tc_b_hi.ptr, P.tc_b_lo.ptr, P.local32.ptr, P.tc_err.ptr));
        IBIM_CHECK_LAUNCH();
        return;
    }
    if (P.tc_h16 && (P.tune.tc_form == 6 || P.tune.tc_form == 7) && !P.batched) {
        // CTA pairs over chunks of up to 256 pairs: one (6) or two (7) row-tile pairs per CTA
        if (S.nchunks_tc2 == 0) return;
        const char *ah = reinterpret_cast<const char *>(P.tc_a_hi.ptr), *al = reinterpret_cast<const char *>(P.tc_a_lo.ptr);
        const char *bh = reinterpret_cast<const char *>(P.tc_b_hi.ptr), *bl = reinterpret_cast<const char *>(P.tc_b_lo.ptr);
        if (P.tune.tc_form == 6)
            (count_launch(), k_m2l_tc2h<1><<<dim3(2 * S.nchunks_tc2, (mt + 1) / 2), TC_THREADS, Tc2hShape<1>::SMEM, s>>>(
                                 n4, P.tc_kpad, mt, S.v_chunk_tc2.ptr, S.v_src.ptr, S.v_tgt.ptr, ah, al, bh, bl,
                                 P.tc_rsc.ptr, P.tc_csc.ptr, P.local32.ptr, P.tc_err.ptr));
        else
            (count_launch(), k_m2l_tc2h<2><<<dim3(2 * S.nchunks_tc2, (mt + 3) / 4), TC_THREADS, Tc2hShape<2>::SMEM, s>>>(
                                 n4, P.tc_kpad, mt, S.v_chunk_tc2.ptr, S.v_src.ptr, S.v_tgt.ptr, ah, al, bh, bl,
                                 P.tc_rsc.ptr, P.tc_csc.ptr, P.local32.ptr, P.tc_err.ptr));
        IBIM_CHECK_LAUNCH();
        return;
    }
    if (P.tc_h16 && P.tune.tc_form == 0 && !P.batched) {
        static_assert(N == 128, "persistent form: 128-pair chunks");
        const int nunits = S.nchunks_tc * ((mt + TCP_RT - 1) / TCP_RT);
        const int grid = std::min(nunits, P.ctx->num_sms);
        (count_launch(), k_m2l_tc_persist<<<grid, TCP_THREADS, TCP_SMEM, s>>>(
                             n4, P.tc_kpad, mt, nunits, S.v_chunk_tc.ptr, S.v_src.ptr, S.v_tgt.ptr, P.tc_a_hi.ptr,
                             P.tc_a_lo.ptr, P.tc_b_hi.ptr, P.tc_b_lo.ptr, P.tc_rsc.ptr, P.tc_csc.ptr, P.local32.ptr,
                             P.tc_err.ptr));
        IBIM_CHECK_LAUNCH();
        return;
    }
    if (P.tune.tc_form != 4) {
        using SH2 = TcShape<N, 2, 2>;
        const dim3 grid(S.nchunks_tc, (mt + SH2::RT - 1) / SH2::RT);
        auto kern = P.tc_h16 ? k_m2l_tc<N, true, 2, 2> : k_m2l_tc<N, false, 2, 2>;
        (count_launch(), kern<<<grid, TC_THREADS, SH2::SMEM, s>>>(
                             n4, P.tc_kpad, mt, S.v_chunk_tc.ptr, S.v_src.ptr, S.v_tgt.ptr, P.tc_a_hi.ptr,
                             P.tc_a_lo.ptr, P.tc_b_hi.ptr, P.tc_b_lo.ptr, P.tc_rsc.ptr, P.tc_csc.ptr, P.local32.ptr,
                             P.tc_err.ptr, S.chunk_mol_tc.ptr, P.mol_active.ptr, P.mol_img.ptr));
        IBIM_CHECK_LAUNCH();
        return;
    }
    const dim3 grid(S.nchunks_tc, (mt + TcShape<N>::RT - 1) / TcShape<N>::RT);
    auto kern = P.tc_h16 ? k_m2l_tc<N, true> : k_m2l_tc<N, false>;
    (count_launch(), kern<<<grid, TC_THREADS, TcShape<N>::SMEM, s>>>(
                         n4, P.tc_kpad, mt, S.v_chunk_tc.ptr, S.v_src.ptr, S.v_tgt.ptr, P.tc_a_hi.ptr, P.tc_a_lo.ptr,
                         P.tc_b_hi.ptr, P.tc_b_lo.ptr, P.tc_rsc.ptr, P.tc_csc.ptr, P.local32.ptr, P.tc_err.ptr,
                         S.chunk_mol_tc.ptr, P.mol_active.ptr, P.mol_img.ptr));
    IBIM_CHECK_LAUNCH();
}

// Digit tiles of the FP64 operators, or of the float-float ones when ff is given: 6 digits of 7
// bits where K <= 800 (orders up to 5), else 7 of 6 bits.
// Shapes and device buffers of the digit images (nops > 0).
static void oz_alloc(Plan &P) {
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R;
    P.oz_kpad = (n4 + OZ_KS - 1) / OZ_KS * OZ_KS;
    P.oz_mtiles = (n4 + OZ_M - 1) / OZ_M;
    P.oz_s = P.oz_kpad <= OZ_K7 ? 6 : 7;
    const int S = P.oz_s, nstage = P.oz_kpad / OZ_KS;
    P.oz_a.alloc((size_t)P.nops * P.oz_mtiles * nstage * S * (OZ_ATILE / 2), s);
    P.oz_sig.alloc((size_t)P.nops * P.oz_mtiles * OZ_M, s);
    P.oz_b.alloc((size_t)P.tree.nnodes * nstage * S * OZ_KS, s);
    P.oz_tau.alloc((size_t)P.tree.nnodes, s);
    if (!P.tc_err.ptr) {
        P.tc_err.alloc(1, s);
        P.tc_err.zero();
    }
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_oz<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, OzShape<6>::SMEM));
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_oz<7>, cudaFuncAttributeMaxDynamicSharedMemorySize, OzShape<7>::SMEM));
}

void m2l_oz_pack(Plan &P, const float2 *ff) {
    if (P.nops == 0) return;
    IBIM_REQUIRE(P.ops64.ptr || ff, "digit images need the FP64-class operators");
    oz_alloc(P);
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R;
    const int S = P.oz_s;
    const long rows = (long)P.nops * P.oz_mtiles * OZ_M;
    DevBuf<int> sexp;
    sexp.alloc((size_t)rows, s);
    const long pieces = rows * (P.oz_kpad / 8);
    const int gs = (int)std::min<long>((rows + 255) / 256, 32L * P.ctx->num_sms);
    const int gp = (int)std::min<long>((pieces + 255) / 256, 64L * P.ctx->num_sms);
    const int sc = 2 * (42 / S);  // 2^(-2D) folded into the row scale
    uint4 *a = reinterpret_cast<uint4 *>(P.oz_a.ptr);
    if (ff)
        (count_launch(), k_scale_ops_oz<float2><<<gs, 256, 0, s>>>(n4, P.oz_mtiles, P.nops, sc, ff, P.oz_sig.ptr,
                                                                   sexp.ptr));
    else
        (count_launch(), k_scale_ops_oz<double><<<gs, 256, 0, s>>>(n4, P.oz_mtiles, P.nops, sc, P.ops64.ptr,
                                                                   P.oz_sig.ptr, sexp.ptr));
    auto pack = [&](auto kf, auto kd) {
        if (ff)
            (count_launch(), kf<<<gp, 256, 0, s>>>(n4, P.oz_mtiles, P.oz_kpad, P.nops, ff, sexp.ptr, a, nullptr,
                                                   nullptr, nullptr));
        else
            (count_launch(), kd<<<gp, 256, 0, s>>>(n4, P.oz_mtiles, P.oz_kpad, P.nops, P.ops64.ptr, sexp.ptr, a,
                                                   nullptr, nullptr, nullptr));
    };
    if (S == 6)
        pack(k_pack_ops_oz<6, float2>, k_pack_ops_oz<6, double>);
    else
        pack(k_pack_ops_oz<7, float2>, k_pack_ops_oz<7, double>);
    IBIM_CHECK_LAUNCH();
}

// Words of a and b (n 32-bit words each) that differ, added into *cnt.
__global__ void k_count_diff(long n, const uint32_t *__restrict__ a, const uint32_t *__restrict__ b,
                             unsigned long long *cnt) {
    unsigned long long c = 0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        c += a[i] != b[i];
    if (c) atomicAdd(cnt, c);
}

// Both images of the float-float operators in one pass over them: the digit tiles and scales of
// the FP64-class contraction and the scaled FP16 tiles and row scales of the mixed one, equal word
// for word to those m2l_oz_pack and m2l_tc_pack make from the same operators (two kernels instead
// of four: the 8 bytes an entry are read twice instead of four times).
void m2l_pack_images_ff(Plan &P, const float2 *ff) {
    IBIM_REQUIRE(tc_fp16(), "one-pass images: the scaled FP16 form only");
    IBIM_REQUIRE(ff || P.nops == 0, "one-pass images need the float-float operators");
    tc_alloc(P);
    if (P.nops == 0) return;
    oz_alloc(P);
    IBIM_REQUIRE(P.oz_kpad == P.tc_kpad && P.oz_mtiles * OZ_M == P.tc_mpad, "image shapes differ");
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R, S = P.oz_s;
    const long rows = (long)P.nops * P.oz_mtiles * OZ_M, pieces = rows * (P.oz_kpad / 8);
    DevBuf<int> sexp;
    sexp.alloc((size_t)rows, s);
    const int gs = (int)std::min<long>((rows + 255) / 256, 32L * P.ctx->num_sms);
    const int gp = (int)std::min<long>((pieces + 255) / 256, 64L * P.ctx->num_sms);
    (count_launch(), k_scale_ops_ff2<<<gs, 256, 0, s>>>(n4, P.oz_mtiles, P.nops, 2 * (42 / S), ff, P.tc_rsc.ptr,
                                                        P.oz_sig.ptr, sexp.ptr));
    uint4 *a = reinterpret_cast<uint4 *>(P.oz_a.ptr), *ah = reinterpret_cast<uint4 *>(P.tc_a_hi.ptr),
          *al = reinterpret_cast<uint4 *>(P.tc_a_lo.ptr);
    if (S == 6)
        (count_launch(), k_pack_ops_oz<6, float2, true><<<gp, 256, 0, s>>>(n4, P.oz_mtiles, P.oz_kpad, P.nops, ff,
                                                                         sexp.ptr, a, P.tc_rsc.ptr, ah, al));
    else
        (count_launch(), k_pack_ops_oz<7, float2, true><<<gp, 256, 0, s>>>(n4, P.oz_mtiles, P.oz_kpad, P.nops, ff,
                                                                         sexp.ptr, a, P.tc_rsc.ptr, ah, al));
    IBIM_CHECK_LAUNCH();
}

// The one-pass images of m2l_pack_images_ff against those of m2l_oz_pack and m2l_tc_pack from the
// same operators, word for word (a check for tests, IBIM_CHECK_IMAGES=1); the plan keeps the
// four-kernel images.  Throws when a word differs.
void m2l_check_images_ff(Plan &P, const float2 *ff) {
    if (P.nops == 0) return;
    cudaStream_t s = P.ctx->stream;
    DevBuf<uint16_t> oz_a = std::move(P.oz_a);
    DevBuf<double> oz_sig = std::move(P.oz_sig);
    DevBuf<float> a_hi = std::move(P.tc_a_hi), a_lo = std::move(P.tc_a_lo), rsc = std::move(P.tc_rsc);
    m2l_oz_pack(P, ff);
    m2l_tc_pack(P, ff);
    DevBuf<unsigned long long> cnt;
    cnt.alloc(5, s);
    cnt.zero();
    auto diff = [&](const void *x, size_t xbytes, const void *y, size_t ybytes, int slot) {
        IBIM_REQUIRE(xbytes == ybytes && xbytes % 4 == 0, "image sizes differ");
        const long n = (long)(xbytes / 4);
        if (n == 0) return;
        (count_launch(), k_count_diff<<<(int)std::min<long>(div_up(n, 256), 8L * P.ctx->num_sms), 256, 0, s>>>(
                             n, static_cast<const uint32_t *>(x), static_cast<const uint32_t *>(y), cnt.ptr + slot));
        IBIM_CHECK_LAUNCH();
    };
    diff(oz_a.ptr, oz_a.n * 2, P.oz_a.ptr, P.oz_a.n * 2, 0);
    diff(oz_sig.ptr, oz_sig.n * 8, P.oz_sig.ptr, P.oz_sig.n * 8, 1);
    diff(a_hi.ptr, a_hi.n * 4, P.tc_a_hi.ptr, P.tc_a_hi.n * 4, 2);
    diff(a_lo.ptr, a_lo.n * 4, P.tc_a_lo.ptr, P.tc_a_lo.n * 4, 3);
    diff(rsc.ptr, rsc.n * 4, P.tc_rsc.ptr, P.tc_rsc.n * 4, 4);
    unsigned long long h[5];
    cnt.download(h, 5);
    IBIM_CUDA(cudaStreamSynchronize(s));
    static const char *what[5] = {"digit tiles", "digit row scales", "FP16 hi tiles", "FP16 lo tiles",
                                  "FP16 row scales"};
    for (int i = 0; i < 5; ++i)
        if (h[i]) throw Error(IBIM_ERR_CUDA, std::string("one-pass operator images differ: ") + what[i]);
}

// V-list M2L of the FP64 operator by digit products on the tensor cores; mult -> local.
void m2l_oz_run(Plan &P, const TargetSet &S) {
    if (S.nchunks_oz == 0) return;
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R, ns = P.oz_s;
    const int gsplit = 4 * P.ctx->num_sms;
    if (ns == 6)
        (count_launch(), k_split_mult_oz<6><<<gsplit, 256, 0, s>>>(P.tree.nnodes, n4, P.oz_kpad, P.mult.ptr,
                                                                   P.oz_b.ptr, P.oz_tau.ptr));
    else
        (count_launch(), k_split_mult_oz<7><<<gsplit, 256, 0, s>>>(P.tree.nnodes, n4, P.oz_kpad, P.mult.ptr,
                                                                   P.oz_b.ptr, P.oz_tau.ptr));
    const dim3 grid(S.nchunks_oz, P.oz_mtiles);
    IBIM_REQUIRE(!S.chunk_mol_oz.ptr || (P.mol_img.ptr && P.mol_active.ptr), "merged plan without its image table");
    {
        const double nst = P.oz_kpad / OZ_KS;
        ProfScope ps_(PROF_M2L_VOZ, 2.0 * n4 * (double)n4 * S.nvpairs,
                      2.0 * ns * nst * OZ_KS * ((double)P.oz_mtiles * OZ_M * P.nops + (double)S.nvpairs));
        auto kern = ns == 6 ? k_m2l_oz<6> : k_m2l_oz<7>;
        const int smem = ns == 6 ? OzShape<6>::SMEM : OzShape<7>::SMEM;
        (count_launch(), kern<<<grid, OZ_THREADS, smem, s>>>(n4, P.oz_kpad, P.oz_mtiles, S.v_chunk_oz.ptr, S.v_src.ptr,
                                                            S.v_tgt.ptr, P.oz_a.ptr, P.oz_sig.ptr, P.oz_b.ptr,
                                                            P.oz_tau.ptr, P.local.ptr, P.tc_err.ptr, S.chunk_mol_oz.ptr,
                                                            P.mol_active.ptr, P.mol_img.ptr));
    }
    IBIM_CHECK_LAUNCH();
}

int m2l_tc_error(Plan &P) {
    if (!P.tc_err.ptr) return 0;  // allocated by the first image pack of either kind
    int e = 0;
    P.tc_err.download(&e, 1);
    IBIM_CUDA(cudaStreamSynchronize(P.ctx->stream));
    return e;
}

}  // namespace ibim
