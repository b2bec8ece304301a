// V-list M2L of the mixed-precision path on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// Per operator o (level, lattice offset) the V-list pairs form a dense contraction
//     L[tgt_j] += K_o . M[src_j]        K_o: 4p^3 x 4p^3,  j = pairs of the operator
// computed as D[128 rows x 128 pairs] (FP32, in TMEM) += A[128 x K] . B[K x 128 pairs] with
// kind::tf32 MMAs (M = 128, N = 128, K = 8 per instruction).  FP32 accuracy comes from the
// 3xTF32 split: A = A_hi + A_lo, B = B_hi + B_lo with hi = x rounded to TF32 and lo = x - hi, and
// D accumulates A_hi.B_hi + A_hi.B_lo + A_lo.B_hi (the dropped A_lo.B_lo is below FP32 rounding).
//
// Operand staging: operator rows (padded to 128) and the pairs' multipoles (gathered by source
// node) are copied with cp.async into shared memory in the canonical no-swizzle K-major layout
// (8-row x 16-byte core matrices; K-direction core-matrix stride 128 B, row-group stride 1 KB),
// 32 K-elements per stage.  One elected thread issues the MMAs and commits them to an mbarrier;
// every wait is bounded and reports through an error flag instead of hanging.  The epilogue
// reads the accumulator with tcgen05.ld (each warp its 32 TMEM lanes) and adds it into the
// target nodes' local expansions.

#include <cstdint>

#include "fmm_common.cuh"

namespace ibim {

namespace {

constexpr int TC_M = 128, TC_N = 128, TC_KS = 32;  // rows, pairs, K elements per stage
constexpr int TC_THREADS = 128;
constexpr int TC_TILE_BYTES = TC_M * TC_KS * 4;    // 16 KB per operand tile
constexpr long TC_WAIT_LIMIT = 1L << 20;           // bounded mbarrier polling

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

// Instruction descriptor: D FP32, A and B TF32, both K-major, M = 128, N = 128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                            ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
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

// Byte offset of element (row, k) of a 128 x 32 tile in the canonical no-swizzle K-major layout:
// core matrix (row / 8, k / 4) at ((row / 8) * 8 + k / 4) * 128, row % 8 at 16 B, k % 4 at 4 B.
__device__ __forceinline__ uint32_t tile_off(int row, int kchunk) {
    return (uint32_t)((((row >> 3) << 3) + kchunk) * 128 + (row & 7) * 16);
}

__global__ void __launch_bounds__(TC_THREADS) k_m2l_tc(int n4, int kpad, int mpad, const int *__restrict__ chunks,
                                                       const int *__restrict__ vsrc, const int *__restrict__ vtgt,
                                                       const float *__restrict__ a_hi, const float *__restrict__ a_lo,
                                                       const float *__restrict__ b_hi, const float *__restrict__ b_lo,
                                                       float *local, int *err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int src_s[TC_N], tgt_s[TC_N];
    unsigned char *sAh = tc_smem, *sAl = tc_smem + TC_TILE_BYTES, *sBh = tc_smem + 2 * TC_TILE_BYTES,
                  *sBl = tc_smem + 3 * TC_TILE_BYTES;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int op = chunks[3 * blockIdx.x], b = chunks[3 * blockIdx.x + 1], cnt = chunks[3 * blockIdx.x + 2];
    const int row0 = blockIdx.y * TC_M;
    src_s[tid] = tid < cnt ? vsrc[b + tid] : -1;
    tgt_s[tid] = tid < cnt ? vtgt[b + tid] : -1;
    const uint32_t mb = smem_u32(&mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(TC_N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem_d = tmem_base;
    const float *Ah = a_hi + ((long)op * mpad + row0) * kpad;
    const float *Al = a_lo + ((long)op * mpad + row0) * kpad;
    bool ok = true;
    const int nstage = kpad / TC_KS;
    for (int st = 0; st < nstage && ok; ++st) {
        const int k0 = st * TC_KS;
        // 4 tiles x 128 rows x 8 chunks of 16 B; thread tid copies rows tid (all chunks)
        {
            const int r = tid;
            const float *ga_h = Ah + (long)r * kpad + k0, *ga_l = Al + (long)r * kpad + k0;
            const int sn = src_s[r];
            const float *gb_h = sn >= 0 ? b_hi + (long)sn * kpad + k0 : b_hi;
            const float *gb_l = sn >= 0 ? b_lo + (long)sn * kpad + k0 : b_lo;
            const uint32_t nb = sn >= 0 ? 16u : 0u;
#pragma unroll
            for (int c = 0; c < TC_KS / 4; ++c) {
                const uint32_t o = tile_off(r, c);
                cp_async16(smem_u32(sAh + o), ga_h + 4 * c, 16u);
                cp_async16(smem_u32(sAl + o), ga_l + 4 * c, 16u);
                cp_async16(smem_u32(sBh + o), sn >= 0 ? (const void *)(gb_h + 4 * c) : (const void *)gb_h, nb);
                cp_async16(smem_u32(sBl + o), sn >= 0 ? (const void *)(gb_l + 4 * c) : (const void *)gb_l, nb);
            }
        }
        asm volatile("cp.async.commit_group;");
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
            for (int s = 0; s < TC_KS / 8; ++s) {
                // K = 8 TF32 = 2 core matrices along K: advance 256 B per step
                const uint64_t ah = make_desc(smem_u32(sAh) + 256 * s, 128, 1024);
                const uint64_t al = make_desc(smem_u32(sAl) + 256 * s, 128, 1024);
                const uint64_t bh = make_desc(smem_u32(sBh) + 256 * s, 128, 1024);
                const uint64_t bl = make_desc(smem_u32(sBl) + 256 * s, 128, 1024);
                mma_tf32(tmem_d, ah, bh, (st > 0 || s > 0) ? 1u : 0u);
                mma_tf32(tmem_d, ah, bl, 1u);
                mma_tf32(tmem_d, al, bh, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                         : "memory");
        }
        // every thread waits for this stage's MMAs before the tiles are overwritten
        ok = __syncthreads_and(mbar_wait(mb, (uint32_t)(st & 1)) ? 1 : 0) != 0;
        if (!ok) {
            if (tid == 0) atomicExch(err, 1);
            // give the stage one more bounded wait before the accumulator is released
            mbar_wait(mb, (uint32_t)(st & 1));
            __syncthreads();
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (ok) {
        // epilogue: warp w owns TMEM lanes 32w..32w+31 = operator rows row0 + 32w + lane
        const int row = row0 + 32 * warp + lane;
        const uint32_t taddr = tmem_d + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < TC_N; c0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                : "r"(taddr + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < n4) {
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int t = tgt_s[c0 + q];
                    if (t >= 0) atomicAdd(local + (long)t * n4 + row, __uint_as_float(v[q]));
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(TC_N));
}

// hi = x rounded to TF32 (10 explicit mantissa bits, to nearest even), lo = x - hi.
__device__ __forceinline__ float tf32_round(float x) {
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x0fffu + ((u >> 13) & 1u);
    u &= 0xffffe000u;
    return __uint_as_float(u);
}

// Operators (column-major n4 x n4 per op, FP32) -> row-major [mpad][kpad] hi / lo, zero padded.
__global__ void k_pack_ops_tc(int n4, int mpad, int kpad, int nops, const float *__restrict__ ops, float *a_hi,
                              float *a_lo) {
    const long total = (long)nops * mpad * kpad;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i % kpad);
        const long rr = i / kpad;
        const int row = (int)(rr % mpad);
        const int op = (int)(rr / mpad);
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

}  // namespace

bool m2l_tc_supported() {
    int dev = 0, major = 0, minor = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    return major == 10 && minor == 3;
}

void m2l_tc_prepare(Plan &P) {
    if (P.tc_ready) return;
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R;
    P.tc_kpad = (n4 + TC_KS - 1) / TC_KS * TC_KS;
    P.tc_mpad = (n4 + TC_M - 1) / TC_M * TC_M;
    const size_t na = (size_t)std::max(1, P.nops) * P.tc_mpad * P.tc_kpad;
    P.tc_a_hi.alloc(na, s);
    P.tc_a_lo.alloc(na, s);
    if (P.nops > 0)
        (count_launch(), k_pack_ops_tc<<<8 * P.ctx->num_sms, 256, 0, s>>>(n4, P.tc_mpad, P.tc_kpad, P.nops, P.ops32.ptr,
                                                                      P.tc_a_hi.ptr, P.tc_a_lo.ptr));
    P.tc_b_hi.alloc((size_t)P.tree.nnodes * P.tc_kpad, s);
    P.tc_b_lo.alloc((size_t)P.tree.nnodes * P.tc_kpad, s);
    P.tc_err.alloc(1, s);
    P.tc_err.zero();
    IBIM_CHECK_LAUNCH();
    IBIM_CUDA(cudaFuncSetAttribute(k_m2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * TC_TILE_BYTES));
    P.tc_ready = true;
}

// V-list M2L on the tensor cores; mult32 -> local32 (accumulating).
void m2l_tc_run(Plan &P, TargetSet &S) {
    if (S.nchunks_tc == 0) return;
    cudaStream_t s = P.ctx->stream;
    const int n4 = 4 * P.R;
    (count_launch(), k_split_mult_tc<<<4 * P.ctx->num_sms, 256, 0, s>>>(P.tree.nnodes, n4, P.tc_kpad, P.mult32.ptr,
                                                                        P.tc_b_hi.ptr, P.tc_b_lo.ptr));
    const dim3 grid(S.nchunks_tc, P.tc_mpad / TC_M);
    {
        ProfScope ps_(PROF_M2L_V, 2.0 * n4 * (double)n4 * S.nvpairs,
                      4.0 * 2.0 * ((double)P.tc_mpad * P.tc_kpad * P.nops + (double)P.tc_kpad * S.nvpairs));
        (count_launch(), k_m2l_tc<<<grid, TC_THREADS, 4 * TC_TILE_BYTES, s>>>(
                             n4, P.tc_kpad, P.tc_mpad, S.v_chunk_tc.ptr, S.v_src.ptr, S.v_tgt.ptr, P.tc_a_hi.ptr,
                             P.tc_a_lo.ptr, P.tc_b_hi.ptr, P.tc_b_lo.ptr, P.local32.ptr, P.tc_err.ptr));
    }
    IBIM_CHECK_LAUNCH();
}

int m2l_tc_error(Plan &P) {
    if (!P.tc_ready) return 0;
    int e = 0;
    P.tc_err.download(&e, 1);
    IBIM_CUDA(cudaStreamSynchronize(P.ctx->stream));
    return e;
}

}  // namespace ibim
