/*
 * mlp_tc.cuh - the surrogate's GEMM on the fifth-generation tensor cores
 * (tcgen05, accumulator in tensor memory).  Included by mlp.cu inside its
 * anonymous namespace, after the bf16 typedef, gelu() and the EPI_* codes.
 *
 * C[R, Cc] = sum_l A(r, l) B(c, l) over the reduction range of blockIdx.z's
 * slice, one CTA of 128 threads per 128 x BN output tile (BN = 64 or 32):
 * the M = 128, N = BN shape of tcgen05.mma.cta_group::1.kind::f16 with BF16
 * operands and an FP32 accumulator of BN TMEM columns.
 *
 * Operands: the threads stage K-chunks of 64 into shared memory without
 * swizzle, in 8 x 16-byte core matrices of 128 contiguous bytes, core
 * matrix (g, j) (row group g, reduction group j) at byte (g * 8 + j) * 128
 * of the tile.  Untransposed operands are K-major (a core-matrix row holds
 * 8 reduction indices of one row); transposed ones (the weight gradient's
 * operands, stored with the rows contiguous) are staged MN-major (a
 * core-matrix row holds 8 rows at one reduction index) and flagged so in
 * the instruction descriptor, which makes both stagings plain 16-byte
 * copies.  In the matrix descriptor the offset between reduction groups is
 * 128 and between row groups 1024.  One MMA of K = 16 covers two reduction
 * groups, so MMA kk of a chunk starts 256 * kk bytes into each tile.
 *
 * Pipeline: four shared-memory stages filled by cp.async (16 bytes per
 * copy, zero-filled outside the matrix), so a 256-deep reduction has all its
 * operands in flight at once; one thread issues each chunk's four MMAs and
 * commits them to the stage's mbarrier, which frees the stage for the chunk
 * four later.
 *
 * Epilogue: tcgen05.ld of 32 lanes x 16 columns per warp (warp w owns TMEM
 * lanes 32w..32w+31, one output row per thread), then the same fused
 * epilogues as the mma.sync kernel, stored 16 columns per thread.
 *
 * Every wait is bounded by the global timer (one second); a CTA that gives
 * up writes NaN into its tile, so the result cannot pass for a product.
 */
#pragma once

constexpr int TBM = 128, TBK = 64, TNT = 128;
constexpr uint32_t TC_A_BYTES = TBM * TBK * 2;                 /* 16 KB */
constexpr uint64_t TC_WAIT_NS = 1000000000ull;

constexpr int TC_STAGES = 4;                                   /* K = 256 fits in flight at once */

template <int BN>
struct TcShape {
    static constexpr uint32_t B_BYTES = BN * TBK * 2;
    static constexpr uint32_t STAGE = TC_A_BYTES + B_BYTES;
    static constexpr uint32_t BARS = TC_STAGES * STAGE;         /* one mbarrier per stage */
    static constexpr uint32_t TADDR = BARS + 8 * TC_STAGES;     /* the TMEM address */
    static constexpr uint32_t SMEM = TADDR + 16;
};

/* kind::f16 instruction descriptor: FP32 accumulator (bits 4-5 = 1), BF16 A
   and B (bits 7-9, 10-12 = 1), A and B major-ness (bits 15, 16: 0 = K-major,
   1 = MN-major), N >> 3 at bits 17-22, M >> 4 at bits 24-28. */
template <int BN, bool TA, bool TB>
__device__ __forceinline__ constexpr uint32_t tc_idesc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((TA ? 1u : 0u) << 15) | ((TB ? 1u : 0u) << 16) |
           ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);
}

__device__ __forceinline__ uint64_t tc_clock_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* Shared-memory matrix descriptor, no swizzle: start address >> 4 (bits
   0-13), leading byte offset >> 4 (16-29), stride byte offset >> 4 (32-45),
   descriptor version 1 (bits 46-47).  Both tile layouts below put core
   matrix (g, j) (8-row group g, 8-wide reduction group j) at byte
   (g * TBK/8 + j) * 128, so the offset between reduction groups is 128 and
   between row groups TBK * 16 in either major-ness. */
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) |
           ((uint64_t)((uint32_t)(TBK * 16) >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

/* Wait for the phase of the given parity to complete; false after the time limit. */
__device__ __forceinline__ bool tc_mbar_wait(uint32_t bar, uint32_t parity, uint64_t t_end) {
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (tc_clock_ns() > t_end) return false;
    }
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

/* 32 lanes x 16 consecutive FP32 columns: thread t of the warp gets lane
   (base lane + t), columns col..col+15. */
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
                   "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]),
                   "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_cp16(uint32_t dst, const void *src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void tc_cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

/* Wait until at most n (0..TC_STAGES-1) of this thread's copy groups are pending. */
__device__ __forceinline__ void tc_cp_wait(int n) {
    switch (n) {
        case 0: asm volatile("cp.async.wait_group 0;" ::: "memory"); break;
        case 1: asm volatile("cp.async.wait_group 1;" ::: "memory"); break;
        case 2: asm volatile("cp.async.wait_group 2;" ::: "memory"); break;
        default: asm volatile("cp.async.wait_group 3;" ::: "memory"); break;
    }
}

/* Operand staging with cp.async, 16 bytes per copy, zero-filled outside the
   matrix.  X(r, l) = TR ? X[l*ld + r] : X[r*ld + l]; rows >= R and
   reduction indices >= L are zero (R, L, r0, l0 are multiples of 8).
   Vector j of thread t is v = t + 128 j:
     K-major (!TR): row-in-group v & 7, reduction group (v >> 3) & 7, row
       group v >> 6; 16 bytes of 8 reduction indices of one row, stored as
       row (v & 7) of core matrix (row group, reduction group);
     MN-major (TR): reduction index l from v & 15 and (v >> 5), row group
       from (v >> 4) & 1 and (v >> 5); 16 bytes of 8 rows at one reduction
       index, stored as row (l & 7) of core matrix (row group, l >> 3).
   Every 8-lane phase of a warp's 16-byte copies covers 128 contiguous
   bytes of shared memory (no bank conflicts). */
template <bool TR, int ROWS>
struct TcStage {
    static constexpr int N = ROWS * TBK / 8 / TNT;
    __device__ __forceinline__ static void map(int v, int &row, int &l) {
        if (!TR) {
            row = (v >> 6) * 8 + (v & 7);
            l = ((v >> 3) & 7) * 8;
        } else {
            const int hi = v >> 5;
            l = (hi % (TBK / 16)) * 16 + (v & 15);
            row = ((hi / (TBK / 16)) * 2 + ((v >> 4) & 1)) * 8;
        }
    }
    __device__ __forceinline__ static void issue(uint32_t S, const bf16 *__restrict__ X, int ld, int R, int L,
                                                 int r0, int l0) {
#pragma unroll
        for (int j = 0; j < N; ++j) {
            int row, l;
            map(threadIdx.x + TNT * j, row, l);
            const int r = r0 + row, ll = l0 + l;
            const bool valid = r < R && ll < L;
            const bf16 *src = valid ? (TR ? X + (size_t)ll * ld + r : X + (size_t)r * ld + ll) : X;
            const uint32_t off = TR ? (uint32_t)(((row >> 3) * (TBK / 8) + (l >> 3)) * 128 + (l & 7) * 16)
                                    : (uint32_t)(((row >> 3) * (TBK / 8) + (l >> 3)) * 128 + (row & 7) * 16);
            tc_cp16(S + off, src, valid);
        }
    }
};

template <int BN, bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(TNT)
gemm_tc(const bf16 *__restrict__ A, int lda, const bf16 *__restrict__ B, int ldb, int R, int Cc, int L,
        int l_slice, const float *__restrict__ bias, int act, bf16 *Cb, float *Cf, float *pre, int ldc) {
    typedef TcShape<BN> Sh;
    typedef TcStage<TA, TBM> StA;
    typedef TcStage<TB, BN> StB;
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(tc_smem);
    const uint32_t bar0 = sbase + Sh::BARS, taddr_slot = sbase + Sh::TADDR;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r0 = blockIdx.y * TBM, c0 = blockIdx.x * BN;
    const int lb = blockIdx.z * l_slice;
    const int le = min(L, lb + l_slice);
    const int nch = le > lb ? (le - lb + TBK - 1) / TBK : 0;

    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < TC_STAGES; ++s) tc_mbar_init(bar0 + 8 * s);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(taddr_slot),
                     "r"((uint32_t)BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    /* the first TC_STAGES chunks go in flight at once */
    for (int i = 0; i < nch && i < TC_STAGES; ++i) {
        const uint32_t st = sbase + i * Sh::STAGE;
        StA::issue(st, A, lda, R, le, r0, lb + i * TBK);
        StB::issue(st + TC_A_BYTES, B, ldb, Cc, le, c0, lb + i * TBK);
        tc_cp_commit();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(tc_smem + Sh::TADDR);
    const uint64_t t_end = tc_clock_ns() + TC_WAIT_NS;

    bool ok = true;
    for (int i = 0; i < nch; ++i) {
        const int s = i % TC_STAGES;
        const uint32_t bar = bar0 + 8 * s;
        /* chunk i has landed once no more than the later committed groups are pending */
        tc_cp_wait(min(nch, i + TC_STAGES) - i - 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a = sbase + s * Sh::STAGE, b = a + TC_A_BYTES;
#pragma unroll
            for (int kk = 0; kk < TBK / 16; ++kk)
                tc_mma(tmem, tc_desc(a + 256u * kk), tc_desc(b + 256u * kk), tc_idesc<BN, TA, TB>(),
                       (i | kk) ? 1u : 0u);
            tc_commit(bar);
        }
        if (i + TC_STAGES < nch) {
            /* refill the stage once its MMAs have read it */
            if (ok) ok = tc_mbar_wait(bar, (uint32_t)(i / TC_STAGES) & 1u, t_end);
            const uint32_t st = sbase + s * Sh::STAGE;
            const int l0 = lb + (i + TC_STAGES) * TBK;
            StA::issue(st, A, lda, R, le, r0, l0);
            StB::issue(st + TC_A_BYTES, B, ldb, Cc, le, c0, l0);
            tc_cp_commit();
        }
    }
    if (nch > 0 && ok) {
        const int i = nch - 1;
        ok = tc_mbar_wait(bar0 + 8 * (i % TC_STAGES), (uint32_t)(i / TC_STAGES) & 1u, t_end);
    }
    tc_fence_after();

    const int r = r0 + warp * 32 + lane;
#pragma unroll 1
    for (int j = 0; j < BN / 16; ++j) {
        const int c = c0 + j * 16;
        float v[16];
        if (nch > 0) {
            tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * 16), v);
        } else {
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = 0.0f;
        }
        if (!ok) {
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = __int_as_float(0x7fc00000);
        }
        if (r >= R || c >= Cc) continue;
        const size_t o = (size_t)r * ldc + c;
        if (EPI == EPI_FWD) {
            if (bias) {
#pragma unroll
                for (int q = 0; q < 16; ++q) v[q] += bias[c + q];
            }
            if (pre) {
                float4 *p4 = reinterpret_cast<float4 *>(pre + o);
#pragma unroll
                for (int q = 0; q < 4; ++q) p4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
            uint32_t h[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                float x0 = act ? gelu(v[2 * q]) : v[2 * q], x1 = act ? gelu(v[2 * q + 1]) : v[2 * q + 1];
                __nv_bfloat162 t2 = __floats2bfloat162_rn(x0, x1);
                h[q] = *reinterpret_cast<uint32_t *>(&t2);
            }
            uint4 *c4 = reinterpret_cast<uint4 *>(Cb + o);
            c4[0] = make_uint4(h[0], h[1], h[2], h[3]);
            c4[1] = make_uint4(h[4], h[5], h[6], h[7]);
        } else if (EPI == EPI_BF16) {
            uint32_t h[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                __nv_bfloat162 t2 = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
                h[q] = *reinterpret_cast<uint32_t *>(&t2);
            }
            uint4 *c4 = reinterpret_cast<uint4 *>(Cb + o);
            c4[0] = make_uint4(h[0], h[1], h[2], h[3]);
            c4[1] = make_uint4(h[4], h[5], h[6], h[7]);
        } else {
            float4 *p4 = reinterpret_cast<float4 *>(Cf + (size_t)blockIdx.z * R * ldc + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) p4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN)
                     : "memory");
}
