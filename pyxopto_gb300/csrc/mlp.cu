/*
 * mlp.cu - training and inference kernels of the radial-reflectance MLP
 * surrogate: BF16 tensor-core GEMMs with FP32 accumulation and fused
 * epilogues (bias + GELU forward; input and weight gradients), the GELU
 * backward with a deterministic bias-gradient reduction, the MSE gradient
 * and AdamW.
 *
 * GEMM: C[R, Cc] = sum_l A(r, l) B(c, l) with a fused epilogue.  Two
 * implementations of the same contract:
 *   - gemm_tc (mlp_tc.cuh, the default): tcgen05.mma on 128x64 tiles with
 *     the FP32 accumulator in tensor memory;
 *   - gemm_bf16 (below, selectable with mcgb_mlp_gemm_path(1)): 64x64 tiles,
 *     4 warps of 32x32, k-steps of 16 through mma.sync m16n8k16.
 * The forward epilogue also stores the FP32 pre-activation when asked; the
 * last layer's FP32 pre-activation is the network output.
 * Operands are staged in shared memory with the reduction index contiguous;
 * transposed operands (activations in the weight gradient) are transposed
 * while staging.  The weight gradient splits the batch rows into fixed
 * slices and adds the slice results in a fixed order (deterministic).
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cstdarg>
#include <string>
#include "../../include/xopto_gb300.h"
#include "errors.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int BM = 64, BN = 64, BK = 16, PAD = 8, NT = 128;

enum { EPI_FWD = 0, EPI_BF16 = 1, EPI_F32 = 2 };

__device__ __forceinline__ float gelu(float x) {
    const float c = 0.7978845608028654f;   /* sqrt(2/pi) */
    float t = tanhf(c * (x + 0.044715f * x * x * x));
    return 0.5f * x * (1.0f + t);
}

__device__ __forceinline__ float gelu_grad(float x) {
    const float c = 0.7978845608028654f;
    float u = c * (x + 0.044715f * x * x * x);
    float t = tanhf(u);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * c * (1.0f + 3.0f * 0.044715f * x * x);
}

#include "mlp_tc.cuh"

/* 0 = tcgen05 (gemm_tc), 1 = mma.sync (gemm_bf16) */
int g_gemm_path = 0;

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

/* Stage a 64 x 16 tile of op(X) (rows r0.., reduction l0..) into S[row][l].
   X(r, l) = TR ? X[l*ld + r] : X[r*ld + l].  Rows >= R are zero. */
template <bool TR>
__device__ __forceinline__ void stage(bf16 (*S)[BK + PAD], const bf16 *X, int ld, int R, int L,
                                      int r0, int l0) {
    const int t = threadIdx.x;
    if (!TR) {
        int row = t >> 1, col = (t & 1) * 8;
        int r = r0 + row;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r < R && l0 + col + 8 <= L) v = *reinterpret_cast<const uint4 *>(X + (size_t)r * ld + l0 + col);
        *reinterpret_cast<uint4 *>(&S[row][col]) = v;
    } else {
        int l = t >> 3, rc = (t & 7) * 8;
        int r = r0 + rc;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r + 8 <= R && l0 + l < L) v = *reinterpret_cast<const uint4 *>(X + (size_t)(l0 + l) * ld + r);
        const bf16 *e = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
        for (int i = 0; i < 8; ++i) S[rc + i][l] = e[i];
    }
}

/* C = op(A) op(B)^T over the reduction range of blockIdx.z's slice. */
template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(NT)
gemm_bf16(const bf16 *__restrict__ A, int lda, const bf16 *__restrict__ B, int ldb, int R, int Cc,
          int L, int l_slice, const float *__restrict__ bias, int act, bf16 *Cb, float *Cf,
          float *pre, int ldc) {
    __shared__ __align__(16) bf16 As[BM][BK + PAD];
    __shared__ __align__(16) bf16 Bs[BN][BK + PAD];
    const int r0 = blockIdx.y * BM, c0 = blockIdx.x * BN;
    const int lb = blockIdx.z * l_slice;
    const int le = min(L, lb + l_slice);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, tig = lane & 3;
    const int wr = (warp >> 1) * 32, wc = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0f;

    for (int l0 = lb; l0 < le; l0 += BK) {
        stage<TA>(As, A, lda, R, le, r0, l0);
        stage<TB>(Bs, B, ldb, Cc, le, c0, l0);
        __syncthreads();
        uint32_t a[2][4], b[4][2];
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
            int rb = wr + mi * 16;
            a[mi][0] = *reinterpret_cast<const uint32_t *>(&As[rb + g][tig * 2]);
            a[mi][1] = *reinterpret_cast<const uint32_t *>(&As[rb + g + 8][tig * 2]);
            a[mi][2] = *reinterpret_cast<const uint32_t *>(&As[rb + g][tig * 2 + 8]);
            a[mi][3] = *reinterpret_cast<const uint32_t *>(&As[rb + g + 8][tig * 2 + 8]);
        }
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
            int cb = wc + ni * 8;
            b[ni][0] = *reinterpret_cast<const uint32_t *>(&Bs[cb + g][tig * 2]);
            b[ni][1] = *reinterpret_cast<const uint32_t *>(&Bs[cb + g][tig * 2 + 8]);
        }
#pragma unroll
        for (int mi = 0; mi < 2; ++mi)
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) mma_bf16(acc[mi][ni], a[mi], b[ni]);
        __syncthreads();
    }

#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int r = r0 + wr + mi * 16 + g + (q >> 1) * 8;
                int c = c0 + wc + ni * 8 + tig * 2 + (q & 1);
                if (r >= R || c >= Cc) continue;
                float v = acc[mi][ni][q];
                size_t o = (size_t)r * ldc + c;
                if (EPI == EPI_FWD) {
                    v += bias ? bias[c] : 0.0f;
                    if (pre) pre[o] = v;
                    Cb[o] = __float2bfloat16_rn(act ? gelu(v) : v);
                } else if (EPI == EPI_BF16) {
                    Cb[o] = __float2bfloat16_rn(v);
                } else {
                    Cf[(size_t)blockIdx.z * R * ldc + o] = v;
                }
            }
}

/* out[i] = sum over z of part[z*n + i] in a fixed order: warp w of a block
   adds slices w, w + 8, w + 16, ... of 32 consecutive entries, then the
   eight warp sums are added in warp order.  One block per 32 entries. */
constexpr int SUM_THREADS = 256;

__global__ void __launch_bounds__(SUM_THREADS)
sum_slices(const float *__restrict__ part, float *out, int slices, size_t n) {
    __shared__ float red[SUM_THREADS / 32][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const size_t i = (size_t)blockIdx.x * 32 + lane;
    float s = 0.0f;
    if (i < n)
        for (int z = w; z < slices; z += SUM_THREADS / 32) s += part[(size_t)z * n + i];
    red[w][lane] = s;
    __syncthreads();
    if (w == 0 && i < n) {
        float t = 0.0f;
#pragma unroll
        for (int k = 0; k < SUM_THREADS / 32; ++k) t += red[k][lane];
        out[i] = t;
    }
}

void launch_sum_slices(const float *part, float *out, int slices, size_t n, cudaStream_t st) {
    sum_slices<<<(unsigned)((n + 31) / 32), SUM_THREADS, 0, st>>>(part, out, slices, n);
}

/* Rows per block of the activation backward: one column partial sum per
   chunk of this many rows (the bias gradient adds them in chunk order). */
constexpr int ACT_ROWS = 64;

/* dPre = dY * act'(pre); column partial sums of dPre over row chunks of ACT_ROWS. */
__global__ void act_bwd_kernel(const bf16 *__restrict__ dy, const float *__restrict__ pre, bf16 *dpre,
                               float *part, int M, int N, int act) {
    const int c = blockIdx.x * 32 + (threadIdx.x & 31);
    const int rbeg = blockIdx.y * ACT_ROWS;
    const int rend = min(M, rbeg + ACT_ROWS);
    __shared__ float red[8][33];
    float s = 0.0f;
    if (c < N) {
        for (int r = rbeg + (threadIdx.x >> 5); r < rend; r += 8) {
            size_t o = (size_t)r * N + c;
            float v = __bfloat162float(dy[o]);
            if (act) v *= gelu_grad(pre[o]);
            dpre[o] = __float2bfloat16_rn(v);
            s += v;
        }
    }
    red[threadIdx.x >> 5][threadIdx.x & 31] = s;
    __syncthreads();
    if (threadIdx.x < 32 && c < N) {
        float t = 0.0f;
        for (int i = 0; i < 8; ++i) t += red[i][threadIdx.x];
        part[(size_t)blockIdx.y * N + c] = t;
    }
}

/* Loss gradient of the network output Y [M, N] (FP32, the last layer's
   pre-activation) against the target T [M, N], over the first nv columns,
   with optional column weights W [N]:
     mode 0 (squared error):  d = Y - T, loss W d^2, gradient 2 W d;
     mode 1 (relative error of exp(scale Y)):  ratio = T exp(-scale Y),
       loss W (ratio - 1)^2, gradient -2 scale W (min(ratio, clip) - 1) --
       the derivative of (T - R)^2 / R^2 with R = exp(scale Y) and the
       denominator held at the current prediction, so the fit converges to
       the mean of T (unbiased in linear units), not to the mean of log T.
   Loss and gradient are divided by M nv; the loss is reduced per block of
   256 rows (fixed order).  Gradients are stored as bf16. */
constexpr int LOSS_THREADS = 1024;

__global__ void __launch_bounds__(LOSS_THREADS)
loss_grad_kernel(const float *__restrict__ y, const float *__restrict__ tgt, const float *__restrict__ wcol,
                 bf16 *dy, float *loss, int M, int N, int nv, int mode, float scale, float clip) {
    __shared__ float red[LOSS_THREADS];
    const float inv = 1.0f / ((float)M * (float)nv);
    float s = 0.0f;
    size_t base = (size_t)blockIdx.x * 256;
    for (int i = threadIdx.x; i < 256 * N; i += blockDim.x) {
        size_t r = base + i / N;
        int c = i % N;
        if (r >= (size_t)M) continue;
        size_t o = r * N + c;
        float g = 0.0f;
        if (c < nv) {
            float w = wcol ? wcol[c] : 1.0f;
            if (mode == 0) {
                float d = y[o] - tgt[o];
                s += w * d * d * inv;
                g = 2.0f * w * d * inv;
            } else {
                float ratio = tgt[o] * expf(-scale * y[o]);
                float d = ratio - 1.0f;
                s += w * d * d * inv;
                g = -2.0f * scale * w * (fminf(ratio, clip) - 1.0f) * inv;
            }
        }
        dy[o] = __float2bfloat16_rn(g);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = LOSS_THREADS / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss[blockIdx.x] = red[0];
}

/* One AdamW element: FP32 master weight, bf16 copy and (when wt) the
   transposed bf16 copy of a rows x cols tensor. */
__device__ __forceinline__ void adamw_element(size_t i, float *w, bf16 *wb, bf16 *wt, const float *gr, float *m,
                                              float *v, int rows, int cols, float lr, float b1, float b2,
                                              float eps, float wd, float c1, float c2) {
    float g = gr[i];
    float mi = b1 * m[i] + (1.0f - b1) * g;
    float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float upd = (mi / c1) / (sqrtf(vi / c2) + eps);
    float wi = w[i] - lr * (upd + wd * w[i]);
    w[i] = wi;
    bf16 h = __float2bfloat16_rn(wi);
    wb[i] = h;
    if (wt) {
        size_t r = i / cols, c = i % cols;
        wt[c * rows + r] = h;
    }
}

__global__ void adamw_kernel(float *w, bf16 *wb, bf16 *wt, const float *__restrict__ gr, float *m, float *v,
                             int rows, int cols, float lr, float b1, float b2, float eps, float wd,
                             float c1, float c2) {
    size_t n = (size_t)rows * cols;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        adamw_element(i, w, wb, wt, gr, m, v, rows, cols, lr, b1, b2, eps, wd, c1, c2);
}

/* Several tensors in one launch: element i of the concatenation belongs to
   the tensor k with start[k] <= i < start[k + 1]. */
struct AdamwMulti {
    McgbAdamwTensor t[MCGB_ADAMW_MAX_TENSORS];
    uint64_t start[MCGB_ADAMW_MAX_TENSORS + 1];
    int count;
    float lr, b1, b2, eps, c1, c2;
};

__global__ void adamw_multi_kernel(const __grid_constant__ AdamwMulti p) {
    const uint64_t total = p.start[p.count];
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        int k = 0;
        while (k + 1 < p.count && i >= p.start[k + 1]) ++k;
        const McgbAdamwTensor &T = p.t[k];
        adamw_element((size_t)(i - p.start[k]), T.w, (bf16 *)T.w_bf16, (bf16 *)T.wt_bf16, T.grad, T.m, T.v, T.rows,
                      T.cols, p.lr, p.b1, p.b2, p.eps, T.weight_decay, p.c1, p.c2);
    }
}

/* dW[:, j] = dW[:, j + shift] = dW[:, j] + dW[:, j + shift] for j < count:
   the gradient of a weight shared by two input columns (the high and low
   bf16 parts of one input), so that AdamW moves both copies alike. */
__global__ void tie_columns_kernel(float *dw, int rows, int cols, int count, int shift) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * count) return;
    int r = i / count, j = i % count;
    float *row = dw + (size_t)r * cols;
    float s = row[j] + row[j + shift];
    row[j] = s;
    row[j + shift] = s;
}

int fail(int code, const char *fmt, ...) {
    char buf[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return mcgb_internal::set_error(code, buf);
}

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MCGB_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return MCGB_OK;
}

int shape_ok(int m, int n, int k) {
    if (m <= 0 || n <= 0 || k <= 0) return fail(MCGB_E_INVALID, "MLP shapes must be positive");
    if (m % 8 || n % 16 || k % 16) return fail(MCGB_E_INVALID, "MLP shapes need M%%8, N%%16, K%%16 == 0");
    return MCGB_OK;
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            n = v;
        else
            n = 152;
    }
    return n;
}

/* Reduction slices of the weight gradient for a GEMM path: enough that the
   grid of output tiles times slices covers every SM twice, each slice at
   least one k-step of rows, at most 64 slices. */
int weight_slices(int m, int n, int k, int path) {
    const int tm = path == 0 ? TBM : BM, tn = 64, tk = path == 0 ? TBK : BK;
    int tiles = ((n + tm - 1) / tm) * ((k + tn - 1) / tn);
    int s = (2 * sm_count() + tiles - 1) / tiles;
    int most = m / tk;
    if (s > most) s = most;
    if (s > 64) s = 64;
    return s < 1 ? 1 : s;
}

template <int TBN_, bool TA, bool TB, int EPI>
int launch_tc(const bf16 *A, int lda, const bf16 *B, int ldb, int R, int Cc, int L, int l_slice, int slices,
              const float *bias, int act, bf16 *Cb, float *Cf, float *pre, int ldc, cudaStream_t st,
              const char *what) {
    typedef TcShape<TBN_> Sh;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(gemm_tc<TBN_, TA, TB, EPI>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Sh::SMEM);
        if (e != cudaSuccess) return fail(MCGB_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
        attr = true;
    }
    dim3 grid((Cc + TBN_ - 1) / TBN_, (R + TBM - 1) / TBM, slices);
    gemm_tc<TBN_, TA, TB, EPI><<<grid, TNT, Sh::SMEM, st>>>(A, lda, B, ldb, R, Cc, L, l_slice, bias, act, Cb, Cf,
                                                            pre, ldc);
    return check_launch(what);
}

/* One GEMM launch on the selected path; `slices` reduction slices of
   l_slice each along blockIdx.z.  The tcgen05 path takes 128 x 64 tiles,
   or 128 x 32 when 64-wide tiles would leave SMs without a CTA. */
template <bool TA, bool TB, int EPI>
int launch_gemm(const bf16 *A, int lda, const bf16 *B, int ldb, int R, int Cc, int L, int l_slice, int slices,
                const float *bias, int act, bf16 *Cb, float *Cf, float *pre, int ldc, cudaStream_t st,
                const char *what) {
    if (g_gemm_path == 0) {
        const long tiles64 = (long)((Cc + 63) / 64) * ((R + TBM - 1) / TBM) * slices;
        if (tiles64 >= sm_count())
            return launch_tc<64, TA, TB, EPI>(A, lda, B, ldb, R, Cc, L, l_slice, slices, bias, act, Cb, Cf, pre,
                                              ldc, st, what);
        return launch_tc<32, TA, TB, EPI>(A, lda, B, ldb, R, Cc, L, l_slice, slices, bias, act, Cb, Cf, pre, ldc,
                                          st, what);
    }
    dim3 grid((Cc + BN - 1) / BN, (R + BM - 1) / BM, slices);
    gemm_bf16<TA, TB, EPI><<<grid, NT, 0, st>>>(A, lda, B, ldb, R, Cc, L, l_slice, bias, act, Cb, Cf, pre, ldc);
    return check_launch(what);
}

}  // namespace

extern "C" {

int mcgb_mlp_linear_fwd(const uint16_t *x, const uint16_t *w, const float *b, uint16_t *y, float *pre,
                        int m, int n, int k, int act, void *stream) {
    int r = shape_ok(m, n, k);
    if (r) return r;
    if (!x || !w || !y) return fail(MCGB_E_INVALID, "NULL operand");
    return launch_gemm<false, false, EPI_FWD>((const bf16 *)x, k, (const bf16 *)w, k, m, n, k, k, 1, b, act,
                                              (bf16 *)y, nullptr, pre, n, (cudaStream_t)stream, "mlp forward");
}

uint64_t mcgb_mlp_bwd_weight_scratch(int m, int n, int k) {
    if (m <= 0 || n <= 0 || k <= 0) return 0;
    int s0 = weight_slices(m, n, k, 0), s1 = weight_slices(m, n, k, 1);
    return (uint64_t)(s0 > s1 ? s0 : s1) * (uint64_t)n * (uint64_t)k;
}

int mcgb_mlp_gemm_path(int path) {
    int prev = g_gemm_path;
    if (path == -1) return prev;
    if (path != 0 && path != 1) {
        fail(MCGB_E_INVALID, "GEMM path must be 0 (tcgen05) or 1 (mma.sync)");
        return -1;
    }
    g_gemm_path = path;
    return prev;
}

int mcgb_mlp_linear_bwd_input(const uint16_t *dpre, const uint16_t *wt, uint16_t *dx, int m, int n, int k,
                              void *stream) {
    int r = shape_ok(m, n, k);
    if (r) return r;
    if (!dpre || !wt || !dx) return fail(MCGB_E_INVALID, "NULL operand");
    /* dX[m,k] = sum_n dPre[m,n] Wt[k,n] */
    return launch_gemm<false, false, EPI_BF16>((const bf16 *)dpre, n, (const bf16 *)wt, n, m, k, n, n, 1, nullptr,
                                               0, (bf16 *)dx, nullptr, nullptr, k, (cudaStream_t)stream,
                                               "mlp backward input");
}

int mcgb_mlp_linear_bwd_weight(const uint16_t *dpre, const uint16_t *x, float *dw, float *scratch,
                               int m, int n, int k, void *stream) {
    int r = shape_ok(m, n, k);
    if (r) return r;
    if (!dpre || !x || !dw || !scratch) return fail(MCGB_E_INVALID, "NULL operand");
    /* dW[n,k] = sum_m dPre[m,n] X[m,k]: R = n, Cc = k, reduction over m */
    const int path = g_gemm_path, tk = path == 0 ? TBK : BK;
    int slices = weight_slices(m, n, k, path);
    int per = ((m + slices - 1) / slices + tk - 1) / tk * tk;
    slices = (m + per - 1) / per;
    r = launch_gemm<true, true, EPI_F32>((const bf16 *)dpre, n, (const bf16 *)x, k, n, k, m, per, slices, nullptr,
                                         0, nullptr, scratch, nullptr, k, (cudaStream_t)stream,
                                         "mlp backward weight");
    if (r) return r;
    launch_sum_slices(scratch, dw, slices, (size_t)n * k, (cudaStream_t)stream);
    return check_launch("mlp weight slice sum");
}

uint64_t mcgb_mlp_act_bwd_scratch(int m, int n) {
    if (m <= 0 || n <= 0) return 0;
    return (uint64_t)((m + ACT_ROWS - 1) / ACT_ROWS) * (uint64_t)n;
}

int mcgb_mlp_act_bwd(const uint16_t *dy, const float *pre, uint16_t *dpre, float *db, float *scratch,
                      int m, int n, int act, void *stream) {
    if (m <= 0 || n <= 0 || !dy || !dpre || !db || !scratch || (act && !pre))
        return fail(MCGB_E_INVALID, "bad act_bwd arguments");
    dim3 grid((n + 31) / 32, (m + ACT_ROWS - 1) / ACT_ROWS);
    act_bwd_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>((const bf16 *)dy, pre, (bf16 *)dpre, scratch,
                                                          m, n, act);
    int r = check_launch("mlp activation backward");
    if (r) return r;
    int chunks = (m + ACT_ROWS - 1) / ACT_ROWS;
    launch_sum_slices(scratch, db, chunks, (size_t)n, (cudaStream_t)stream);
    return check_launch("mlp bias gradient");
}

int mcgb_mlp_loss_grad(const float *y, const float *t, const float *w, uint16_t *dy, float *loss, int m,
                       int n, int nv, int mode, float scale, void *stream) {
    if (m <= 0 || n <= 0 || nv <= 0 || nv > n || !y || !t || !dy || !loss || mode < 0 || mode > 1)
        return fail(MCGB_E_INVALID, "bad loss_grad arguments");
    loss_grad_kernel<<<(m + 255) / 256, LOSS_THREADS, 0, (cudaStream_t)stream>>>(y, t, w, (bf16 *)dy, loss, m, n,
                                                                                nv, mode, scale, 4.0f);
    return check_launch("mlp loss gradient");
}

int mcgb_mlp_tie_columns(float *dw, int rows, int cols, int count, int shift, void *stream) {
    if (!dw || rows <= 0 || cols <= 0 || count <= 0 || shift < count || count + shift > cols)
        return fail(MCGB_E_INVALID, "bad tie_columns arguments");
    int n = rows * count;
    tie_columns_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(dw, rows, cols, count, shift);
    return check_launch("mlp tie columns");
}

int mcgb_mlp_adamw(float *w, uint16_t *wb, uint16_t *wt, const float *g, float *m, float *v, int rows,
                   int cols, float lr, float b1, float b2, float eps, float wd, int step, void *stream) {
    if (!w || !wb || !g || !m || !v || rows <= 0 || cols <= 0 || step < 1)
        return fail(MCGB_E_INVALID, "bad adamw arguments");
    float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    size_t n = (size_t)rows * cols;
    unsigned blocks = (unsigned)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    adamw_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(w, (bf16 *)wb, (bf16 *)wt, g, m, v, rows, cols, lr,
                                                           b1, b2, eps, wd, c1, c2);
    return check_launch("mlp adamw");
}

int mcgb_mlp_adamw_multi(const McgbAdamwTensor *tensors, int count, float lr, float b1, float b2, float eps,
                         int step, void *stream) {
    if (!tensors || count < 1 || count > MCGB_ADAMW_MAX_TENSORS || step < 1)
        return fail(MCGB_E_INVALID, "bad adamw_multi arguments");
    AdamwMulti p;
    memset(&p, 0, sizeof(p));
    p.count = count;
    p.start[0] = 0;
    for (int k = 0; k < count; ++k) {
        const McgbAdamwTensor &t = tensors[k];
        if (!t.w || !t.w_bf16 || !t.grad || !t.m || !t.v || t.rows <= 0 || t.cols <= 0)
            return fail(MCGB_E_INVALID, "bad adamw_multi tensor %d", k);
        p.t[k] = t;
        p.start[k + 1] = p.start[k] + (uint64_t)t.rows * (uint64_t)t.cols;
    }
    p.lr = lr;
    p.b1 = b1;
    p.b2 = b2;
    p.eps = eps;
    p.c1 = 1.0f - powf(b1, (float)step);
    p.c2 = 1.0f - powf(b2, (float)step);
    uint64_t blocks = (p.start[count] + 255) / 256;
    uint64_t most = 4ull * (uint64_t)sm_count();
    if (blocks > most) blocks = most;
    adamw_multi_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(p);
    return check_launch("mlp adamw multi");
}

}  // extern "C"
