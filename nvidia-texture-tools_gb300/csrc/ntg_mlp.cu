// The learned endpoint proposal's network on the 5th-generation tensor cores: an MLP
// 48 -> 256 -> 256 -> 8 (GELU, tanh form; BF16 weights and activations, FP32 accumulation) trained
// with Adam.
// Inputs are a block's 16 texels x RGB; outputs 0-5 are the two endpoints of the block's cluster
// fit, output 6 the fit's log-error (used to decide when the pruned search falls back to the full
// one), output 7 is unused. No counterpart in the reference.
//
// Every matrix product is one kernel, k_gemm: D[M x N] = A[M x K] * B[N x K]^T with both operands
// K-major BF16, staged by the CTA's threads into shared memory in the canonical no-swizzle layout
// (8-row x 16-byte core matrices), multiplied by tcgen05.mma (kind::f16, M = 128) issued by one
// thread into a TMEM accumulator, double-buffered with an mbarrier per stage that the MMA's
// tcgen05.commit arrives on. The epilogue reads the accumulator back with tcgen05.ld (thread t owns
// row t) and applies bias + GELU, GELU', or split-K atomics. Every wait is bounded (a poll count the
// host sets per network, ntg_mlp_set_wait_limit): on timeout the kernel records an error, waits (with
// the default limit) for the tensor-core work it has already issued, frees its TMEM and returns.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "ntg.h"
#include "ntg_async.cuh"
#include "ntg_internal.h"

namespace ntg {
namespace mlp {

constexpr int IN = 48, HID = 256, OUT = 8, OUTP = 16;  // OUTP: output rows padded for the MMA's N
constexpr int BM = 128, BK = 64;                       // CTA tile rows, K chunk
constexpr uint32_t LBO = 128, SBO = 1024;              // K-direction and row-group core-matrix strides

enum Epi { EPI_F32 = 0, EPI_GELU = 1, EPI_DGELU = 2, EPI_ATOMIC = 3 };

struct GemmArgs {
    const __nv_bfloat16 *A;  // [M x K], row stride lda (elements)
    const __nv_bfloat16 *B;  // [N x K], row stride ldb
    int lda, ldb, M, N, K;
    int k_split;             // K per blockIdx.z (multiple of BK)
    int epi;
    const float *bias;       // [N] or null
    float *C;                // fp32 [M x N] (ldc), or null
    int ldc;
    __nv_bfloat16 *H;        // bf16 [M x N] (ldh), or null
    int ldh;
    __nv_bfloat16 *HT;       // bf16 [N x M] (ldht), or null
    int ldht;
    const float *Z;          // pre-activation [M x N] (ldz) for EPI_DGELU
    int ldz;
    int *status;             // set to a non-zero code when a wait gives up
    int polls;               // polls of each wait before it gives up
};

// ---- PTX wrappers (tcgen05, mbarrier) ----

// Shared-memory matrix descriptor: start address, leading (K) and stride (row-group) byte offsets,
// the fixed 0b001 field at bits 46-48, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo = SBO) {
    uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)((LBO >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N and M.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Polls of a wait by default, and of the drain after a wait gave up: the MMAs already issued
// still write the TMEM accumulator, so they must finish before it is freed.
constexpr int kWaitPolls = 1 << 22;

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// GELU in its tanh form (Hendrycks & Gimpel, "Gaussian Error Linear Units", 2016):
// gelu(z) = z / 2 (1 + tanh(sqrt(2 / pi) (z + 0.044715 z^3))), with the hardware tanh
// (tanh.approx.f32, about 2^-11 relative error, below the BF16 rounding of the activations), and its
// derivative for training. The network is defined with this activation, in training, inference and
// the oracle alike.
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float GELU_S = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float GELU_C = 0.044715f;
__device__ __forceinline__ float gelu(float z) {
    const float t = tanh_hw(GELU_S * (z + GELU_C * (z * z * z)));
    return 0.5f * z * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float z) {
    const float z2 = z * z;
    const float t = tanh_hw(GELU_S * (z + GELU_C * (z2 * z)));
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * GELU_S * (1.0f + 3.0f * GELU_C * z2);
}

// Copies rows [r0, r0 + rows) x K-chunk [k0, k0 + BK) of a K-major matrix into the canonical
// layout at `dst` (rows beyond `nrows` or columns beyond K read as zero).
__device__ __forceinline__ void stage_tile(uint8_t *dst, const __nv_bfloat16 *src, int ld, int r0, int nrows, int rows,
                                           int k0, int K) {
    const int pieces = rows * (BK / 8);  // 16-byte pieces
    for (int p = threadIdx.x; p < pieces; p += blockDim.x) {
        const int rr = p & 7, kc = (p >> 3) & 7, rg = p >> 6;  // row in core matrix, K chunk, row group
        const int r = rg * 8 + rr, k = k0 + kc * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (r0 + r < nrows && k < K) v = *reinterpret_cast<const uint4 *>(src + (size_t)(r0 + r) * ld + k);
        *reinterpret_cast<uint4 *>(dst + rg * SBO + kc * LBO + rr * 16) = v;
    }
}

template <int BN>
__global__ void __launch_bounds__(128) k_gemm(GemmArgs g) {
    constexpr int TMEM_COLS = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
    constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
    constexpr uint32_t IDESC = idesc_bf16(BM, BN);
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bars[3];
    __shared__ uint32_t tmem_base;
    uint8_t *a_st[2] = {smem, smem + A_BYTES + B_BYTES};
    uint8_t *b_st[2] = {smem + A_BYTES, smem + 2 * A_BYTES + B_BYTES};
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * g.k_split, kend = min(g.K, kbeg + g.k_split);
    const int chunks = (kend - kbeg + BK - 1) / BK;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == 0) tmem_alloc(&tmem_base, TMEM_COLS);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_init(&bars[2], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    bool ok = true;
    int committed = -1;  // last chunk whose MMAs were issued and committed

    for (int c = 0; c < chunks && ok; c++) {
        const int s = c & 1;
        if (c >= 2) {  // the MMAs of chunk c-2 read this stage; the CTA agrees on the outcome
            ok = __syncthreads_and(mbar_wait(&bars[s], ((c - 2) >> 1) & 1, g.polls)) != 0;
            if (!ok) break;
        }
        const int k0 = kbeg + c * BK;
        stage_tile(a_st[s], g.A, g.lda, m0, g.M, BM, k0, kend);
        stage_tile(b_st[s], g.B, g.ldb, n0, g.N, BN, k0, kend);
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_u32(a_st[s]), b0 = smem_u32(b_st[s]);
#pragma unroll
            for (int j = 0; j < BK / 16; j++)
                mma_bf16(tmem, smem_desc(a0 + j * 2 * LBO), smem_desc(b0 + j * 2 * LBO), IDESC, (c > 0 || j > 0) ? 1u : 0u);
            mma_commit(&bars[s]);
        }
        committed = c;
    }
    // all MMAs done: the last chunk's commit completes after every earlier one
    if (ok && chunks > 0) ok = __syncthreads_and(mbar_wait(&bars[(chunks - 1) & 1], ((chunks - 1) >> 1) & 1, g.polls)) != 0;
    if (!ok) {
        if (g.status && threadIdx.x == 0) atomicExch(g.status, 1);
        // drain: the last commit's barrier completes once every MMA issued so far has finished
        if (committed >= 0) __syncthreads_and(mbar_wait(&bars[committed & 1], (committed >> 1) & 1, kWaitPolls));
    }
    tc_fence_after();

    if (ok) {
        const int row = warp * 32 + lane, m = m0 + row;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            if (chunks > 0) tmem_ld16(lane_addr + c0, v);
            else
#pragma unroll
                for (int i = 0; i < 16; i++) v[i] = 0.0f;
            if (m >= g.M) continue;
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const int n = n0 + c0 + i;
                if (n >= g.N) break;
                float x = v[i];
                if (g.epi == EPI_ATOMIC) {
                    atomicAdd(g.C + (size_t)m * g.ldc + n, x);
                    continue;
                }
                if (g.bias) x += g.bias[n];
                float y = x;
                if (g.epi == EPI_GELU) {
                    if (g.C) g.C[(size_t)m * g.ldc + n] = x;
                    y = gelu(x);
                } else if (g.epi == EPI_DGELU) {
                    y = x * gelu_grad(g.Z[(size_t)m * g.ldz + n]);
                    if (g.C) g.C[(size_t)m * g.ldc + n] = y;
                } else if (g.C) {
                    g.C[(size_t)m * g.ldc + n] = x;
                }
                const __nv_bfloat16 hb = __float2bfloat16_rn(y);
                if (g.H) g.H[(size_t)m * g.ldh + n] = hb;
                if (g.HT) g.HT[(size_t)n * g.ldht + m] = hb;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
}

size_t gemm_smem(int bn) { return 2 * (size_t)(BM * BK * 2 + bn * BK * 2) + 1024; }

template <int BN>
int launch_gemm_t(const GemmArgs &g, int splits, cudaStream_t s) {
    static std::atomic<unsigned long long> configured{0};
    const size_t sm = gemm_smem(BN);
    if (first_use_on_device(configured)) cudaFuncSetAttribute(k_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    dim3 grid((g.M + BM - 1) / BM, (g.N + BN - 1) / BN, splits);
    k_gemm<BN><<<grid, 128, sm, s>>>(g);
    return launch_status();
}

// Picks the N tile (16, 48, 64 or 256 columns) for the product's N.
int launch_gemm(GemmArgs g, int splits, cudaStream_t s) {
    if (g.K % 8 || g.lda % 8 || g.ldb % 8) return NTG_ERROR_INVALID_INPUT;
    splits = splits < 1 ? 1 : splits;
    g.k_split = ((g.K + splits - 1) / splits + BK - 1) / BK * BK;
    splits = (g.K + g.k_split - 1) / g.k_split;
    if (g.N <= 16) return launch_gemm_t<16>(g, splits, s);
    if (g.N <= 48) return launch_gemm_t<48>(g, splits, s);
    if (g.N <= 64) return launch_gemm_t<64>(g, splits, s);
    return launch_gemm_t<256>(g, splits, s);
}

// ---- elementwise kernels ----

// fp32 [rows x cols] -> bf16 row-major and (optionally) bf16 transposed [cols x rows]
__global__ void k_to_bf16(const float *__restrict__ x, int rows, int cols, __nv_bfloat16 *__restrict__ y,
                          __nv_bfloat16 *__restrict__ yt) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)rows * cols;
         i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i % cols);
        const __nv_bfloat16 b = __float2bfloat16_rn(x[i]);
        if (y) y[i] = b;
        if (yt) yt[(size_t)c * rows + r] = b;
    }
}

// Loss and output gradient: dY = 2 w (Y - T) / (B * OUT) for the weighted outputs, loss += w (Y - T)^2 / (B * OUT).
__global__ void k_loss(const float *__restrict__ y, const float *__restrict__ t, int batch, const float *__restrict__ wout,
                       float *__restrict__ dy, __nv_bfloat16 *__restrict__ dyb, __nv_bfloat16 *__restrict__ dyt,
                       float *__restrict__ loss) {
    float acc = 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < batch * OUTP; i += gridDim.x * blockDim.x) {
        const int r = i / OUTP, c = i % OUTP;
        float g = 0.0f;
        if (c < OUT) {
            const float d = y[(size_t)r * OUTP + c] - t[(size_t)r * OUT + c];
            const float w = wout[c] / (float)(batch * OUT);
            acc += w * d * d;
            g = 2.0f * w * d;
        }
        dy[i] = g;
        const __nv_bfloat16 b = __float2bfloat16_rn(g);
        dyb[i] = b;
        dyt[(size_t)c * batch + r] = b;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// Column sums of an fp32 [rows x cols] matrix into out[cols] (bias gradients).
__global__ void k_colsum(const float *__restrict__ x, int rows, int cols, float *__restrict__ out) {
    const int c = blockIdx.x;
    float acc = 0.0f;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) acc += x[(size_t)r * cols + c];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ float part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += part[w];
        out[c] = s;
    }
}

// Parameter layout (flat fp32): W1 [HID x IN], b1 [HID], W2 [HID x HID], b2 [HID], W3 [OUT x HID], b3 [OUT].
constexpr size_t OFF_W1 = 0, OFF_B1 = OFF_W1 + (size_t)HID * IN, OFF_W2 = OFF_B1 + HID, OFF_B2 = OFF_W2 + (size_t)HID * HID,
                 OFF_W3 = OFF_B2 + HID, OFF_B3 = OFF_W3 + (size_t)OUT * HID, NPARAM = OFF_B3 + OUT;

// Gathers the gradient pieces into the flat layout (dW3 arrives transposed, [HID x OUTP]).
__global__ void k_gather_grads(const float *__restrict__ dw1, const float *__restrict__ db1, const float *__restrict__ dw2,
                               const float *__restrict__ db2, const float *__restrict__ dw3t, const float *__restrict__ db3,
                               float *__restrict__ g) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (int)NPARAM; i += gridDim.x * blockDim.x) {
        float v;
        if (i < (int)OFF_B1) v = dw1[i];
        else if (i < (int)OFF_W2) v = db1[i - OFF_B1];
        else if (i < (int)OFF_B2) v = dw2[i - OFF_W2];
        else if (i < (int)OFF_W3) v = db2[i - OFF_B2];
        else if (i < (int)OFF_B3) {
            const int k = i - (int)OFF_W3, o = k / HID, j = k % HID;
            v = dw3t[(size_t)j * OUTP + o];
        } else v = db3[i - OFF_B3];
        g[i] = v;
    }
}

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// BF16 operand copies of the weights: W1 [HID x IN], W2 [HID x HID], W2^T, W3 padded [OUTP x HID],
// W3^T [HID x OUTP]; biases as fp32 (b3 padded to OUTP).
__global__ void k_refresh(const float *__restrict__ p, __nv_bfloat16 *__restrict__ w1, __nv_bfloat16 *__restrict__ w2,
                          __nv_bfloat16 *__restrict__ w2t, __nv_bfloat16 *__restrict__ w3, __nv_bfloat16 *__restrict__ w3t,
                          float *__restrict__ b3p) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < HID * HID; i += gridDim.x * blockDim.x) {
        const int r = i / HID, c = i % HID;
        const __nv_bfloat16 b = __float2bfloat16_rn(p[OFF_W2 + i]);
        w2[i] = b;
        w2t[(size_t)c * HID + r] = b;
        if (i < HID * IN) w1[i] = __float2bfloat16_rn(p[OFF_W1 + i]);
        if (i < OUTP * HID) {
            const int o = i / HID, j = i % HID;
            const __nv_bfloat16 q = o < OUT ? __float2bfloat16_rn(p[OFF_W3 + (size_t)o * HID + j]) : __float2bfloat16_rn(0.0f);
            w3[i] = q;
            w3t[(size_t)j * OUTP + o] = q;
        }
        if (i < OUTP) b3p[i] = i < OUT ? p[OFF_B3 + i] : 0.0f;
    }
}

// ---- fused inference: the whole network per 128-row tile, on one CTA per SM ----
// The weights stay in shared memory for the kernel's lifetime (canonical layout, whole K per
// operand: row group stride = K / 8 x 128 bytes); a tile's activations go X -> TMEM -> GELU -> the
// same shared-memory operand buffer -> TMEM -> ... so nothing but x and y touches global memory.
// TMEM: layer 1 in columns [0, 256), layer 2 in [256, 512), layer 3 in [0, 16).
constexpr uint32_t SBO_IN = IN / 8 * 128, SBO_HID = HID / 8 * 128;
constexpr size_t F_W1 = 0, F_W2 = F_W1 + (size_t)HID * IN * 2, F_W3 = F_W2 + (size_t)HID * HID * 2,
                 F_ACT = F_W3 + (size_t)OUTP * HID * 2, F_BIAS = F_ACT + (size_t)BM * HID * 2,
                 F_BYTES = F_BIAS + (size_t)(HID + HID + OUTP) * 4;

// Writes 8 bf16 (16 bytes) at row r, K chunk kc of a canonical operand with row-group stride sbo.
__device__ __forceinline__ void put8(uint8_t *base, uint32_t sbo, int r, int kc, uint4 v) {
    *reinterpret_cast<uint4 *>(base + (r >> 3) * sbo + kc * LBO + (r & 7) * 16) = v;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Copies a bf16 row-major [rows x K] matrix from global memory into the canonical layout.
__device__ void load_operand(uint8_t *dst, const __nv_bfloat16 *src, int rows, int K) {
    const int chunks = K / 8;
    for (int p = threadIdx.x; p < rows * chunks; p += blockDim.x) {
        const int r = p / chunks, kc = p % chunks;
        put8(dst, (uint32_t)chunks * LBO, r, kc, *reinterpret_cast<const uint4 *>(src + (size_t)r * K + kc * 8));
    }
}

// Bias + GELU of this thread's quarter (64 columns from c_begin) of its row's accumulator, into its
// row of the activation operand.
__device__ __forceinline__ void hidden_epilogue(uint32_t lane_addr, const float *bias, uint8_t *act, int row, int c_begin) {
#pragma unroll 1
    for (int c0 = c_begin; c0 < c_begin + HID / 4; c0 += 16) {
        float v[16];
        tmem_ld16(lane_addr + c0, v);
        uint32_t p[8];
#pragma unroll
        for (int i = 0; i < 8; i++) p[i] = pack_bf16(gelu(v[2 * i] + bias[c0 + 2 * i]), gelu(v[2 * i + 1] + bias[c0 + 2 * i + 1]));
        put8(act, SBO_HID, row, c0 / 8, make_uint4(p[0], p[1], p[2], p[3]));
        put8(act, SBO_HID, row, c0 / 8 + 1, make_uint4(p[4], p[5], p[6], p[7]));
    }
}

__global__ void __launch_bounds__(512, 1) k_mlp_infer(const __nv_bfloat16 *__restrict__ w1, const __nv_bfloat16 *__restrict__ w2,
                                                       const __nv_bfloat16 *__restrict__ w3, const float *__restrict__ b1,
                                                       const float *__restrict__ b2, const float *__restrict__ b3,
                                                       const float *__restrict__ x, long long rows, float *__restrict__ y,
                                                       int *status, int polls) {
    extern __shared__ __align__(16) uint8_t smem[];  // 226 KB of the 227 KB a CTA may have
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    uint8_t *sw1 = smem + F_W1, *sw2 = smem + F_W2, *sw3 = smem + F_W3, *act = smem + F_ACT;
    float *sb = reinterpret_cast<float *>(smem + F_BIAS);
    // 16 warps: thread t owns row t % 128 (TMEM lane: warp t / 32 reads lane quarter (t / 32) % 4) and
    // quarter t / 128 of its columns
    const int warp = threadIdx.x >> 5, row = threadIdx.x & 127, quarter = threadIdx.x >> 7;
    if (warp == 0) tmem_alloc(&tmem_base, 512);
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    load_operand(sw1, w1, HID, IN);
    load_operand(sw2, w2, HID, HID);
    load_operand(sw3, w3, OUTP, HID);
    for (int i = threadIdx.x; i < HID; i += blockDim.x) { sb[i] = b1[i]; sb[HID + i] = b2[i]; }
    if (threadIdx.x < OUTP) sb[2 * HID + threadIdx.x] = b3[threadIdx.x];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base, lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t a_act = smem_u32(act), a_w1 = smem_u32(sw1), a_w2 = smem_u32(sw2), a_w3 = smem_u32(sw3);
    uint32_t phase = 0;
    bool ok = true;
    const long long tiles = (rows + BM - 1) / BM;
    // X of the next tile is loaded into registers while the current tile is in the tensor cores and
    // the epilogues (quarters 0 and 1: half a row each, rows past the end are zero)
    constexpr int XC = IN / 16;  // 8-element chunks per half row
    float4 xr[2 * XC];
    auto load_x = [&](long long tile) {
        const long long r = tile * BM + row;
#pragma unroll
        for (int k = 0; k < XC; k++) {
            const int kc = quarter * XC + k;
            xr[2 * k] = xr[2 * k + 1] = make_float4(0, 0, 0, 0);
            if (quarter < 2 && tile < tiles && r < rows) {
                xr[2 * k] = *reinterpret_cast<const float4 *>(x + r * IN + kc * 8);
                xr[2 * k + 1] = *reinterpret_cast<const float4 *>(x + r * IN + kc * 8 + 4);
            }
        }
    };
    load_x(blockIdx.x);
    for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const long long r = tile * BM + row;
        if (quarter < 2) {
#pragma unroll
            for (int k = 0; k < XC; k++) {
                const float4 a = xr[2 * k], b = xr[2 * k + 1];
                put8(act, SBO_IN, row, quarter * XC + k,
                     make_uint4(pack_bf16(a.x, a.y), pack_bf16(a.z, a.w), pack_bf16(b.x, b.y), pack_bf16(b.z, b.w)));
            }
        }
#pragma unroll 1
        for (int layer = 0; layer < 3 && ok; layer++) {
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            if (threadIdx.x == 0) {
                tc_fence_after();
                if (layer == 0) {
#pragma unroll
                    for (int j = 0; j < IN / 16; j++)
                        mma_bf16(tmem, smem_desc(a_act + j * 2 * LBO, SBO_IN), smem_desc(a_w1 + j * 2 * LBO, SBO_IN),
                                 idesc_bf16(BM, HID), j > 0);
                } else if (layer == 1) {
#pragma unroll 4
                    for (int j = 0; j < HID / 16; j++)
                        mma_bf16(tmem + HID, smem_desc(a_act + j * 2 * LBO, SBO_HID), smem_desc(a_w2 + j * 2 * LBO, SBO_HID),
                                 idesc_bf16(BM, HID), j > 0);
                } else {
#pragma unroll 4
                    for (int j = 0; j < HID / 16; j++)
                        mma_bf16(tmem, smem_desc(a_act + j * 2 * LBO, SBO_HID), smem_desc(a_w3 + j * 2 * LBO, SBO_HID),
                                 idesc_bf16(BM, OUTP), j > 0);
                }
                mma_commit(&bar);
            }
            ok = __syncthreads_and(mbar_wait(&bar, phase & 1, polls)) != 0;
            // gave up: drain this layer's MMAs (they write the accumulator) before TMEM is freed
            if (!ok) __syncthreads_and(mbar_wait(&bar, phase & 1, kWaitPolls));
            phase++;
            tc_fence_after();
            if (!ok) break;
            if (layer == 0) load_x(tile + gridDim.x);  // layer 1 has read this tile's X
            if (layer < 2) {
                hidden_epilogue(lane_addr + (layer == 0 ? 0u : (uint32_t)HID), sb + layer * HID, act, row, quarter * (HID / 4));
            } else if (quarter == 0) {
                float v[16];
                tmem_ld16(lane_addr, v);
                if (r < rows) {
                    float4 *o = reinterpret_cast<float4 *>(y + r * OUTP);
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        o[q] = make_float4(v[4 * q] + sb[2 * HID + 4 * q], v[4 * q + 1] + sb[2 * HID + 4 * q + 1],
                                           v[4 * q + 2] + sb[2 * HID + 4 * q + 2], v[4 * q + 3] + sb[2 * HID + 4 * q + 3]);
                }
            }
        }
    }
    if (!ok && status && threadIdx.x == 0) atomicExch(status, 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

int grid_of(long long n) { return (int)std::min<long long>(152LL * 8, std::max<long long>(1, (n + 255) / 256)); }

}  // namespace mlp
}  // namespace ntg

using namespace ntg;
using namespace ntg::mlp;

struct ntg_mlp {
    int device = 0;
    int cap = 0;      // batch capacity of the activation buffers
    int step = 0;     // Adam steps taken
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // flat params, grads, Adam moments
    __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w2t = nullptr, *w3 = nullptr, *w3t = nullptr;
    float *b3p = nullptr, *wout = nullptr, *loss = nullptr;
    int *status = nullptr;
    int polls = kWaitPolls;  // polls of each tensor-core wait before it gives up
    // activations and gradients, batch `cap`
    __nv_bfloat16 *xb = nullptr, *xt = nullptr, *h1 = nullptr, *h1t = nullptr, *h2 = nullptr, *h2t = nullptr;
    __nv_bfloat16 *dyb = nullptr, *dyt = nullptr, *dz2b = nullptr, *dz2t = nullptr, *dz1b = nullptr, *dz1t = nullptr;
    float *z1 = nullptr, *z2 = nullptr, *y = nullptr, *dy = nullptr, *dz2 = nullptr, *dz1 = nullptr;
    float *dw1 = nullptr, *db1 = nullptr, *dw2 = nullptr, *db2 = nullptr, *dw3t = nullptr, *db3 = nullptr;
    std::vector<void *> owned, act;

    ~ntg_mlp() {
        cudaSetDevice(device);
        for (void *q : act) cudaFree(q);
        for (void *q : owned) cudaFree(q);
    }
};

namespace {

int mlp_fail(int code, const std::string &msg) {
    set_last_error(msg);
    return code;
}

#define MLP_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) return mlp_fail(NTG_ERROR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

#define MLP_LAUNCH(call)                                                                                \
    do {                                                                                                \
        int r_ = (call);                                                                                \
        if (r_ != 0) return r_ >= kLaunchErrorBase ? mlp_fail(NTG_ERROR_CUDA, std::string(#call ": ") +     \
                                                               cudaGetErrorString((cudaError_t)(r_ - kLaunchErrorBase))) \
                                                   : mlp_fail(r_, #call);                               \
    } while (0)

template <typename T>
int dalloc(std::vector<void *> &list, T **p, size_t n) {
    MLP_CUDA(cudaMalloc((void **)p, n * sizeof(T)));
    list.push_back(*p);
    return NTG_OK;
}

int ensure_batch(ntg_mlp *m, int batch) {
    if (batch <= m->cap) return NTG_OK;
    for (void *q : m->act) cudaFree(q);
    m->act.clear();
    const size_t B = (size_t)batch;
    auto &L = m->act;
    if (dalloc(L, &m->xb, B * IN) || dalloc(L, &m->xt, B * IN) || dalloc(L, &m->h1, B * HID) || dalloc(L, &m->h1t, B * HID) ||
        dalloc(L, &m->h2, B * HID) || dalloc(L, &m->h2t, B * HID) || dalloc(L, &m->dyb, B * OUTP) ||
        dalloc(L, &m->dyt, B * OUTP) || dalloc(L, &m->dz2b, B * HID) || dalloc(L, &m->dz2t, B * HID) ||
        dalloc(L, &m->dz1b, B * HID) || dalloc(L, &m->dz1t, B * HID) || dalloc(L, &m->z1, B * HID) ||
        dalloc(L, &m->z2, B * HID) || dalloc(L, &m->y, B * OUTP) || dalloc(L, &m->dy, B * OUTP) ||
        dalloc(L, &m->dz2, B * HID) || dalloc(L, &m->dz1, B * HID))
        return NTG_ERROR_CUDA;
    m->cap = batch;
    return NTG_OK;
}

GemmArgs gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K, int epi, int *status,
              int polls = kWaitPolls) {
    GemmArgs g;
    std::memset(&g, 0, sizeof g);
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.M = M; g.N = N; g.K = K; g.epi = epi; g.status = status;
    g.polls = polls;
    return g;
}

// Forward pass: X (bf16) -> Z1, H1, Z2, H2 -> Y [batch x OUTP]. `train` also writes the
// transposed activations the weight gradients need.
int forward(ntg_mlp *m, int batch, bool train, cudaStream_t s) {
    GemmArgs g = gemm(m->xb, IN, m->w1, IN, batch, HID, IN, EPI_GELU, m->status, m->polls);
    g.bias = m->p + OFF_B1; g.C = train ? m->z1 : nullptr; g.ldc = HID; g.H = m->h1; g.ldh = HID;
    g.HT = train ? m->h1t : nullptr; g.ldht = batch;
    MLP_LAUNCH(launch_gemm(g, 1, s));
    g = gemm(m->h1, HID, m->w2, HID, batch, HID, HID, EPI_GELU, m->status, m->polls);
    g.bias = m->p + OFF_B2; g.C = train ? m->z2 : nullptr; g.ldc = HID; g.H = m->h2; g.ldh = HID;
    g.HT = train ? m->h2t : nullptr; g.ldht = batch;
    MLP_LAUNCH(launch_gemm(g, 1, s));
    g = gemm(m->h2, HID, m->w3, HID, batch, OUTP, HID, EPI_F32, m->status, m->polls);
    g.bias = m->b3p; g.C = m->y; g.ldc = OUTP;
    MLP_LAUNCH(launch_gemm(g, 1, s));
    return NTG_OK;
}

// Backward pass into the flat gradient vector m->g (needs forward(train = true) first).
int backward(ntg_mlp *m, const float *d_t, int batch, cudaStream_t s) {
    const int splits = std::max(1, batch / 256);
    MLP_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), s));
    k_loss<<<grid_of((long long)batch * OUTP), 256, 0, s>>>(m->y, d_t, batch, m->wout, m->dy, m->dyb, m->dyt, m->loss);
    MLP_LAUNCH(launch_status());
    MLP_CUDA(cudaMemsetAsync(m->dw3t, 0, sizeof(float) * HID * OUTP, s));
    MLP_CUDA(cudaMemsetAsync(m->dw2, 0, sizeof(float) * HID * HID, s));
    MLP_CUDA(cudaMemsetAsync(m->dw1, 0, sizeof(float) * HID * IN, s));
    // dW3^T = H2^T dY
    GemmArgs g = gemm(m->h2t, batch, m->dyt, batch, HID, OUTP, batch, EPI_ATOMIC, m->status, m->polls);
    g.C = m->dw3t; g.ldc = OUTP;
    MLP_LAUNCH(launch_gemm(g, splits, s));
    k_colsum<<<OUTP, 256, 0, s>>>(m->dy, batch, OUTP, m->db3);
    // dZ2 = (dY W3) * gelu'(Z2)
    g = gemm(m->dyb, OUTP, m->w3t, OUTP, batch, HID, OUTP, EPI_DGELU, m->status, m->polls);
    g.Z = m->z2; g.ldz = HID; g.C = m->dz2; g.ldc = HID; g.H = m->dz2b; g.ldh = HID; g.HT = m->dz2t; g.ldht = batch;
    MLP_LAUNCH(launch_gemm(g, 1, s));
    k_colsum<<<HID, 256, 0, s>>>(m->dz2, batch, HID, m->db2);
    // dW2 = dZ2^T H1
    g = gemm(m->dz2t, batch, m->h1t, batch, HID, HID, batch, EPI_ATOMIC, m->status, m->polls);
    g.C = m->dw2; g.ldc = HID;
    MLP_LAUNCH(launch_gemm(g, splits, s));
    // dZ1 = (dZ2 W2) * gelu'(Z1)
    g = gemm(m->dz2b, HID, m->w2t, HID, batch, HID, HID, EPI_DGELU, m->status, m->polls);
    g.Z = m->z1; g.ldz = HID; g.C = m->dz1; g.ldc = HID; g.H = m->dz1b; g.ldh = HID; g.HT = m->dz1t; g.ldht = batch;
    MLP_LAUNCH(launch_gemm(g, 1, s));
    k_colsum<<<HID, 256, 0, s>>>(m->dz1, batch, HID, m->db1);
    // dW1 = dZ1^T X
    g = gemm(m->dz1t, batch, m->xt, batch, HID, IN, batch, EPI_ATOMIC, m->status, m->polls);
    g.C = m->dw1; g.ldc = IN;
    MLP_LAUNCH(launch_gemm(g, splits, s));
    k_gather_grads<<<grid_of(NPARAM), 256, 0, s>>>(m->dw1, m->db1, m->dw2, m->db2, m->dw3t, m->db3, m->g);
    MLP_LAUNCH(launch_status());
    return NTG_OK;
}

int load_inputs(ntg_mlp *m, const float *d_x, int batch, cudaStream_t s) {
    k_to_bf16<<<grid_of((long long)batch * IN), 256, 0, s>>>(d_x, batch, IN, m->xb, m->xt);
    MLP_LAUNCH(launch_status());
    return NTG_OK;
}

int refresh(ntg_mlp *m, cudaStream_t s) {
    k_refresh<<<grid_of(HID * HID), 256, 0, s>>>(m->p, m->w1, m->w2, m->w2t, m->w3, m->w3t, m->b3p);
    MLP_LAUNCH(launch_status());
    return NTG_OK;
}

int check_status(ntg_mlp *m, cudaStream_t s) {
    int st = 0;
    MLP_CUDA(cudaMemcpyAsync(&st, m->status, sizeof st, cudaMemcpyDeviceToHost, s));
    MLP_CUDA(cudaStreamSynchronize(s));
    if (st) return mlp_fail(NTG_ERROR_CUDA, "tensor-core wait timed out");
    return NTG_OK;
}

}  // namespace

namespace ntg {
// Forward pass for callers inside the library (the learned encoder): x fp32 [batch x 48] ->
// y fp32 [batch x 16].
int mlp_forward_device(ntg_mlp *m, const float *d_x, long long rows, float *d_y, cudaStream_t s) {
    if (!m || !d_x || !d_y || rows <= 0) return NTG_ERROR_INVALID_INPUT;
    static std::atomic<unsigned long long> configured{0};
    if (first_use_on_device(configured))
        cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F_BYTES);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
    const long long tiles = (rows + BM - 1) / BM;
    const int grid = (int)std::min<long long>(tiles, std::max(1, sms));
    k_mlp_infer<<<grid, 512, F_BYTES, s>>>(m->w1, m->w2, m->w3, m->p + OFF_B1, m->p + OFF_B2, m->b3p, d_x, rows, d_y,
                                           m->status, m->polls);
    MLP_LAUNCH(launch_status());
    return NTG_OK;
}
}  // namespace ntg

extern "C" {

int ntg_mlp_create(int device, unsigned long long seed, ntg_mlp **out) {
    if (!out) return mlp_fail(NTG_ERROR_INVALID_INPUT, "null output");
    MLP_CUDA(cudaSetDevice(device));
    std::unique_ptr<ntg_mlp> m(new ntg_mlp);
    m->device = device;
    auto &L = m->owned;
    if (dalloc(L, &m->p, NPARAM) || dalloc(L, &m->g, NPARAM) || dalloc(L, &m->m, NPARAM) || dalloc(L, &m->v, NPARAM) ||
        dalloc(L, &m->w1, (size_t)HID * IN) || dalloc(L, &m->w2, (size_t)HID * HID) || dalloc(L, &m->w2t, (size_t)HID * HID) ||
        dalloc(L, &m->w3, (size_t)OUTP * HID) || dalloc(L, &m->w3t, (size_t)HID * OUTP) || dalloc(L, &m->b3p, OUTP) ||
        dalloc(L, &m->wout, OUT) || dalloc(L, &m->loss, 1) || dalloc(L, &m->status, 1) || dalloc(L, &m->dw1, (size_t)HID * IN) ||
        dalloc(L, &m->db1, HID) || dalloc(L, &m->dw2, (size_t)HID * HID) || dalloc(L, &m->db2, HID) ||
        dalloc(L, &m->dw3t, (size_t)HID * OUTP) || dalloc(L, &m->db3, OUTP))
        return NTG_ERROR_CUDA;
    // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases, seeded
    std::vector<float> p(NPARAM);
    std::mt19937_64 rng(seed);
    auto fill = [&](size_t off, size_t n, int fan_in) {
        std::uniform_real_distribution<float> u(-1.0f / std::sqrt((float)fan_in), 1.0f / std::sqrt((float)fan_in));
        for (size_t i = 0; i < n; i++) p[off + i] = u(rng);
    };
    fill(OFF_W1, (size_t)HID * IN, IN); fill(OFF_B1, HID, IN);
    fill(OFF_W2, (size_t)HID * HID, HID); fill(OFF_B2, HID, HID);
    fill(OFF_W3, (size_t)OUT * HID, HID); fill(OFF_B3, OUT, HID);
    const float wout[OUT] = {1, 1, 1, 1, 1, 0.25f, 0, 0};
    MLP_CUDA(cudaMemcpy(m->p, p.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    MLP_CUDA(cudaMemset(m->m, 0, NPARAM * sizeof(float)));
    MLP_CUDA(cudaMemset(m->v, 0, NPARAM * sizeof(float)));
    MLP_CUDA(cudaMemset(m->status, 0, sizeof(int)));
    MLP_CUDA(cudaMemcpy(m->wout, wout, sizeof wout, cudaMemcpyHostToDevice));
    int r = refresh(m.get(), nullptr);
    if (r) return r;
    MLP_CUDA(cudaDeviceSynchronize());
    *out = m.release();
    return NTG_OK;
}

int ntg_mlp_destroy(ntg_mlp *m) {
    delete m;
    return NTG_OK;
}

int ntg_mlp_param_count(void) { return (int)NPARAM; }

int ntg_mlp_get_params(ntg_mlp *m, float *h_params) {
    if (!m || !h_params) return mlp_fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    MLP_CUDA(cudaSetDevice(m->device));
    MLP_CUDA(cudaMemcpy(h_params, m->p, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return NTG_OK;
}

int ntg_mlp_set_params(ntg_mlp *m, const float *h_params) {
    if (!m || !h_params) return mlp_fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    MLP_CUDA(cudaSetDevice(m->device));
    MLP_CUDA(cudaMemcpy(m->p, h_params, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    int r = refresh(m, nullptr);
    if (r) return r;
    MLP_CUDA(cudaDeviceSynchronize());
    return NTG_OK;
}

int ntg_mlp_infer(ntg_mlp *m, const float *d_x, int batch, float *d_y, void *stream) {
    if (!m || !d_x || !d_y || batch <= 0) return mlp_fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    MLP_CUDA(cudaSetDevice(m->device));
    return mlp_forward_device(m, d_x, batch, d_y, (cudaStream_t)stream);
}

// The unfused forward pass (three k_gemm launches), as training runs it; for testing.
int ntg_mlp_infer_unfused(ntg_mlp *m, const float *d_x, int batch, float *d_y, void *stream) {
    if (!m || !d_x || !d_y || batch <= 0) return mlp_fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    int r = ensure_batch(m, batch);
    if (!r) r = load_inputs(m, d_x, batch, s);
    if (!r) r = forward(m, batch, false, s);
    if (r) return r;
    MLP_CUDA(cudaMemcpyAsync(d_y, m->y, sizeof(float) * batch * OUTP, cudaMemcpyDeviceToDevice, s));
    return NTG_OK;
}

int ntg_mlp_gradients(ntg_mlp *m, const float *d_x, const float *d_t, int batch, float *d_grads, float *h_loss,
                      void *stream) {
    if (!m || !d_x || !d_t || batch <= 0) return mlp_fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    int r = ensure_batch(m, batch);
    if (!r) r = load_inputs(m, d_x, batch, s);
    if (!r) r = forward(m, batch, true, s);
    if (!r) r = backward(m, d_t, batch, s);
    if (r) return r;
    if (d_grads) MLP_CUDA(cudaMemcpyAsync(d_grads, m->g, NPARAM * sizeof(float), cudaMemcpyDeviceToDevice, s));
    if (h_loss) {
        MLP_CUDA(cudaMemcpyAsync(h_loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    }
    return check_status(m, s);
}

int ntg_mlp_train_step(ntg_mlp *m, const float *d_x, const float *d_t, int batch, float lr, float *d_loss, void *stream) {
    if (!m || !d_x || !d_t || batch <= 0) return mlp_fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    int r = ensure_batch(m, batch);
    if (!r) r = load_inputs(m, d_x, batch, s);
    if (!r) r = forward(m, batch, true, s);
    if (!r) r = backward(m, d_t, batch, s);
    if (r) return r;
    m->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)m->step), c2 = 1.0f - std::pow(b2, (float)m->step);
    k_adam<<<grid_of(NPARAM), 256, 0, s>>>(m->p, m->g, m->m, m->v, (int)NPARAM, lr, b1, b2, 1e-8f, c1, c2);
    MLP_LAUNCH(launch_status());
    r = refresh(m, s);
    if (r) return r;
    if (d_loss) MLP_CUDA(cudaMemcpyAsync(d_loss, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, s));
    return NTG_OK;
}

int ntg_mlp_status(ntg_mlp *m) {
    if (!m) return mlp_fail(NTG_ERROR_INVALID_INPUT, "null network");
    MLP_CUDA(cudaSetDevice(m->device));
    return check_status(m, nullptr);
}

int ntg_mlp_set_wait_limit(ntg_mlp *m, int polls) {
    if (!m) return mlp_fail(NTG_ERROR_INVALID_INPUT, "null network");
    MLP_CUDA(cudaSetDevice(m->device));
    MLP_CUDA(cudaDeviceSynchronize());
    m->polls = polls < 0 ? kWaitPolls : polls;
    MLP_CUDA(cudaMemset(m->status, 0, sizeof(int)));
    MLP_CUDA(cudaDeviceSynchronize());
    return NTG_OK;
}

int ntg_gemm_bf16(const void *d_a, const void *d_b, int M, int N, int K, float *d_c, void *stream) {
    if (!d_a || !d_b || !d_c || M <= 0 || N <= 0 || K <= 0) return mlp_fail(NTG_ERROR_INVALID_INPUT, "bad arguments");
    GemmArgs g = gemm((const __nv_bfloat16 *)d_a, K, (const __nv_bfloat16 *)d_b, K, M, N, K, EPI_F32, nullptr);
    g.C = d_c; g.ldc = N;
    MLP_LAUNCH(launch_gemm(g, 1, (cudaStream_t)stream));
    return NTG_OK;
}

}  // extern "C"
