// Surrogate warm start: a GELU multilayer perceptron with BF16 weights and activations and
// FP32 accumulation, trained and evaluated by hand-written kernels (tensor-core GEMM with
// mma.sync m16n8k16, bias/GELU epilogues, MSE loss, Adam), plus the kernel that resamples
// grid guesses onto each instance's initial mesh. The reference has no surrogate; its
// output replaces the constant initial guess copied to every mesh node
// (lib/BoundaryValueDiffEqCore/src/utils.jl:766-769).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "bvpgpu.h"

namespace {

using bf16 = __nv_bfloat16;

// ---- GEMM: C (Mr x Nc, fp32, row-major, ldc) = op(A) (Mr x K) * op(B) (K x Nc) ----------
// op(A)(m,k) = TA ? A[k*lda + m] : A[m*lda + k];  op(B)(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n]
// 64 x 64 CTA tile, 4 warps of 32 x 32, K steps of 32 staged in shared memory as
// As[m][k] and Bs[n][k] (k contiguous), the operand layouts of mma.m16n8k16.row.col.
constexpr int TM = 64, TN = 64, TK = 32, SP = TK + 8;

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) gemm_bf16(int Mr, int Nc, int K, const bf16* __restrict__ A, int lda,
                                                 const bf16* __restrict__ B, int ldb, float* __restrict__ C,
                                                 int ldc) {
    __shared__ __align__(16) bf16 As[TM][SP];
    __shared__ __align__(16) bf16 Bs[TN][SP];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
    const bf16 zero = __float2bfloat16(0.f);
    for (int k0 = 0; k0 < K; k0 += TK) {
        for (int e = tid; e < TM * TK; e += 128) {
            const int mm = e / TK, kk = e % TK;
            const int gm = m0 + mm, gk = k0 + kk;
            bf16 v = zero;
            if (gm < Mr && gk < K) v = TA ? A[(long long)gk * lda + gm] : A[(long long)gm * lda + gk];
            As[mm][kk] = v;
        }
        for (int e = tid; e < TN * TK; e += 128) {
            const int nn = e / TK, kk = e % TK;
            const int gn = n0 + nn, gk = k0 + kk;
            bf16 v = zero;
            if (gn < Nc && gk < K) v = TB ? B[(long long)gn * ldb + gk] : B[(long long)gk * ldb + gn];
            Bs[nn][kk] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16;
                af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r + g][kk + 2 * t]);
                af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + g + 8][kk + 2 * t]);
                af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r + g][kk + 2 * t + 8]);
                af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + g + 8][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = wn + j * 8;
                bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c + g][kk + 2 * t]);
                bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c + g][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = m0 + wm + i * 16 + g, c = n0 + wn + j * 8 + 2 * t;
            if (r < Mr && c < Nc) C[(long long)r * ldc + c] = acc[i][j][0];
            if (r < Mr && c + 1 < Nc) C[(long long)r * ldc + c + 1] = acc[i][j][1];
            if (r + 8 < Mr && c < Nc) C[(long long)(r + 8) * ldc + c] = acc[i][j][2];
            if (r + 8 < Mr && c + 1 < Nc) C[(long long)(r + 8) * ldc + c + 1] = acc[i][j][3];
        }
}

// ---- elementwise kernels -------------------------------------------------------------------
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.3989422804014327f * expf(-0.5f * z * z);
}

// x_n = (x - mu) / sd as BF16
__global__ void k_input(int B, int N, const float* x, const float* mu, const float* sd, bf16* h) {
    const long long n = (long long)B * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int c = int(e % N);
        h[e] = __float2bfloat16((x[e] - mu[c]) / sd[c]);
    }
}

// Z += b; hidden: H = bf16(gelu(Z)); output: y = Z * sd + mu (when y non-null)
__global__ void k_bias_act(int B, int N, float* Z, const float* b, bf16* H, float* y, const float* mu,
                           const float* sd) {
    const long long n = (long long)B * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int c = int(e % N);
        const float z = Z[e] + b[c];
        Z[e] = z;
        if (H) H[e] = __float2bfloat16(gelu(z));
        if (y) y[e] = z * sd[c] + mu[c];
    }
}

// MSE on normalised outputs: L = mean((z - (t - mu)/sd)^2); dZ = dL/dz
__global__ void k_mse(int B, int N, const float* Z, const float* T, const float* mu, const float* sd, float* dZ,
                      bf16* dZb, float* loss) {
    const long long n = (long long)B * N;
    const float s = 1.f / float(n);
    float part = 0.f;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int c = int(e % N);
        const float d = Z[e] - (T[e] - mu[c]) / sd[c];
        part += d * d * s;
        dZ[e] = 2.f * d * s;
        dZb[e] = __float2bfloat16(2.f * d * s);
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, part);
}

// dZ = dH * gelu'(Z) (fp32 and bf16 copies)
__global__ void k_gelu_bwd(int B, int N, const float* dH, const float* Z, float* dZ, bf16* dZb) {
    const long long n = (long long)B * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float v = dH[e] * gelu_d(Z[e]);
        dZ[e] = v;
        dZb[e] = __float2bfloat16(v);
    }
}

// db[c] = sum_r dZ[r][c]
__global__ void k_colsum(int B, int N, const float* dZ, float* db) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    float s = 0.f;
    for (int r = 0; r < B; ++r) s += dZ[(long long)r * N + c];
    db[c] = s;
}

__global__ void k_adam(long long n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float gg = g[e];
        const float mm = b1 * m[e] + (1.f - b1) * gg;
        const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
        m[e] = mm;
        v[e] = vv;
        w[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
}

__global__ void k_to_bf16(long long n, const float* src, bf16* dst) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        dst[e] = __float2bfloat16(src[e]);
}

__global__ void k_gather(int B, int N, const int* idx, const float* src, float* dst) {
    const long long n = (long long)B * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / N;
        dst[e] = src[(long long)idx[r] * N + e % N];
    }
}

// linear resampling of a uniform-grid guess onto each instance's uniform initial mesh
__global__ void k_resample(int n_inst, int n_grid, int M, const float* grid, const double* tspans, const int* nint,
                           const long long* off, double* y0) {
    const int q = blockIdx.x;
    if (q >= n_inst) return;
    const int n = nint[q];
    const float* gq = grid + (long long)q * n_grid * M;
    double* out = y0 + off[q] * M;
    const double inv_n = 1.0 / double(n);
    for (int j = threadIdx.x; j <= n; j += blockDim.x) {
        const double s = __dmul_rn(__dmul_rn(double(j), inv_n), double(n_grid - 1));
        int i0 = int(floor(s));
        i0 = i0 < 0 ? 0 : (i0 > n_grid - 2 ? n_grid - 2 : i0);
        const double f = s - i0;
        // separately rounded products and sum (no FMA contraction): the same values as the
        // host twin of this resampling
        for (int m = 0; m < M; ++m)
            out[(long long)j * M + m] =
                __dadd_rn(__dmul_rn(1.0 - f, double(gq[i0 * M + m])), __dmul_rn(f, double(gq[(i0 + 1) * M + m])));
    }
}

int grid1d(long long n) { return int(std::min<long long>((n + 255) / 256, 4096)); }

// ---- fused inference: every layer of the network in one kernel --------------------------
// A CTA takes FR rows of the batch through all layers: the activations stay in shared
// memory (BF16, two buffers used in turn); each layer's weights, kept in a transposed BF16
// copy [N][Kp] (k contiguous), are staged into shared memory with 16-byte loads (rows padded
// by 8 elements: the B-fragment reads are bank-conflict free), and each warp computes
// 8-column tiles of the layer output with mma.m16n8k16 (FP32 accumulation over k16 steps in
// order, as gemm_bf16 does). The epilogue adds the bias and applies GELU (hidden layers) or
// the output de-normalisation (last layer), with the same operations as k_bias_act, so the
// result equals the layer-by-layer forward.
constexpr int FR = 32;            // rows per CTA
constexpr int FWMAX = 256;        // widest layer the fused kernel takes
constexpr int FLD = FWMAX + 8;    // shared row stride (bf16): conflict-free fragment loads
constexpr int FLMAX = 8;          // layers
constexpr int FW = 8;              // warps per CTA: each takes every FW-th 8-column tile
constexpr int FT = FW * 32;        // threads per CTA
constexpr int FQ = FWMAX / 8 / FW; // 8-column tiles per warp at the widest layer

struct FusedNet {
    int L;
    int w[FLMAX + 1];
    int kp[FLMAX];                // layer input width rounded up to 16
    long long offWt[FLMAX];       // layer l's [N][kp] block in the transposed weights
    long long offb[FLMAX];        // bias offsets in the FP32 parameters
};

__global__ void k_build_wt(int L, FusedNet fn, const long long* offW, const bf16* pb, bf16* wt) {
    for (int l = 0; l < L; ++l) {
        const int K = fn.w[l], N = fn.w[l + 1], Kp = fn.kp[l];
        const bf16* W = pb + offW[l];
        bf16* T = wt + fn.offWt[l];
        const long long n = (long long)N * Kp;
        for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
             e += (long long)gridDim.x * blockDim.x) {
            const int nn = int(e / Kp), k = int(e % Kp);
            T[e] = k < K ? W[(long long)k * N + nn] : __float2bfloat16(0.f);
        }
    }
}

constexpr int FWLD = FWMAX + 8;   // staged weight row stride (bf16)
constexpr size_t FUSED_SMEM = size_t(2) * FR * FLD * 2 + size_t(FWMAX) * FWLD * 2;

__global__ void __launch_bounds__(FT) k_mlp_forward_fused(const FusedNet fn, int B, const float* __restrict__ x,
                                                           const bf16* __restrict__ wt, const float* __restrict__ p,
                                                           const float* __restrict__ nrm, float* __restrict__ y) {
    extern __shared__ __align__(16) unsigned char fsm[];
    bf16 (*act)[FR][FLD] = reinterpret_cast<bf16 (*)[FR][FLD]>(fsm);
    bf16* wsm = reinterpret_cast<bf16*>(fsm + size_t(2) * FR * FLD * 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const int r0 = blockIdx.x * FR;
    const int w0 = fn.w[0], wL = fn.w[fn.L];
    {
        const int kp = fn.kp[0];
        for (int e = tid; e < FR * kp; e += FT) {
            const int r = e / kp, c = e % kp;
            float v = 0.f;
            if (c < w0 && r0 + r < B) v = (x[(long long)(r0 + r) * w0 + c] - nrm[c]) / nrm[w0 + c];
            act[0][r][c] = __float2bfloat16(v);
        }
    }
    __syncthreads();
    int cur = 0;
    for (int l = 0; l < fn.L; ++l) {
        const int K = fn.kp[l], N = fn.w[l + 1];
        const int ntiles = N / 8;
        const int WLD = K + 8;
        {
            // stage the layer's [N][K] weights with asynchronous 16-byte copies, all in flight
            // at once (rows 16-byte aligned: K is a multiple of 16)
            const bf16* src = wt + fn.offWt[l];
            const int per_row = K / 8;
            for (int e = tid; e < N * per_row; e += FT) {
                const int nn = e / per_row, c = e - nn * per_row;
                const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(wsm + nn * WLD + c * 8));
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src + size_t(e) * 8));
            }
            asm volatile("cp.async.wait_all;\n" ::: "memory");
        }
        __syncthreads();
        const bf16* W = wsm;
        float acc[FQ][2][4];
#pragma unroll
        for (int q = 0; q < FQ; ++q)
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[q][i][c] = 0.f;
        for (int k0 = 0; k0 < K; k0 += 16) {
            uint32_t af[2][4];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = i * 16 + g;
                af[i][0] = *reinterpret_cast<const uint32_t*>(&act[cur][r][k0 + 2 * t]);
                af[i][1] = *reinterpret_cast<const uint32_t*>(&act[cur][r + 8][k0 + 2 * t]);
                af[i][2] = *reinterpret_cast<const uint32_t*>(&act[cur][r][k0 + 2 * t + 8]);
                af[i][3] = *reinterpret_cast<const uint32_t*>(&act[cur][r + 8][k0 + 2 * t + 8]);
            }
#pragma unroll
            for (int q = 0; q < FQ; ++q) {
                const int j = warp + FW * q;
                if (j < ntiles) {
                    const bf16* wr = W + (j * 8 + g) * WLD + k0 + 2 * t;
                    uint32_t bfr[2];
                    bfr[0] = *reinterpret_cast<const uint32_t*>(wr);
                    bfr[1] = *reinterpret_cast<const uint32_t*>(wr + 8);
                    mma_bf16(acc[q][0], af[0], bfr);
                    mma_bf16(acc[q][1], af[1], bfr);
                }
            }
        }
        const float* bias = p + fn.offb[l];
        const bool last = l == fn.L - 1;
        const float* mu = nrm + 2 * w0;
        const float* sd = nrm + 2 * w0 + wL;
#pragma unroll
        for (int q = 0; q < FQ; ++q) {
            const int j = warp + FW * q;
            if (j >= ntiles) continue;
            const int c = j * 8 + 2 * t;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int r = i * 16 + g + 8 * hh;
#pragma unroll
                    for (int cc = 0; cc < 2; ++cc) {
                        const float z = acc[q][i][2 * hh + cc] + bias[c + cc];
                        if (!last) act[cur ^ 1][r][c + cc] = __float2bfloat16(gelu(z));
                        else if (r0 + r < B) y[(long long)(r0 + r) * wL + c + cc] = z * sd[c + cc] + mu[c + cc];
                    }
                }
            }
        }
        __syncthreads();
        cur ^= 1;
    }
}

// ---- fused forward on the 5th-generation tensor cores (tcgen05, accumulators in TMEM) ---------
// A CTA takes TR = 128 rows through all layers. Shared memory holds the layer input (A, BF16,
// 128 x K) and the layer's weights (B, BF16, N x K, k contiguous) in the no-swizzle K-major
// core-matrix layout: 8 rows x 16 bytes per core matrix, the core matrices of an 8-row group
// consecutive along K (leading byte offset 128), the 8-row groups K * 16 bytes apart (stride
// byte offset). One thread issues K / 16 tcgen05.mma (M = 128, N = layer width, K = 16, BF16 x
// BF16 -> FP32) into a TMEM accumulator of N columns and commits them to an mbarrier; the 16
// warps then read the accumulator back (tcgen05.ld, warp w the TMEM lanes of its subpartition
// w % 4 and a quarter of the columns), add the bias, apply GELU and write the BF16 result as the next
// layer's A, while the next layer's weights stream into B with cp.async. The last layer writes
// the de-normalised output. Every wait is bounded: a timeout sets g_mlp_tc_timeout and the CTA
// still frees its TMEM.
constexpr int TR = 128;                       // rows per CTA (the MMA's M)
constexpr int TC_THREADS = 512;               // 16 warps: four per TMEM subpartition
constexpr int TC_KMAX = 256;                  // widest layer input
constexpr int TC_NMAX = 256;                  // widest layer output (TMEM columns)
constexpr size_t TC_A_BYTES = size_t(TR) * TC_KMAX * 2;
constexpr size_t TC_B_BYTES = size_t(TC_NMAX) * TC_KMAX * 2;
constexpr size_t TC_SMEM = TC_A_BYTES + TC_B_BYTES + 64;
__device__ int g_mlp_tc_timeout = 0;

// byte offset of element (row r, k) in the no-swizzle K-major core-matrix layout with K columns
__device__ __forceinline__ unsigned tc_off(int r, int k, int K) {
    return unsigned((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
// shared memory descriptor: start >> 4 (bits 0-13), leading byte offset >> 4 (16-29), stride
// byte offset >> 4 (32-45), descriptor version 1 (bit 46), no swizzle (bits 61-63 zero)
__device__ __forceinline__ unsigned long long tc_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
    return (unsigned long long)((saddr & 0x3FFFF) >> 4) | ((unsigned long long)(lbo >> 4) << 16) |
           ((unsigned long long)(sbo >> 4) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9
// and 10-12 = 1), both K-major, N >> 3 (bits 17-22), M >> 4 (bits 24-28)
__device__ __forceinline__ unsigned tc_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (unsigned(n >> 3) << 17) | (unsigned(TR >> 4) << 24);
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_forward_tc(const FusedNet fn, int B, const float* __restrict__ x,
                                                                  const bf16* __restrict__ wt, const float* __restrict__ p,
                                                                  const float* __restrict__ nrm, float* __restrict__ y) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    unsigned char* As = tsm;
    unsigned char* Bs = tsm + TC_A_BYTES;
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(tsm + TC_A_BYTES + TC_B_BYTES);
    unsigned* tslot = reinterpret_cast<unsigned*>(tsm + TC_A_BYTES + TC_B_BYTES + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r0 = blockIdx.x * TR;
    const int w0 = fn.w[0], wL = fn.w[fn.L];
    const unsigned a_s = static_cast<unsigned>(__cvta_generic_to_shared(As));
    const unsigned b_s = static_cast<unsigned>(__cvta_generic_to_shared(Bs));
    const unsigned mb_s = static_cast<unsigned>(__cvta_generic_to_shared(mbar));
    if (warp == 0) {
        const unsigned slot = static_cast<unsigned>(__cvta_generic_to_shared(tslot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(TC_NMAX));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb_s));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // the input rows, normalised, as the first A (columns up to kp[0] zero-padded)
    {
        const int kp = fn.kp[0];
        for (int e = tid; e < TR * kp; e += TC_THREADS) {
            const int r = e / kp, c = e % kp;
            float v = 0.f;
            if (c < w0 && r0 + r < B) v = (x[(long long)(r0 + r) * w0 + c] - nrm[c]) / nrm[w0 + c];
            *reinterpret_cast<bf16*>(As + tc_off(r, c, kp)) = __float2bfloat16(v);
        }
    }
    auto stage_weights = [&](int l) {
        const int K = fn.kp[l], N = fn.w[l + 1];
        const bf16* src = wt + fn.offWt[l];
        const int per_row = K / 8;
        for (int e = tid; e < N * per_row; e += TC_THREADS) {
            const int n = e / per_row, c = e - n * per_row;
            const unsigned dst = b_s + tc_off(n, c * 8, K);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src + size_t(e) * 8));
        }
    };
    stage_weights(0);
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tslot;
    unsigned phase = 0;
    bool timed_out = false;
    const float* mu = nrm + 2 * w0;
    const float* sd = nrm + 2 * w0 + wL;
    for (int l = 0; l < fn.L; ++l) {
        const int K = fn.kp[l], N = fn.w[l + 1];
        const bool last = l == fn.L - 1;
        if (tid == 0) {
            const unsigned idesc = tc_idesc(N);
            for (int ks = 0; ks < K / 16; ++ks) {
                const unsigned long long ad = tc_desc(a_s + ks * 256, 128, unsigned(K * 16));
                const unsigned long long bd = tc_desc(b_s + ks * 256, 128, unsigned(K * 16));
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(ks));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb_s)
                         : "memory");
        }
        // wait for the layer's products (bounded)
        {
            unsigned done = 0;
            for (long long it = 0; it < (1LL << 26) && !done; ++it)
                asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                             : "=r"(done) : "r"(mb_s), "r"(phase) : "memory");
            if (!done) { timed_out = true; atomicExch(&g_mlp_tc_timeout, 1); }
            phase ^= 1u;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (timed_out) break;
        if (!last) stage_weights(l + 1);   // B is free: the products are done
        // epilogue: warp w reads rows 32 (w % 4) .. + 31 of the accumulator, a quarter of the
        // columns (N / 4 is a multiple of 8 when N is a multiple of 32; otherwise the last
        // quarter is empty and the others take 8-column steps up to N)
        const int sub = warp & 3;
        const int r = sub * 32 + lane;
        const int quarter = (N / 4 + 7) / 8 * 8;
        const int cbeg = min((warp >> 2) * quarter, N), cend = min(cbeg + quarter, N);
        const float* bias = p + fn.offb[l];
        for (int c = cbeg; c < cend; c += 8) {
            unsigned v[8];
            const unsigned taddr = tmem + (unsigned(sub * 32) << 16) + unsigned(c);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (!last) {
                __align__(16) bf16 o[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) o[q] = __float2bfloat16(gelu(__uint_as_float(v[q]) + bias[c + q]));
                *reinterpret_cast<uint4*>(As + tc_off(r, c, N)) = *reinterpret_cast<const uint4*>(o);
            } else if (r0 + r < B) {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float z = __uint_as_float(v[q]) + bias[c + q];
                    y[(long long)(r0 + r) * wL + c + q] = z * sd[c + q] + mu[c + q];
                }
            }
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_NMAX));
}

}  // namespace

struct bvp_mlp_s {
    int L = 0;
    std::vector<int> w;
    std::vector<long long> offW, offb;
    long long np = 0;
    float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
    bf16* d_pb = nullptr;  // BF16 copy of the parameters (the W blocks are used)
    float *d_norm = nullptr;  // in_mu (w0), in_sd (w0), out_mu (wL), out_sd (wL)
    int cap = 0;
    std::vector<float*> Z;   // per layer pre-activations (cap x w[l+1])
    std::vector<bf16*> H;    // per layer inputs (cap x w[l]); H[0] the input
    float *d_dH = nullptr, *d_dZ = nullptr, *d_x = nullptr, *d_t = nullptr, *d_y = nullptr, *d_loss = nullptr;
    bf16* d_dZb = nullptr;
    int* d_idx = nullptr;
    cudaStream_t stream = nullptr;
    long long step = 0;
    std::string err;
    // fused inference (k_mlp_forward_fused) when every width fits it; on request the tcgen05
    // kernel (k_mlp_forward_tc) when, in addition, every layer width is a multiple of 16
    bool fused = false;
    bool tc = false;
    FusedNet fn{};
    bf16* d_wt = nullptr;         // transposed BF16 weights, [N][Kp] per layer
    long long* d_offW = nullptr;
};

namespace {

bool mlp_reserve(bvp_mlp* n, int batch) {
    if (batch <= n->cap) return true;
    for (auto p : n->Z) cudaFree(p);
    for (auto p : n->H) cudaFree(p);
    cudaFree(n->d_dH); cudaFree(n->d_dZ); cudaFree(n->d_dZb); cudaFree(n->d_x); cudaFree(n->d_t);
    cudaFree(n->d_y); cudaFree(n->d_idx);
    n->Z.assign(n->L, nullptr);
    n->H.assign(n->L, nullptr);
    int wmax = 0;
    for (int v : n->w) wmax = std::max(wmax, v);
    bool ok = true;
    for (int l = 0; l < n->L; ++l) {
        ok = ok && cudaMalloc(&n->Z[l], size_t(batch) * n->w[l + 1] * 4) == cudaSuccess;
        ok = ok && cudaMalloc(&n->H[l], size_t(batch) * n->w[l] * 2) == cudaSuccess;
    }
    ok = ok && cudaMalloc(&n->d_dH, size_t(batch) * wmax * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->d_dZ, size_t(batch) * wmax * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->d_dZb, size_t(batch) * wmax * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&n->d_x, size_t(batch) * n->w[0] * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->d_t, size_t(batch) * n->w[n->L] * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->d_y, size_t(batch) * n->w[n->L] * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&n->d_idx, size_t(batch) * 4) == cudaSuccess;
    if (ok) n->cap = batch;
    return ok;
}

void gemm(cudaStream_t s, bool ta, bool tb, int Mr, int Nc, int K, const bf16* A, int lda, const bf16* B, int ldb,
          float* C, int ldc) {
    dim3 grid((Nc + TN - 1) / TN, (Mr + TM - 1) / TM);
    if (!ta && !tb) gemm_bf16<false, false><<<grid, 128, 0, s>>>(Mr, Nc, K, A, lda, B, ldb, C, ldc);
    else if (ta && !tb) gemm_bf16<true, false><<<grid, 128, 0, s>>>(Mr, Nc, K, A, lda, B, ldb, C, ldc);
    else if (!ta && tb) gemm_bf16<false, true><<<grid, 128, 0, s>>>(Mr, Nc, K, A, lda, B, ldb, C, ldc);
    else gemm_bf16<true, true><<<grid, 128, 0, s>>>(Mr, Nc, K, A, lda, B, ldb, C, ldc);
}

// forward of a batch already in n->d_x; writes Z of every layer, y when y != nullptr
void forward(bvp_mlp* n, int B, const float* d_x, float* d_y) {
    const int L = n->L;
    const float* nrm = n->d_norm;
    const long long w0 = n->w[0], wL = n->w[L];
    k_input<<<grid1d(B * w0), 256, 0, n->stream>>>(B, int(w0), d_x, nrm, nrm + w0, n->H[0]);
    for (int l = 0; l < L; ++l) {
        const int ni = n->w[l], no = n->w[l + 1];
        gemm(n->stream, false, false, B, no, ni, n->H[l], ni, n->d_pb + n->offW[l], no, n->Z[l], no);
        const bool last = l == L - 1;
        k_bias_act<<<grid1d((long long)B * no), 256, 0, n->stream>>>(
            B, no, n->Z[l], n->d_p + n->offb[l], last ? nullptr : n->H[l + 1], last ? d_y : nullptr,
            nrm + 2 * w0, nrm + 2 * w0 + wL);
    }
}

// backward of the MSE loss for the batch in d_x / d_t; gradient into n->d_g, loss added to *d_loss
void backward(bvp_mlp* n, int B, const float* d_t) {
    const int L = n->L;
    const long long w0 = n->w[0], wL = n->w[L];
    const float* nrm = n->d_norm;
    k_mse<<<grid1d(B * wL), 256, 0, n->stream>>>(B, int(wL), n->Z[L - 1], d_t, nrm + 2 * w0, nrm + 2 * w0 + wL,
                                                  n->d_dZ, n->d_dZb, n->d_loss);
    for (int l = L - 1; l >= 0; --l) {
        const int ni = n->w[l], no = n->w[l + 1];
        // dW = H_l^T dZ (ni x no), db = colsum dZ
        gemm(n->stream, true, false, ni, no, B, n->H[l], ni, n->d_dZb, no, n->d_g + n->offW[l], no);
        k_colsum<<<(no + 127) / 128, 128, 0, n->stream>>>(B, no, n->d_dZ, n->d_g + n->offb[l]);
        if (l > 0) {
            // dH = dZ W^T (B x ni), then through the activation of layer l-1
            gemm(n->stream, false, true, B, ni, no, n->d_dZb, no, n->d_pb + n->offW[l], no, n->d_dH, ni);
            k_gelu_bwd<<<grid1d((long long)B * ni), 256, 0, n->stream>>>(B, ni, n->d_dH, n->Z[l - 1], n->d_dZ,
                                                                          n->d_dZb);
        }
    }
}

// transposed weights for the fused forward, rebuilt whenever the BF16 weights change
void refresh_wt(bvp_mlp* n) {
    if (!n->fused) return;
    k_build_wt<<<256, 256, 0, n->stream>>>(n->L, n->fn, n->d_offW, n->d_pb, n->d_wt);
}

// inference on device pointers: the fused kernel when the network fits it, else layer by layer
void infer(bvp_mlp* n, int B, const float* d_x, float* d_y, cudaStream_t s) {
    if (n->tc) {
        k_mlp_forward_tc<<<(B + TR - 1) / TR, TC_THREADS, TC_SMEM, s>>>(n->fn, B, d_x, n->d_wt, n->d_p, n->d_norm, d_y);
    } else if (n->fused) {
        k_mlp_forward_fused<<<(B + FR - 1) / FR, FT, FUSED_SMEM, s>>>(n->fn, B, d_x, n->d_wt, n->d_p, n->d_norm, d_y);
    } else {
        cudaStream_t prev = n->stream;
        n->stream = s;
        forward(n, B, d_x, d_y);
        n->stream = prev;
    }
}

}  // namespace

extern "C" {

bvp_status bvp_mlp_create(int32_t n_layers, const int32_t* widths, bvp_mlp** out) {
    if (!out || n_layers < 1 || n_layers > 16 || !widths) return BVP_ERR_INVALID;
    *out = nullptr;
    for (int l = 0; l <= n_layers; ++l)
        if (widths[l] < 1 || widths[l] > 8192) return BVP_ERR_INVALID;
    bvp_mlp* n = new bvp_mlp_s();
    n->L = n_layers;
    n->w.assign(widths, widths + n_layers + 1);
    long long o = 0;
    for (int l = 0; l < n_layers; ++l) {
        n->offW.push_back(o);
        o += (long long)n->w[l] * n->w[l + 1];
        n->offb.push_back(o);
        o += n->w[l + 1];
    }
    n->np = o;
    *out = n;
    const long long w0 = n->w[0], wL = n->w[n_layers];
    bool ok = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMalloc(&n->d_p, o * 4) == cudaSuccess && cudaMalloc(&n->d_g, o * 4) == cudaSuccess &&
         cudaMalloc(&n->d_m, o * 4) == cudaSuccess && cudaMalloc(&n->d_v, o * 4) == cudaSuccess &&
         cudaMalloc(&n->d_pb, o * 2) == cudaSuccess && cudaMalloc(&n->d_norm, (2 * w0 + 2 * wL) * 4) == cudaSuccess &&
         cudaMalloc(&n->d_loss, 4) == cudaSuccess;
    if (!ok) { n->err = "allocation failed"; return BVP_ERR_CUDA; }
    n->fused = n_layers <= FLMAX && n->w[0] <= FWMAX;
    for (int l = 1; l <= n_layers && n->fused; ++l) n->fused = n->w[l] <= FWMAX && n->w[l] % 8 == 0;
    if (n->fused) {
        FusedNet& f = n->fn;
        f.L = n_layers;
        long long ot = 0;
        for (int l = 0; l <= n_layers; ++l) f.w[l] = n->w[l];
        for (int l = 0; l < n_layers; ++l) {
            f.kp[l] = (n->w[l] + 15) / 16 * 16;
            f.offWt[l] = ot;
            ot += (long long)n->w[l + 1] * f.kp[l];
            f.offb[l] = n->offb[l];
        }
        // the tcgen05 kernel on request (BVPGPU_MLP_TC=1): on the 3-256-256-256-128 surrogate
        // it takes 52 us for 4096 rows against the mma.sync kernel's 30 us (32 CTAs of 128 rows
        // against 128 CTAs of 32, each layer a dependent chain of weight staging, products and
        // epilogue), so the mma.sync kernel stays the default
        const char* env = std::getenv("BVPGPU_MLP_TC");
        n->tc = env && env[0] == '1';
        for (int l = 1; l <= n_layers; ++l) n->tc = n->tc && n->w[l] % 16 == 0 && n->w[l] >= 16;
        if (n->tc)
            ok = cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(TC_SMEM)) ==
                 cudaSuccess;
        ok = ok &&
             cudaFuncSetAttribute(k_mlp_forward_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, int(FUSED_SMEM)) ==
                 cudaSuccess &&
             cudaMalloc(&n->d_wt, ot * 2) == cudaSuccess && cudaMalloc(&n->d_offW, n_layers * 8) == cudaSuccess &&
             cudaMemcpy(n->d_offW, n->offW.data(), n_layers * 8, cudaMemcpyHostToDevice) == cudaSuccess;
        if (!ok) { n->err = "allocation failed"; return BVP_ERR_CUDA; }
    }
    std::vector<float> nrm(2 * w0 + 2 * wL);
    for (long long k = 0; k < w0; ++k) { nrm[k] = 0.f; nrm[w0 + k] = 1.f; }
    for (long long k = 0; k < wL; ++k) { nrm[2 * w0 + k] = 0.f; nrm[2 * w0 + wL + k] = 1.f; }
    cudaMemcpy(n->d_norm, nrm.data(), nrm.size() * 4, cudaMemcpyHostToDevice);
    cudaMemset(n->d_p, 0, o * 4);
    cudaMemset(n->d_pb, 0, o * 2);
    return BVP_OK;
}

int64_t bvp_mlp_num_params(bvp_mlp* n) { return n ? n->np : 0; }

bvp_status bvp_mlp_set_params(bvp_mlp* n, const float* params) {
    if (!n || !params) return BVP_ERR_INVALID;
    if (cudaMemcpy(n->d_p, params, n->np * 4, cudaMemcpyHostToDevice) != cudaSuccess) return BVP_ERR_CUDA;
    cudaMemset(n->d_m, 0, n->np * 4);
    cudaMemset(n->d_v, 0, n->np * 4);
    n->step = 0;
    k_to_bf16<<<grid1d(n->np), 256, 0, n->stream>>>(n->np, n->d_p, n->d_pb);
    refresh_wt(n);
    return cudaStreamSynchronize(n->stream) == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
}

bvp_status bvp_mlp_get_params(bvp_mlp* n, float* params) {
    if (!n || !params) return BVP_ERR_INVALID;
    cudaStreamSynchronize(n->stream);
    return cudaMemcpy(params, n->d_p, n->np * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
}

// Input and output normalisation: x_n = (x - in_mu)/in_sd, y = z out_sd + out_mu.
bvp_status bvp_mlp_set_normalization(bvp_mlp* n, const float* in_mu, const float* in_sd, const float* out_mu,
                                     const float* out_sd) {
    if (!n || !in_mu || !in_sd || !out_mu || !out_sd) return BVP_ERR_INVALID;
    const long long w0 = n->w[0], wL = n->w[n->L];
    std::vector<float> nrm(2 * w0 + 2 * wL);
    std::memcpy(nrm.data(), in_mu, w0 * 4);
    std::memcpy(nrm.data() + w0, in_sd, w0 * 4);
    std::memcpy(nrm.data() + 2 * w0, out_mu, wL * 4);
    std::memcpy(nrm.data() + 2 * w0 + wL, out_sd, wL * 4);
    return cudaMemcpy(n->d_norm, nrm.data(), nrm.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess ? BVP_OK
                                                                                                  : BVP_ERR_CUDA;
}

bvp_status bvp_mlp_forward_device(bvp_mlp* n, int32_t B, const float* d_x, float* d_y, void* stream) {
    if (!n || B < 1 || !d_x || !d_y) return BVP_ERR_INVALID;
    if (!n->fused && !mlp_reserve(n, B)) return BVP_ERR_NOMEM;
    infer(n, B, d_x, d_y, stream ? static_cast<cudaStream_t>(stream) : n->stream);
    return cudaGetLastError() == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
}

bvp_status bvp_mlp_forward(bvp_mlp* n, int32_t B, const float* x, float* y) {
    if (!n || B < 1 || !x || !y) return BVP_ERR_INVALID;
    if (!mlp_reserve(n, B)) return BVP_ERR_NOMEM;
    const long long w0 = n->w[0], wL = n->w[n->L];
    cudaMemcpyAsync(n->d_x, x, B * w0 * 4, cudaMemcpyHostToDevice, n->stream);
    infer(n, B, n->d_x, n->d_y, n->stream);
    cudaMemcpyAsync(y, n->d_y, B * wL * 4, cudaMemcpyDeviceToHost, n->stream);
    return cudaStreamSynchronize(n->stream) == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
}

bvp_status bvp_mlp_loss_grad(bvp_mlp* n, int32_t B, const float* x, const float* t, float* loss, float* grad) {
    if (!n || B < 1 || !x || !t) return BVP_ERR_INVALID;
    if (!mlp_reserve(n, B)) return BVP_ERR_NOMEM;
    const long long w0 = n->w[0], wL = n->w[n->L];
    cudaMemcpyAsync(n->d_x, x, B * w0 * 4, cudaMemcpyHostToDevice, n->stream);
    cudaMemcpyAsync(n->d_t, t, B * wL * 4, cudaMemcpyHostToDevice, n->stream);
    cudaMemsetAsync(n->d_loss, 0, 4, n->stream);
    forward(n, B, n->d_x, nullptr);
    backward(n, B, n->d_t);
    if (loss) cudaMemcpyAsync(loss, n->d_loss, 4, cudaMemcpyDeviceToHost, n->stream);
    if (grad) cudaMemcpyAsync(grad, n->d_g, n->np * 4, cudaMemcpyDeviceToHost, n->stream);
    return cudaStreamSynchronize(n->stream) == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
}

bvp_status bvp_mlp_train(bvp_mlp* n, int32_t N, const float* x, const float* t, int32_t epochs, int32_t B, float lr,
                         uint64_t seed, float* last_loss) {
    if (!n || N < 1 || !x || !t || epochs < 1 || B < 1) return BVP_ERR_INVALID;
    B = std::min(B, N);
    if (!mlp_reserve(n, B)) return BVP_ERR_NOMEM;
    const long long w0 = n->w[0], wL = n->w[n->L];
    float *dX = nullptr, *dT = nullptr;
    int* dperm = nullptr;
    if (cudaMalloc(&dX, (long long)N * w0 * 4) != cudaSuccess || cudaMalloc(&dT, (long long)N * wL * 4) != cudaSuccess ||
        cudaMalloc(&dperm, (long long)N * 4) != cudaSuccess) {
        cudaFree(dX); cudaFree(dT); cudaFree(dperm);
        return BVP_ERR_NOMEM;
    }
    cudaMemcpyAsync(dX, x, (long long)N * w0 * 4, cudaMemcpyHostToDevice, n->stream);
    cudaMemcpyAsync(dT, t, (long long)N * wL * 4, cudaMemcpyHostToDevice, n->stream);
    std::mt19937_64 rng(seed);
    std::vector<int> perm(N);
    const int steps = N / B;
    float epoch_loss = 0.f;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int i = 0; i < N; ++i) perm[i] = i;
        std::shuffle(perm.begin(), perm.end(), rng);
        cudaMemcpyAsync(dperm, perm.data(), (long long)N * 4, cudaMemcpyHostToDevice, n->stream);
        cudaMemsetAsync(n->d_loss, 0, 4, n->stream);
        // cosine decay of the step size over the run
        for (int s = 0; s < steps; ++s) {
            const double frac = (double(ep) * steps + s) / (double(epochs) * steps);
            const float lr_s = float(0.5 * lr * (1.0 + std::cos(3.141592653589793 * frac)));
            k_gather<<<grid1d((long long)B * w0), 256, 0, n->stream>>>(B, int(w0), dperm + (long long)s * B, dX, n->d_x);
            k_gather<<<grid1d((long long)B * wL), 256, 0, n->stream>>>(B, int(wL), dperm + (long long)s * B, dT, n->d_t);
            forward(n, B, n->d_x, nullptr);
            backward(n, B, n->d_t);
            ++n->step;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.f - std::pow(b1, float(n->step)), c2 = 1.f - std::pow(b2, float(n->step));
            k_adam<<<grid1d(n->np), 256, 0, n->stream>>>(n->np, n->d_p, n->d_g, n->d_m, n->d_v, lr_s, b1, b2, 1e-8f, c1, c2);
            k_to_bf16<<<grid1d(n->np), 256, 0, n->stream>>>(n->np, n->d_p, n->d_pb);
        }
        cudaMemcpyAsync(&epoch_loss, n->d_loss, 4, cudaMemcpyDeviceToHost, n->stream);
        if (cudaStreamSynchronize(n->stream) != cudaSuccess) break;
        epoch_loss /= float(std::max(steps, 1));
    }
    refresh_wt(n);
    const cudaError_t e = cudaStreamSynchronize(n->stream);
    cudaFree(dX); cudaFree(dT); cudaFree(dperm);
    if (last_loss) *last_loss = epoch_loss;
    return e == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
}

bvp_status bvp_resample_guess_device(int32_t n_inst, int32_t n_grid, int32_t M, const float* d_grid,
                                     const double* d_tspans, const int32_t* d_n_intervals, const int64_t* d_y0_off,
                                     double* d_y0, void* stream) {
    if (n_inst < 1 || n_grid < 2 || M < 1 || !d_grid || !d_n_intervals || !d_y0_off || !d_y0) return BVP_ERR_INVALID;
    (void)d_tspans;  // the grid spans each instance's own tspan
    k_resample<<<n_inst, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        n_inst, n_grid, M, d_grid, d_tspans, d_n_intervals, reinterpret_cast<const long long*>(d_y0_off), d_y0);
    return cudaGetLastError() == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
}

void bvp_mlp_destroy(bvp_mlp* n) {
    if (!n) return;
    for (auto p : n->Z) cudaFree(p);
    for (auto p : n->H) cudaFree(p);
    cudaFree(n->d_p); cudaFree(n->d_g); cudaFree(n->d_m); cudaFree(n->d_v); cudaFree(n->d_pb);
    cudaFree(n->d_norm); cudaFree(n->d_dH); cudaFree(n->d_dZ); cudaFree(n->d_dZb); cudaFree(n->d_x);
    cudaFree(n->d_t); cudaFree(n->d_y); cudaFree(n->d_loss); cudaFree(n->d_idx);
    cudaFree(n->d_wt); cudaFree(n->d_offW);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
}

}  // extern "C"

// ---- forward without allocation ------------------------------------------------------------
// bvp_mlp_forward_noalloc: a network the fused kernel takes (every width <= 256 and, past the
// input, a multiple of 8) runs k_mlp_forward_fused, which needs no scratch beyond shared
// memory. Any other network runs the layer-by-layer kernels on scratch carved from this
// static device array instead of the network's cudaMalloc'd activation buffers: two BF16
// activation buffers used in turn (layer input / layer output) and one FP32 pre-activation
// buffer.
static __device__ __align__(256) unsigned char bvp_mlp_static_scratch[BVP_MLP_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kNoAllocDevices = 64;
std::atomic<void*> g_noalloc_scratch[kNoAllocDevices];  // device address of the array, per device
std::mutex g_noalloc_mu;

size_t round256(size_t b) { return (b + 255) & ~size_t(255); }
}  // namespace

extern "C" bvp_status bvp_mlp_forward_noalloc(bvp_mlp* n, int32_t B, const float* d_x, float* d_y, void* stream) {
    if (!n || B < 1 || !d_x || !d_y) return BVP_ERR_INVALID;
    const cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : n->stream;
    if (n->fused) {
        infer(n, B, d_x, d_y, s);
        return cudaGetLastError() == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
    }
    int wmax = 0;
    for (int v : n->w) wmax = std::max(wmax, v);
    const size_t hb = round256(size_t(B) * wmax * sizeof(bf16)), zb = round256(size_t(B) * wmax * sizeof(float));
    if (2 * hb + zb > size_t(BVP_MLP_NOALLOC_SCRATCH_BYTES)) return BVP_ERR_TOO_LARGE;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return BVP_ERR_CUDA;
    if (dev < 0 || dev >= kNoAllocDevices) return BVP_ERR_INVALID;
    void* base = g_noalloc_scratch[dev].load(std::memory_order_acquire);
    if (!base) {
        // first call on this device: the lookup loads the module that holds the array
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        base = g_noalloc_scratch[dev].load(std::memory_order_relaxed);
        if (!base) {
            if (cudaGetSymbolAddress(&base, bvp_mlp_static_scratch) != cudaSuccess || !base) return BVP_ERR_CUDA;
            g_noalloc_scratch[dev].store(base, std::memory_order_release);
        }
    }
    char* scr = static_cast<char*>(base);
    bf16* hin = reinterpret_cast<bf16*>(scr);
    bf16* hout = reinterpret_cast<bf16*>(scr + hb);
    float* Z = reinterpret_cast<float*>(scr + 2 * hb);
    const int L = n->L;
    const float* nrm = n->d_norm;
    const long long w0 = n->w[0], wL = n->w[L];
    k_input<<<grid1d(B * w0), 256, 0, s>>>(B, int(w0), d_x, nrm, nrm + w0, hin);
    for (int l = 0; l < L; ++l) {
        const int ni = n->w[l], no = n->w[l + 1];
        gemm(s, false, false, B, no, ni, hin, ni, n->d_pb + n->offW[l], no, Z, no);
        const bool last = l == L - 1;
        k_bias_act<<<grid1d((long long)B * no), 256, 0, s>>>(B, no, Z, n->d_p + n->offb[l], last ? nullptr : hout,
                                                              last ? d_y : nullptr, nrm + 2 * w0, nrm + 2 * w0 + wL);
        std::swap(hin, hout);
    }
    return cudaGetLastError() == cudaSuccess ? BVP_OK : BVP_ERR_CUDA;
}
