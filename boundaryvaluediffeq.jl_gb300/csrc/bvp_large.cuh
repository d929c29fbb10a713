// Batched adaptive MIRK for larger state dimensions (9 <= M <= 32) on sm_103a: device code.
//
// NVRTC compiles this file instead of bvp_kernels.cuh when the problem's state dimension is
// above what one warp keeps in registers. The algorithm is the same (the reference's MIRK
// solve: collocation.jl:44-72, mirk.jl:286-388, adaptivity.jl:6-75, 250-461); the work is
// laid out differently:
//   bl_residual  one thread per (instance, interval): FP64 stages and collocation residual,
//                the BC rows on the instance's last thread; max |F| and sum F^2 per instance
//   bl_jacobian  one warp per run of 8 intervals: J_f at the stage points one column per
//                lane (one-direction duals, node stages shared between neighbours), then
//                the stage chain to the blocks S_i = dr_i/dy_i, R_i = dr_i/dy_{i+1} in
//                BVP_JT; the warp after an instance's last run computes the BC blocks
//   bl_linsolve  one CTA per instance: each warp eliminates a chunk of intervals node by
//                node (the 2M x M pivot panel LU-factorised with row pivoting in registers,
//                the trailing columns by a column-parallel triangular solve and Schur
//                update from shared memory), the chunk relations are combined pairwise, a
//                2M x 2M system with the BC rows gives the end values, and the warps
//                back-substitute their chunks
//   bl_update    y += delta (or y = ybase + alpha delta for the line search)
//   bl_defect    one thread per interval: extra stages and the defect at tau*, 1 - tau*
//   bl_transfer  one warp per refined instance: the new guess from the old interpolant
// The host runs the Newton iterations and the mesh rounds between these launches (the mesh
// selection itself is sequential per instance and runs there).
// Two-point boundary conditions only (bca at t0, bcb at t1).
#pragma once

#ifndef BVP_JT
#define BVP_JT float
#endif
#define BVP_JT_PTR BVP_JT
#include "bvp_shared.h"
#ifndef BVP_TWOPOINT
#define BVP_TWOPOINT 1
#endif
#ifndef BVP_LA
#define BVP_LA 0
#endif
#include "bvp_tableau.cuh"

template <class T, class P> BVP_DEV void bvp_bc(T*, const T* const*, const P*) {}

namespace bvp {

static_assert(BVP_TWOPOINT == 1, "the larger-state kernels take two-point boundary conditions");
constexpr unsigned FULL = 0xffffffffu;
constexpr int M = BVP_M;
constexpr int LA = BVP_LA;
using JT = BVP_JT;
constexpr int RECW = 3 * M * M + M;
#define BVP_B16(n) ((((n) + 15) / 16) * 16)

// Jacobian kernel layout: JG intervals per warp, JW tangent directions per chain pass, per
// warp S stage-Jacobian slots (M x JLD), the primal stage points and one pass of dY rows
constexpr bool LNODE = S >= 2 && ORD >= 4;   // stage 0 at the left node, stage 1 at the right
constexpr int JG = 8;
constexpr int JW = 16;
constexpr int JLD = M + 1;                   // odd: lane m reading row m is conflict-free
constexpr int DYLD = JW + 4;
constexpr int JWARP_BYTES = BVP_B16((S * M * JLD + S * M + M * DYLD) * int(sizeof(JT)));
constexpr int JPMAX = 6144;                  // parameters staged in shared memory up to this count
// slot of stage r's J_f for the kk-th interval of a run: the two node stages alternate
BVP_DEV int jslot(int r, int kk) {
    if (LNODE && r == 0) return kk & 1;
    if (LNODE && r == 1) return (kk + 1) & 1;
    return r;
}
// 4 entries of a register row (zero past its end) to 16-byte aligned shared memory
template <int N>
BVP_DEV void st4(JT* p, const JT (&a)[N], int j) {
    const JT v0 = a[j], v1 = j + 1 < N ? a[j + 1] : JT(0), v2 = j + 2 < N ? a[j + 2] : JT(0),
             v3 = j + 3 < N ? a[j + 3] : JT(0);
    if constexpr (sizeof(JT) == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(v0, v1, v2, v3);
    } else {
        *reinterpret_cast<double2*>(p) = make_double2(v0, v1);
        *reinterpret_cast<double2*>(p + 2) = make_double2(v2, v3);
    }
}
// TF32 head and tail of an FP32 value (x = head + tail to about 2^-22 relative)
BVP_DEV void tf32_split(float x, unsigned& hi, unsigned& lo) {
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(hi) : "f"(x));
    const float r = x - __uint_as_float(hi);
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(lo) : "f"(r));
}
// d += a b on the tensor cores: a 16 x 8 (row), b 8 x 8 (column), d 16 x 8, FP32 accumulation
BVP_DEV void mma_tf32(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
// the Schur update of the larger-state elimination runs on the tensor cores for FP32 blocks
// of state dimension 32
constexpr bool MMA_SCHUR = sizeof(JT) == 4 && M == 32;
// correctly rounded reciprocal
BVP_DEV float rcp_rn(float x) { return __frcp_rn(x); }
BVP_DEV double rcp_rn(double x) { return __drcp_rn(x); }
// 4 consecutive entries from shared memory (16-byte aligned)
BVP_DEV void ld4(const JT* p, JT* v) {
    if constexpr (sizeof(JT) == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else {
        const double2 t0 = *reinterpret_cast<const double2*>(p);
        const double2 t1 = *reinterpret_cast<const double2*>(p + 2);
        v[0] = t0.x; v[1] = t0.y; v[2] = t1.x; v[3] = t1.y;
    }
}
static_assert(M <= 32 && M > 0, "M <= 32");

BVP_DEV int lane_id() { return threadIdx.x & 31; }
BVP_DEV unsigned long long norm_bits(double v) { return (unsigned long long)__double_as_longlong(v); }

#ifndef BVP_SINGULAR
#define BVP_SINGULAR 0
#endif
// A collocation stage: f plus the singular term S u / t for t > 0 (collocation.jl:60-66 with
// __add_singular_term!, Core/src/utils.jl:936-941); the interpolant's extra stages and the
// defect evaluate f alone, as the reference does.
template <class T, class PT> BVP_DEV void stage_f(T* du, const T* u, const PT* p, PT t) {
    bvp_f<T, PT>(du, u, p, t);
#if BVP_SINGULAR
    if (t > PT(0)) {
        T su[M];
        bvp_sing<T, PT>(su, u, p);
        const PT it = PT(1) / t;
#pragma unroll
        for (int m = 0; m < M; ++m) du[m] = du[m] + su[m] * it;
    }
#endif
}

// stages and residual of one interval (collocation.jl:44-72), the expression order of the
// warp-per-instance kernels
template <class T, class PT, class TT>
BVP_DEV void phi_large(const T* yi, const T* yi1, T* K, T* r, const PT* p, TT ti, TT hi_t) {
    const PT hi = PT(hi_t);
    T Y[M];
#pragma unroll
    for (int rr = 0; rr < S; ++rr) {
#pragma unroll 4
        for (int m = 0; m < M; ++m) Y[m] = PT(1.0 - tab_v(rr)) * yi[m] + PT(tab_v(rr)) * yi1[m];
#pragma unroll
        for (int j = 0; j < rr; ++j) {
            if (tab_x(rr, j) != 0.0) {
#pragma unroll 4
                for (int m = 0; m < M; ++m) Y[m] = Y[m] + hi * (K[j * M + m] * PT(tab_x(rr, j)));
            }
        }
        stage_f<T, PT>(&K[rr * M], Y, p, PT(ti + TT(tab_c(rr)) * hi_t));
    }
#pragma unroll 4
    for (int m = 0; m < M; ++m) {
        T acc = K[m] * PT(tab_b(0));
#pragma unroll
        for (int rr = 1; rr < S; ++rr) acc = acc + K[rr * M + m] * PT(tab_b(rr));
        r[m] = (yi1[m] - yi[m]) - hi * acc;
    }
}

// extra interpolant stages (interpolation.jl:337-372)
BVP_DEV void interp_large(const double* yi, const double* yi1, const double* K, double* KI, const double* p,
                          double ti, double hi) {
    double Y[M];
#pragma unroll
    for (int r = 0; r < NSX; ++r) {
#pragma unroll 4
        for (int m = 0; m < M; ++m) {
            double acc = K[m] * tab_xs(r, 0);
#pragma unroll
            for (int j = 1; j < S; ++j) acc = acc + K[j * M + m] * tab_xs(r, j);
#pragma unroll
            for (int q = 0; q < r; ++q) acc = acc + KI[q * M + m] * tab_xs(r, S + q);
            Y[m] = acc * hi + (1.0 - tab_vs(r)) * yi[m] + tab_vs(r) * yi1[m];
        }
        bvp_f<double, double>(&KI[r * M], Y, p, ti + tab_cs(r) * hi);
    }
}

BVP_DEV void reduce_norm(const BvpLargeArgs& a, int q, double mx, double sq, bool bad) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(FULL, mx, o));
        sq += __shfl_xor_sync(FULL, sq, o);
        bad |= __shfl_xor_sync(FULL, int(bad), o) != 0;
    }
    if (lane_id() == 0) {
        if (bad) mx = __longlong_as_double(0x7ff0000000000000LL);
        atomicMax(&a.norm[q], norm_bits(mx));
        atomicAdd(&a.sq[q], sq);
    }
}

}  // namespace bvp

// ---- residual: blockIdx.y = active instance, threads over intervals (+ one BC thread) ----
extern "C" __global__ void __launch_bounds__(128) bl_residual(const BvpLargeArgs a) {
    using namespace bvp;
    const int q = a.active[blockIdx.y];
    const int N = a.N[q];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x * blockDim.x > N - 1) return;   // whole block past the instance (uniform)
    const long long nb = a.node_off[q];
    const double* p = a.params + (long long)q * a.n_params;
    const double* y = a.y + nb * M;
    const double* mesh = a.mesh + nb;
    const double* h = a.h + nb;
    double mx = 0.0, sq = 0.0;
    bool bad = false;
    if (i < N - 1) {
        double yi[M], yi1[M], K[S * M], r[M];
        for (int m = 0; m < M; ++m) { yi[m] = y[i * M + m]; yi1[m] = y[(i + 1) * M + m]; }
        phi_large<double, double, double>(yi, yi1, K, r, p, mesh[i], h[i]);
        double* Kg = a.K + (nb + i) * (S * M);
        for (int k = 0; k < S * M; ++k) Kg[k] = K[k];
        double* Fg = a.F + (nb + i) * M;
        JT* yj = a.yj + (nb + i) * M;
        for (int m = 0; m < M; ++m) {
            Fg[m] = r[m];
            bad |= !isfinite(r[m]);
            mx = fmax(mx, fabs(r[m]));
            sq += r[m] * r[m];
            yj[m] = JT(yi[m]);
        }
    } else if (i == N - 1) {
        double ya[M], yb[M], ra[M], rb[M];
        for (int m = 0; m < M; ++m) { ya[m] = y[m]; yb[m] = y[(N - 1) * M + m]; ra[m] = 0.0; rb[m] = 0.0; }
        bvp_bca<double, double>(ra, ya, p);
        bvp_bcb<double, double>(rb, yb, p);
        double* bc = a.bcres + (long long)q * M;
        JT* yj = a.yj + (nb + N - 1) * M;
        for (int k = 0; k < M; ++k) {
            const double v = k < LA ? ra[k] : rb[k - LA];
            bc[k] = v;
            bad |= !isfinite(v);
            mx = fmax(mx, fabs(v));
            sq += v * v;
            yj[k] = JT(yb[k]);
        }
    }
    reduce_norm(a, q, mx, sq, bad);
}

// ---- Jacobian blocks: one warp per run of JG intervals ---------------------------------------
// Forward mode in two parts. (1) J_f at each stage point Y_r, column `lane` on lane `lane`
// (a one-direction dual evaluation of the user's f; the primal stage points come from the
// FP64 stages the residual wrote at the same iterate). With node stages (MIRK4-6: c = v = 0
// and c = v = 1) the right node's J_f is the next interval's left node's, so each node is
// evaluated once per run. (2) The stage chain over the 2M tangent directions, in passes of
// JW directions with lane m owning row m: dY_r = (1 - v_r)[I 0] + v_r [0 I] + h Σ_j x_rj dK_j,
// dK_r = J_r dY_r, and the blocks S_i = -I - h Σ_r b_r dK_r[:, :M], R_i = I - h Σ_r b_r dK_r[:, M:]
// (the derivative of r_i = y_i+1 - y_i - h Σ b_r K_r, collocation.jl:44-72; the reference
// differentiates the same function with ForwardDiff, mirk.jl:824-838).
// The warp after the last run of an instance computes the BC blocks.
extern "C" __global__ void __launch_bounds__(128) bl_jacobian(const BvpLargeArgs a) {
    using namespace bvp;
    extern __shared__ __align__(16) unsigned char bj_smem[];
    const int q = a.active[blockIdx.y];
    const int N = a.N[q];
    const int nI = N - 1;
    const int wpb = int(blockDim.x >> 5);
    const int warp = threadIdx.x >> 5, lane = lane_id();
    const int w = blockIdx.x * wpb + warp;
    const int nruns = (nI + JG - 1) / JG;
    if (blockIdx.x * wpb > nruns) return;   // whole block past the instance and its BC warp
    const long long nb = a.node_off[q];
    // the instance's parameters in shared memory: every warp of the block evaluates f with them
    const JT* pg = a.params_j + (long long)q * a.n_params;
    const bool pstage = a.n_params <= JPMAX;
    JT* ps = reinterpret_cast<JT*>(bj_smem);
    if (pstage)
        for (int k = threadIdx.x; k < a.n_params; k += blockDim.x) ps[k] = pg[k];
    __syncthreads();
    const JT* pj = pstage ? ps : pg;
    if (w > nruns) return;
    const double* y = a.y + nb * M;
    if (w == nruns) {
        // BC blocks: column `lane` of dbca/dy0 (rows 0..La-1) and dbcb/dyN (rows La..M-1)
        if (lane < M) {
            JT* G0 = a.G + (long long)q * 2 * M * M;
            JT* G1 = G0 + M * M;
            using D1 = Dual<JT, 1>;
            {
                D1 u[M], r[M];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    u[m] = D1(JT(y[m]));
                    u[m].d[0] = m == lane ? JT(1) : JT(0);
                    r[m] = D1(JT(0));
                }
                bvp_bca<D1, JT>(r, u, pj);
#pragma unroll
                for (int k = 0; k < M; ++k) G0[k * M + lane] = k < LA ? r[k].d[0] : JT(0);
            }
            {
                D1 u[M], r[M];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    u[m] = D1(JT(y[(long long)(N - 1) * M + m]));
                    u[m].d[0] = m == lane ? JT(1) : JT(0);
                    r[m] = D1(JT(0));
                }
                bvp_bcb<D1, JT>(r, u, pj);
#pragma unroll
                for (int k = 0; k < M; ++k) G1[k * M + lane] = k >= LA ? r[k - LA].d[0] : JT(0);
            }
        }
        return;
    }
    const int pb = pstage ? BVP_B16(a.n_params * int(sizeof(JT))) : 0;
    JT* Jm = reinterpret_cast<JT*>(bj_smem + pb + (size_t)warp * JWARP_BYTES);   // S slots x M x JLD
    JT* Yp = Jm + S * M * JLD;                                                   // S x M
    JT* dY = Yp + S * M;                                                         // M x DYLD
    const double* mesh = a.mesh + nb;
    const double* hh = a.h + nb;
    const double* Kg = a.K + nb * (S * M);
    const int i0 = w * JG;
    const int i1 = min(i0 + JG, nI);
#pragma unroll 1
    for (int i = i0; i < i1; ++i) {
        const int kk = i - i0;
        const double ti = mesh[i], hi = hh[i];
        // primal stage points Y_r = (1 - v_r) y_i + v_r y_i+1 + h Σ_j x_rj K_j
        for (int m = lane; m < M; m += 32) {
            const double yi = y[(long long)i * M + m], yi1 = y[(long long)(i + 1) * M + m];
#pragma unroll
            for (int r = 0; r < S; ++r) {
                double Y = (1.0 - tab_v(r)) * yi + tab_v(r) * yi1;
#pragma unroll
                for (int j = 0; j < r; ++j)
                    if (tab_x(r, j) != 0.0) Y = Y + hi * (Kg[((long long)i * S + j) * M + m] * tab_x(r, j));
                Yp[r * M + m] = JT(Y);
            }
        }
        __syncwarp();
        // J_f at the stage points (the left node's comes with the previous interval of the run)
#pragma unroll
        for (int r = 0; r < S; ++r) {
            if (LNODE && r == 0 && kk > 0) continue;
            if (lane < M) {
                using D1 = Dual<JT, 1>;
                D1 u[M], du[M];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    u[m] = D1(Yp[r * M + m]);
                    u[m].d[0] = m == lane ? JT(1) : JT(0);
                }
                stage_f<D1, JT>(du, u, pj, JT(ti + tab_c(r) * hi));
                JT* Js = Jm + jslot(r, kk) * M * JLD;
#pragma unroll
                for (int m = 0; m < M; ++m) Js[m * JLD + lane] = du[m].d[0];
            }
        }
        __syncwarp();
        // the stage chain, JW directions per pass; lane m owns row m
        const JT hj = JT(hi);
        JT* Sg = a.Sb + (nb + i) * (M * M);
        JT* Rg = a.Rb + (nb + i) * (M * M);
#pragma unroll 1
        for (int p = 0; p < (2 * M + JW - 1) / JW; ++p) {
            JT dK[S][JW];
            JT dR[JW];
#pragma unroll
            for (int c = 0; c < JW; ++c) dR[c] = JT(0);
#pragma unroll
            for (int r = 0; r < S; ++r) {
                const JT* Jr = Jm + jslot(r, kk) * M * JLD;
                bool xfree = true;
#pragma unroll
                for (int j = 0; j < r; ++j) xfree = xfree && tab_x(r, j) == 0.0;
                if (xfree) {
                    // dY_r = (1 - v_r)[I 0] + v_r [0 I]: dK_r is a scaled column of J_r
#pragma unroll
                    for (int c = 0; c < JW; ++c) {
                        const int d = p * JW + c;
                        JT v = JT(0);
                        if (lane < M && d < 2 * M)
                            v = d < M ? JT(1.0 - tab_v(r)) * Jr[lane * JLD + d] : JT(tab_v(r)) * Jr[lane * JLD + d - M];
                        dK[r][c] = v;
                    }
                } else {
                    if (lane < M) {
#pragma unroll
                        for (int c = 0; c < JW; ++c) {
                            const int d = p * JW + c;
                            JT v = JT(0);
                            if (d < M) v = lane == d ? JT(1.0 - tab_v(r)) : JT(0);
                            else if (d < 2 * M) v = lane == d - M ? JT(tab_v(r)) : JT(0);
#pragma unroll
                            for (int j = 0; j < r; ++j)
                                if (tab_x(r, j) != 0.0) v = v + hj * (dK[j][c] * JT(tab_x(r, j)));
                            dY[lane * DYLD + c] = v;
                        }
                    }
                    __syncwarp();
                    JT acc[JW];
#pragma unroll
                    for (int c = 0; c < JW; ++c) acc[c] = JT(0);
                    if (lane < M) {
#pragma unroll 4
                        for (int k = 0; k < M; ++k) {
                            const JT jv = Jr[lane * JLD + k];
#pragma unroll
                            for (int c = 0; c < JW; c += 4) {
                                JT v4[4];
                                ld4(&dY[k * DYLD + c], v4);
#pragma unroll
                                for (int t = 0; t < 4; ++t) acc[c + t] += jv * v4[t];
                            }
                        }
                    }
#pragma unroll
                    for (int c = 0; c < JW; ++c) dK[r][c] = acc[c];
                    __syncwarp();
                }
#pragma unroll
                for (int c = 0; c < JW; ++c) dR[c] += dK[r][c] * JT(tab_b(r));
            }
            if (lane < M) {
#pragma unroll
                for (int c = 0; c < JW; ++c) {
                    const int d = p * JW + c;
                    if (d < M) Sg[lane * M + d] = (lane == d ? JT(-1) : JT(0)) - hj * dR[c];
                    else if (d < 2 * M) Rg[lane * M + d - M] = (lane == d - M ? JT(1) : JT(0)) - hj * dR[c];
                }
            }
        }
    }
}

namespace bvp {

// ---- structured elimination of one node (K3 for the larger-state path) -------------------
// The current relation of a warp, `Rel`, is B δ_mid + A δ_lo = g, stored as the M x (2M+1)
// rows [B | A | g]. A new block row (the next interval, S_c δ_c + R_c δ_c+1 = -F_c, or a
// partner warp's relation) brings Sb δ_mid + Rb δ_hi = gb. Eliminating δ_mid:
//   1. the 2M x M panel [B; Sb] is LU-factorised with row pivoting in registers (lane l owns
//      top row l and bottom row l; the pivot row travels by shuffles);
//   2. the pivot rows' trailing columns (δ_lo | δ_hi | rhs) are solved with the unit lower
//      factor L11 (U12 = L11^-1 T_top, column-parallel: lane c owns column c; the rhs column
//      row-parallel), and the unpivoted rows get the Schur complement T_bot - L21 U12 (lane c
//      again owns column c, L21 rows broadcast from shared memory);
//   3. the pivot rows [U11 | U12] are the elimination record (δ_mid = U11^-1 (g - X δ_lo -
//      Y δ_hi)), the Schur rows the new relation [B'' | A' | g'] on δ_hi (the new δ_mid)
//      and δ_lo.
// This is the block Gaussian elimination with row pivoting the reference's almost-banded LU
// performs, ordered by node (LinearSolve/FastAlmostBandedMatrices, mirk.jl:774-778).

// row strides: >= the row length and = 4 (mod 8), so eight lanes reading eight rows with
// 16-byte loads touch distinct banks
#define BVP_PAD48(n) ((n) % 8 <= 4 ? (n) + (4 - (n) % 8) : (n) + (12 - (n) % 8))
constexpr int RLD = BVP_PAD48(2 * M + 1);  // relation rows [B | A | g]
constexpr int LLD = BVP_PAD48(M);          // panel factor rows
constexpr int DLD = 2 * M + 2;             // dense end system rows
constexpr int WJT = M * RLD + 2 * M * LLD + ((M + 3) / 4) * 4;   // JT elements per warp
constexpr int OFF_IDX = BVP_B16(WJT * int(sizeof(JT)));
constexpr int OFF_RS = OFF_IDX + BVP_B16(2 * M * 4);
constexpr int OFF_FS = OFF_RS + BVP_B16(M * M * int(sizeof(JT)));
constexpr int WARP_BYTES = OFF_FS + BVP_B16(M * 8);
constexpr int DENSE_BYTES = BVP_B16(2 * M * DLD * int(sizeof(JT)));

struct WarpMem {
    JT* rel;     // M x RLD
    JT* lf;      // 2M x LLD: rows 0..M-1 pivot rows (L11 | U11) in pivot order, M..2M-1 L21
    JT* xs;      // M: the rhs column of U12
    int* pidx;   // M: physical row of pivot k (top rows 0..M-1, bottom rows M..2M-1)
    int* qidx;   // M: physical row of unpivoted row u
    JT* rs;      // M x M: the next interval's R block, staged by cp.async
    double* fs;  // M: its residual F
};
BVP_DEV WarpMem warp_mem(unsigned char* base, int w) {
    unsigned char* p = base + (size_t)w * WARP_BYTES;
    WarpMem m;
    m.rel = reinterpret_cast<JT*>(p);
    m.lf = m.rel + M * RLD;
    m.xs = m.lf + 2 * M * LLD;
    m.pidx = reinterpret_cast<int*>(p + OFF_IDX);
    m.qidx = m.pidx + M;
    m.rs = reinterpret_cast<JT*>(p + OFF_RS);
    m.fs = reinterpret_cast<double*>(p + OFF_FS);
    return m;
}

// asynchronous global -> shared copies (cp.async, completed by cp_async_wait_all)
BVP_DEV void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src));
}
BVP_DEV void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src));
}
BVP_DEV void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src));
}
BVP_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
BVP_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// warp-cooperative copy of n bytes (a multiple of 4) in the widest pieces both ends allow
BVP_DEV void warp_stage(void* dst, const void* src, int n) {
    char* d = static_cast<char*>(dst);
    const char* s = static_cast<const char*>(src);
    const unsigned long long al = reinterpret_cast<unsigned long long>(d) | reinterpret_cast<unsigned long long>(s);
    if ((al & 15) == 0 && n % 16 == 0) {
        for (int o = lane_id() * 16; o < n; o += 32 * 16) cp_async16(d + o, s + o);
    } else if ((al & 7) == 0 && n % 8 == 0) {
        for (int o = lane_id() * 8; o < n; o += 32 * 8) cp_async8(d + o, s + o);
    } else {
        for (int o = lane_id() * 4; o < n; o += 32 * 4) cp_async4(d + o, s + o);
    }
}

// bottom block row: the next interval (R block and F staged in shared memory; the S block's
// rows come in registers from the caller)
struct BotInterval {
    const JT* rs;
    const double* fs;
    BVP_DEV JT hi(int u, int c) const { return rs[u * M + c]; }
    BVP_DEV JT rhs(int u) const { return JT(-fs[u]); }
    BVP_DEV void wait() const {
        cp_async_wait_all();
        __syncwarp();
    }
};
// bottom block row: a partner warp's relation [B2 | A2 | g2], whose δ_lo is the shared node
struct BotRel {
    const JT* rl;
    BVP_DEV JT panel(int u, int j) const { return rl[u * RLD + M + j]; }
    BVP_DEV JT hi(int u, int c) const { return rl[u * RLD + c]; }
    BVP_DEV JT rhs(int u) const { return rl[u * RLD + 2 * M]; }
    BVP_DEV void wait() const {}
};
struct NoPrefetch {
    BVP_DEV void operator()() const {}
};

// pivot candidate: |x| for rows still unpivoted (NaN ranks first, so it is chosen and fails
// the finiteness test), -1 for pivoted or absent rows
BVP_DEV JT pivot_cand(JT x, bool live) {
    if (!live) return JT(-1);
    const JT v = fabs(x);
    return v == v ? v : JT(__longlong_as_double(0x7ff0000000000000LL));
}


// a register row of M values to global memory (16-byte stores when aligned)
BVP_DEV void store_row(JT* dst, const JT (&x)[M]) {
    if constexpr (sizeof(JT) == 4 && M % 4 == 0) {
        if ((reinterpret_cast<unsigned long long>(dst) & 15) == 0) {
#pragma unroll
            for (int k = 0; k < M; k += 4)
                *reinterpret_cast<float4*>(dst + k) = make_float4(x[k], x[k + 1], x[k + 2], x[k + 3]);
            return;
        }
    }
#pragma unroll
    for (int k = 0; k < M; ++k) dst[k] = x[k];
}

// a1: the bottom block's panel row `lane` (in registers, from the caller). `pre` runs once
// the panel is factorised (the caller's prefetch of the next panel rows); bot.wait() makes
// the staged bottom block visible before its first use.
template <class Bot, class Pre>
BVP_DEV bool warp_eliminate(const WarpMem& wm, JT (&a1)[M], const Bot& bot, JT* rec, const Pre& pre) {
    constexpr int M4 = ((M + 3) / 4) * 4;
    const int lane = lane_id();
    const bool act = lane < M;
    JT* Rel = wm.rel;
    JT* Lf = wm.lf;
    // 1. panel rows in registers: top row `lane` = B, bottom row `lane` = the new block's
    JT a0[M];
#pragma unroll
    for (int j = 0; j < M; ++j) a0[j] = act ? Rel[lane * RLD + j] : JT(0);
    int st0 = act ? -1 : M, st1 = act ? -1 : M;   // pivot step of each row; -1 while unpivoted
    bool ok = true;
#pragma unroll
    for (int k = 0; k < M; ++k) {
        // pivot: largest |entry| in column k among unpivoted rows, ties to the lower row id
        JT v = pivot_cand(a0[k], st0 < 0);
        int pr = lane;
        const JT v1 = pivot_cand(a1[k], st1 < 0);
        if (v1 > v) { v = v1; pr = M + lane; }
        if constexpr (sizeof(JT) == 4) {
            // one warp reduction on (|v| with its 6 lowest mantissa bits replaced by 63 - row,
            // offset by 64 so that every live row outranks the pivoted ones, whose key is 0):
            // the float bits of a non-negative value order like the value, so this selects the
            // largest magnitude to 17 bits, ties (within 2^-17) to the lower row
            const unsigned key = v < JT(0) ? 0u : (((__float_as_uint(v) & ~63u) + 64u) | unsigned(63 - pr));
            const unsigned best = __reduce_max_sync(FULL, key);
            pr = 63 - int(best & 63u);
            v = __uint_as_float((best & ~63u) - 64u);
        } else {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const JT v2 = __shfl_xor_sync(FULL, v, o);
                const int p2 = __shfl_xor_sync(FULL, pr, o);
                if (v2 > v || (v2 == v && p2 < pr)) { v = v2; pr = p2; }
            }
        }
        ok = ok && v > JT(0) && isfinite(v);
        pr = pr < 2 * M ? pr : 2 * M - 1;   // always holds (a live row exists at every step)
        const bool pbot = pr >= M;
        const int own = pbot ? pr - M : pr;
        JT prow[M];
#pragma unroll
        for (int j = k; j < M; ++j) prow[j] = __shfl_sync(FULL, pbot ? a1[j] : a0[j], own);
        if (lane == own) { if (pbot) st1 = k; else st0 = k; }
        if (lane == 0) wm.pidx[k] = pr;
        const JT inv = rcp_rn(prow[k]);
        // branch-free update: pivoted rows take a zero multiplier
        const JT m0 = st0 < 0 ? a0[k] * inv : JT(0);
        const JT m1 = st1 < 0 ? a1[k] * inv : JT(0);
        a0[k] = st0 < 0 ? m0 : a0[k];
        a1[k] = st1 < 0 ? m1 : a1[k];
#pragma unroll
        for (int j = k + 1; j < M; ++j) {
            a0[j] -= m0 * prow[j];
            a1[j] -= m1 * prow[j];
        }
    }
    // 2. factor rows to shared memory: pivot rows by step, unpivoted rows compacted
    //    (top rows first, by lane, then bottom rows)
    const unsigned b0 = __ballot_sync(FULL, st0 < 0);
    const unsigned b1 = __ballot_sync(FULL, st1 < 0);
    const unsigned lt = (1u << lane) - 1u;
    {
        const int r0 = st0 >= 0 ? st0 : M + __popc(b0 & lt);
        const int r1 = st1 >= 0 ? st1 : M + __popc(b0) + __popc(b1 & lt);
        if (act) {
#pragma unroll
            for (int j = 0; j < M; ++j) { Lf[r0 * LLD + j] = a0[j]; Lf[r1 * LLD + j] = a1[j]; }
            if (st0 < 0) wm.qidx[r0 - M] = lane;
            if (st1 < 0) wm.qidx[r1 - M] = M + lane;
        }
    }
    pre();
    bot.wait();
    __syncwarp();
    // 3. U11 into the record, transposed (UT[j][k] = U[k][j]): each pivot row's owner writes
    //    its row as a column (the entries below the diagonal are multipliers, never read)
#pragma unroll
    for (int j = 0; j < M; ++j) {
        if (act && st0 >= 0) rec[j * M + st0] = a0[j];
        if (act && st1 >= 0) rec[j * M + st1] = a1[j];
    }
    // 4. rhs column: forward substitution row-parallel (lane k owns pivot row k), then the
    //    Schur rows (lane u owns unpivoted row u)
    {
        JT xr = JT(0);
        JT Lk[M4];
        if (act) {
            const int p = wm.pidx[lane];
            xr = p < M ? Rel[p * RLD + 2 * M] : bot.rhs(p - M);
#pragma unroll
            for (int j = 0; j < M4; j += 4) ld4(&Lf[lane * LLD + j], &Lk[j]);
        }
#pragma unroll
        for (int j = 0; j < M - 1; ++j) {
            const JT xj = __shfl_sync(FULL, xr, j);
            if (lane > j && act) xr -= Lk[j] * xj;
        }
        if (act) {
            rec[3 * M * M + lane] = xr;
            wm.xs[lane] = xr;
        }
        __syncwarp();
        JT sr = JT(0);
        if (act) {
            const int qq = wm.qidx[lane];
            sr = qq < M ? Rel[qq * RLD + 2 * M] : bot.rhs(qq - M);
#pragma unroll
            for (int j = 0; j < M4; j += 4) {
                JT l4[4], x4[4];
                ld4(&Lf[(M + lane) * LLD + j], l4);
                ld4(&wm.xs[j], x4);
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    if (j + t < M) sr -= l4[t] * x4[t];
            }
        }
        __syncwarp();
        if (act) Rel[lane * RLD + 2 * M] = sr;
    }
    // 5. the δ_lo and δ_hi columns: lane c owns column c (two passes when M > 16)
    // T entry of column c in physical row p, read branch-free from clamped (always valid)
    // addresses: top rows carry the δ_lo coefficients, bottom rows the δ_hi ones
    auto tval = [&](int c, int p) {
        const bool cv = c < 2 * M, lo = c < M;
        const JT tv = Rel[(p < M ? p : 0) * RLD + M + (lo ? c : 0)];
        const JT bv = bot.hi(p < M ? 0 : p - M, (cv && !lo) ? c - M : 0);
        return cv ? (p < M ? (lo ? tv : JT(0)) : (lo ? JT(0) : bv)) : JT(0);
    };
    // column c of U12 = L11^-1 T_top (forward substitution in pivot order)
    auto fwd_col = [&](int c, JT (&x)[M]) {
#pragma unroll
        for (int k = 0; k < M; ++k) {
            JT t = tval(c, wm.pidx[k]);
#pragma unroll
            for (int j = 0; j < k; j += 4) {
                JT l4[4];
                ld4(&Lf[k * LLD + j], l4);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (j + q < k) t -= l4[q] * x[j + q];
            }
            x[k] = t;
        }
    };
    if constexpr (!MMA_SCHUR) {
#pragma unroll 1
        for (int s = 0; s < (2 * M + 31) / 32; ++s) {
            const int c = lane + 32 * s;
            JT x[M];
            fwd_col(c, x);
            JT sc[M];
#pragma unroll
            for (int u = 0; u < M; ++u) {
                JT t = tval(c, wm.qidx[u]);
#pragma unroll
                for (int j = 0; j < M4; j += 4) {
                    JT l4[4];
                    ld4(&Lf[(M + u) * LLD + j], l4);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (j + q < M) t -= l4[q] * x[j + q];
                }
                sc[u] = t;
            }
            __syncwarp();
            if (c < 2 * M) {
                // column c of U12 is row c of XT (δ_lo) or row c - M of YT (δ_hi)
                store_row(rec + (c < M ? M * M + c * M : 2 * M * M + (c - M) * M), x);
                const int dc = c < M ? M + c : c - M;
#pragma unroll
                for (int u = 0; u < M; ++u) Rel[u * RLD + dc] = sc[u];
            }
            __syncwarp();
        }
    } else {
        // M = 32, FP32: the forward substitutions as above, then the Schur update
        // T_bot - L21 U12 (32 x 64 x 32) on the tensor cores, mma.sync m16n8k8 TF32 with each
        // operand split into a TF32 head and tail (three products: near-FP32 accuracy),
        // 32 columns at a time with U12 staged (transposed) in the dead L11 rows of Lf
        JT xh[2][M];
        fwd_col(lane, xh[0]);
        fwd_col(lane + 32, xh[1]);
        store_row(rec + M * M + lane * M, xh[0]);        // XT row `lane`
        store_row(rec + 2 * M * M + lane * M, xh[1]);    // YT row `lane`
        __syncwarp();                                    // L11 is read no more
        const int g = lane >> 2, tg = lane & 3;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            {
                JT* row = Lf + lane * LLD;               // U12 column 32h + lane as a row
#pragma unroll
                for (int k = 0; k < M; k += 4) st4(row + k, xh[h], k);
            }
            __syncwarp();
            float d[2][4][4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int r8 = 0; r8 < 2; ++r8) {
                    const int qq = wm.qidx[16 * mt + g + 8 * r8];
#pragma unroll
                    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                        for (int e = 0; e < 2; ++e) d[mt][nt][2 * r8 + e] = tval(32 * h + 8 * nt + 2 * tg + e, qq);
                }
#pragma unroll
            for (int kt = 0; kt < M / 8; ++kt) {
                unsigned ah[2][4], al[2][4];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    const JT* L0 = Lf + (M + 16 * mt + g) * LLD + 8 * kt + tg;
                    tf32_split(-L0[0], ah[mt][0], al[mt][0]);
                    tf32_split(-L0[8 * LLD], ah[mt][1], al[mt][1]);
                    tf32_split(-L0[4], ah[mt][2], al[mt][2]);
                    tf32_split(-L0[8 * LLD + 4], ah[mt][3], al[mt][3]);
                }
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const JT* B = Lf + (8 * nt + g) * LLD + 8 * kt + tg;
                    unsigned bh[2], bl[2];
                    tf32_split(B[0], bh[0], bl[0]);
                    tf32_split(B[4], bh[1], bl[1]);
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt) {
                        mma_tf32(d[mt][nt], al[mt], bh);
                        mma_tf32(d[mt][nt], ah[mt], bl);
                        mma_tf32(d[mt][nt], ah[mt], bh);
                    }
                }
            }
            __syncwarp();                                // T reads and tile reads done
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int r8 = 0; r8 < 2; ++r8)
#pragma unroll
                    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                        for (int e = 0; e < 2; ++e) {
                            const int u = 16 * mt + g + 8 * r8;
                            const int c = 32 * h + 8 * nt + 2 * tg + e;
                            Rel[u * RLD + (c < M ? M + c : c - M)] = d[mt][nt][2 * r8 + e];
                        }
            __syncwarp();
        }
    }
    return ok;
}

// x = U^{-1} (g - X lo - Y hi) from an elimination record [UT | XT | YT | g] (blocks stored
// transposed, so lane r's reads of row r are coalesced across the warp); lane c holds lo[c]
// and hi[c] on entry, lane r returns x[r]
BVP_DEV JT warp_back_solve(const JT* rg, JT lo_l, JT hi_l) {
    const int lane = lane_id();
    const bool act = lane < M;
    const int l = act ? lane : 0;
    JT t = rg[3 * M * M + l];
#pragma unroll
    for (int c = 0; c < M; ++c) {
        const JT loc = __shfl_sync(FULL, lo_l, c);
        const JT hic = __shfl_sync(FULL, hi_l, c);
        t -= rg[M * M + c * M + l] * loc + rg[2 * M * M + c * M + l] * hic;
    }
    const JT inv = rcp_rn(rg[l * M + l]);
#pragma unroll
    for (int r = M - 1; r >= 0; --r) {
        const JT xr = __shfl_sync(FULL, t * inv, r);
        const JT ur = rg[r * M + l];   // U[lane][r]
        t = lane == r ? xr : (lane < r ? t - ur * xr : t);
    }
    return act ? t : JT(0);
}


}  // namespace bvp

// ---- linear solve: one CTA per active instance ----------------------------------------------
// Dynamic shared memory: WARP_BYTES per warp (relation, panel factors, indices) and the
// dense end system (DENSE_BYTES).
extern "C" __global__ void __launch_bounds__(256) bl_linsolve(const BvpLargeArgs a) {
    using namespace bvp;
    extern __shared__ __align__(16) unsigned char bl_smem[];
    __shared__ int s_lo[8], s_hi[8];
    __shared__ int s_bad;
    const int q = a.active[blockIdx.x];
    const int N = a.N[q];
    const int nI = N - 1;
    const int warp = threadIdx.x >> 5, lane = lane_id();
    const int NWl = int(blockDim.x >> 5);
    const int NW = nI < NWl ? nI : NWl;             // warps with a chunk
    const long long nb = a.node_off[q];
    const WarpMem wm = warp_mem(bl_smem, warp);
    const JT* Sb = a.Sb + nb * (M * M);
    const JT* Rb = a.Rb + nb * (M * M);
    const double* F = a.F + nb * M;
    JT* rec = a.rec + nb * RECW;
    JT* dl = a.delta + nb * M;
    if (threadIdx.x == 0) s_bad = 0;
    bool ok = true;
    // 1. chunk eliminations: warp w owns intervals [c0, c1)
    int c0 = 0, c1 = 0;
    if (warp < NW) {
        c0 = (warp * nI) / NW;
        c1 = ((warp + 1) * nI) / NW;
        // relation of interval c0: S δ_c0 + R δ_c0+1 = -F as [R | S | -F] (δ_mid = δ_c0+1)
        for (int e = lane; e < M * M; e += 32) {
            const int r = e / M, c = e % M;
            wm.rel[r * RLD + c] = Rb[(long long)c0 * M * M + e];
            wm.rel[r * RLD + M + c] = Sb[(long long)c0 * M * M + e];
        }
        for (int r = lane; r < M; r += 32) wm.rel[r * RLD + 2 * M] = JT(-F[(long long)c0 * M + r]);
        __syncwarp();
        // the next interval's S block rows, one interval ahead of the elimination
        const bool act = lane < M;
        JT sp[M];
        auto load_s = [&](int c) {
            const JT* S = Sb + (long long)c * M * M + lane * M;
#pragma unroll
            for (int j = 0; j < M; ++j) sp[j] = act ? S[j] : JT(0);
        };
        if (c0 + 1 < c1) load_s(c0 + 1);
#pragma unroll 1
        for (int c = c0 + 1; c < c1; ++c) {
            warp_stage(wm.rs, Rb + (long long)c * M * M, M * M * int(sizeof(JT)));
            warp_stage(wm.fs, F + (long long)c * M, M * 8);
            cp_async_commit();
            JT a1[M];
#pragma unroll
            for (int j = 0; j < M; ++j) a1[j] = sp[j];
            const BotInterval bot{wm.rs, wm.fs};
            ok &= warp_eliminate(wm, a1, bot, rec + (long long)c * RECW, [&]() {
                if (c + 1 < c1) load_s(c + 1);
            });
        }
        if (lane == 0) { s_lo[warp] = c0; s_hi[warp] = c1; }
    }
    __syncthreads();
    // 2. combine chunk relations pairwise: warp w (multiple of 2s) eliminates the node it shares
    //    with warp w + s; its relation then spans both chunks
    for (int s = 1; s < NW; s <<= 1) {
        if (warp < NW && (warp % (2 * s)) == 0 && warp + s < NW) {
            const BotRel bot{warp_mem(bl_smem, warp + s).rel};
            JT a1[M];
#pragma unroll
            for (int j = 0; j < M; ++j) a1[j] = lane < M ? bot.panel(lane, j) : JT(0);
            ok &= warp_eliminate(wm, a1, bot, rec + (long long)s_hi[warp] * RECW, NoPrefetch{});
            if (lane == 0) s_hi[warp] = s_hi[warp + s];
        }
        __syncthreads();
    }
    // 3. warp 0: [dbca/dy0 rows | relation | dbcb/dyN rows] in δ_0, δ_N-1 (2M x 2M); the
    //    relation is [B | A | g] with A on δ_0 and B on δ_N-1
    if (warp == 0) {
        JT* Wd = reinterpret_cast<JT*>(bl_smem + (size_t)NWl * WARP_BYTES);
        const JT* G0 = a.G + (long long)q * 2 * M * M;
        const JT* G1 = G0 + M * M;
        const double* bc = a.bcres + (long long)q * M;
        const JT* Rl = wm.rel;
        for (int e = lane; e < LA * (2 * M + 1); e += 32) {
            const int r = e / (2 * M + 1), c = e % (2 * M + 1);
            Wd[r * DLD + c] = c < M ? G0[r * M + c] : (c < 2 * M ? JT(0) : JT(-bc[r]));
        }
        for (int e = lane; e < M * (2 * M + 1); e += 32) {
            const int r = e / (2 * M + 1), c = e % (2 * M + 1);
            Wd[(LA + r) * DLD + c] = c < M ? Rl[r * RLD + M + c] : (c < 2 * M ? Rl[r * RLD + c - M] : Rl[r * RLD + 2 * M]);
        }
        for (int e = lane; e < (M - LA) * (2 * M + 1); e += 32) {
            const int r = LA + e / (2 * M + 1), c = e % (2 * M + 1);
            Wd[(M + r) * DLD + c] = c < M ? JT(0) : (c < 2 * M ? G1[r * M + c - M] : JT(-bc[r]));
        }
        __syncwarp();
        // dense elimination with pivoting on all 2M columns, then back substitution
        bool dok = true;
        for (int k = 0; k < 2 * M; ++k) {
            JT v = JT(-1);
            int pr = 0x7fffffff;
#pragma unroll
            for (int h2 = 0; h2 < 2; ++h2) {
                const int r = lane + 32 * h2;
                if (r >= k && r < 2 * M) {
                    const JT av = pivot_cand(Wd[r * DLD + k], true);
                    if (av > v) { v = av; pr = r; }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const JT v2 = __shfl_xor_sync(FULL, v, o);
                const int p2 = __shfl_xor_sync(FULL, pr, o);
                if (v2 > v || (v2 == v && p2 < pr)) { v = v2; pr = p2; }
            }
            dok = dok && v > JT(0) && isfinite(v);
            if (pr != k && pr < 2 * M) {
                for (int c = lane; c <= 2 * M; c += 32) {
                    const JT tmp = Wd[k * DLD + c];
                    Wd[k * DLD + c] = Wd[pr * DLD + c];
                    Wd[pr * DLD + c] = tmp;
                }
            }
            __syncwarp();
            const JT inv = JT(1) / Wd[k * DLD + k];
#pragma unroll
            for (int h2 = 0; h2 < 2; ++h2) {
                const int r = lane + 32 * h2;
                if (r > k && r < 2 * M) {
                    const JT mlt = Wd[r * DLD + k] * inv;
                    for (int c = k; c <= 2 * M; ++c) Wd[r * DLD + c] -= mlt * Wd[k * DLD + c];
                }
            }
            __syncwarp();
        }
        for (int k = 2 * M - 1; k >= 0; --k) {
            if (lane == 0) Wd[k * DLD + 2 * M] = Wd[k * DLD + 2 * M] / Wd[k * DLD + k];
            __syncwarp();
            for (int r = lane; r < k; r += 32) Wd[r * DLD + 2 * M] -= Wd[r * DLD + k] * Wd[k * DLD + 2 * M];
            __syncwarp();
        }
        for (int m = lane; m < M; m += 32) {
            dl[m] = Wd[m * DLD + 2 * M];
            dl[(long long)(N - 1) * M + m] = Wd[(M + m) * DLD + 2 * M];
        }
        ok &= dok;
    }
    __syncthreads();
    // 4. unwind the pairwise combination: the eliminated chunk-end nodes, coarse to fine
    int top = 1;
    while (top < NW) top <<= 1;
    for (int s = top >> 1; s >= 1; s >>= 1) {
        if (warp < NW && (warp % (2 * s)) == 0 && warp + s < NW) {
            const int lo = s_lo[warp];
            const int mid = s_lo[warp + s];
            const int hi = s_hi[warp + s];
            const JT lo_l = lane < M ? dl[(long long)lo * M + lane] : JT(0);
            const JT hi_l = lane < M ? dl[(long long)hi * M + lane] : JT(0);
            const JT x = warp_back_solve(rec + (long long)mid * RECW, lo_l, hi_l);
            if (lane < M) dl[(long long)mid * M + lane] = x;
            __syncwarp();
        }
        __syncthreads();
    }
    // 5. back substitution inside each chunk (the chunk ends are known)
    if (warp < NW) {
        const JT lo_l = lane < M ? dl[(long long)c0 * M + lane] : JT(0);
        JT hi_l = lane < M ? dl[(long long)c1 * M + lane] : JT(0);
#pragma unroll 1
        for (int c = c1 - 1; c > c0; --c) {
            hi_l = warp_back_solve(rec + (long long)c * RECW, lo_l, hi_l);
            if (lane < M) dl[(long long)c * M + lane] = hi_l;
        }
    }
    if (!ok && lane == 0) atomicExch(&s_bad, 1);
    __syncthreads();
    if (threadIdx.x == 0) a.bad[q] = s_bad;
}

// ---- y += delta, or y = ybase + alpha delta (the line search's trial) -------------------
extern "C" __global__ void bl_update(const BvpLargeArgs a) {
    using namespace bvp;
    const int q = a.active[blockIdx.y];
    const int N = a.N[q];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N * M) return;
    const long long o = a.node_off[q] * M + k;
    if (a.alpha == 0.0) a.y[o] = a.y[o] + double(a.delta[o]);
    else a.y[o] = a.ybase[o] + a.alpha * double(a.delta[o]);
}

// ---- copies within the iterate buffers: mode 0 ybase = y, 1 y = ybase, 2 y = 0,
//      3 ybak = y (Newton's restart copy), 4 y = ybak ----------------------------------------
extern "C" __global__ void bl_copy(const BvpLargeArgs a, int mode) {
    using namespace bvp;
    const int q = a.active[blockIdx.y];
    const int N = a.N[q];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N * M) return;
    const long long o = a.node_off[q] * M + k;
    if (mode == 0) a.ybase[o] = a.y[o];
    else if (mode == 1) a.y[o] = a.ybase[o];
    else if (mode == 2) a.y[o] = 0.0;
    else if (mode == 3) a.ybak[o] = a.y[o];
    else a.y[o] = a.ybak[o];
}

// ---- defect (adaptivity.jl:416-461): threads over intervals ----------------------------------
extern "C" __global__ void __launch_bounds__(128) bl_defect(const BvpLargeArgs a) {
    using namespace bvp;
    const int q = a.active[blockIdx.y];
    const int N = a.N[q];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x * blockDim.x >= N - 1) return;
    double ei = 0.0;
    bool bad = false;
    if (i < N - 1) {
        const long long nb = a.node_off[q];
        const double* p = a.params + (long long)q * a.n_params;
        const double* y = a.y + nb * M;
        const double ti = a.mesh[nb + i], hi = a.h[nb + i];
        double yi[M], yi1[M], K[S * M], KI[NSXA * M];
        for (int m = 0; m < M; ++m) { yi[m] = y[i * M + m]; yi1[m] = y[(i + 1) * M + m]; }
        const double* Kg = a.K + (nb + i) * (S * M);
        for (int k = 0; k < S * M; ++k) K[k] = Kg[k];
        interp_large(yi, yi1, K, KI, p, ti, hi);
        double* KIg = a.KI + (nb + i) * (NSXA * M);
        for (int k = 0; k < NSX * M; ++k) KIg[k] = KI[k];
        double w[2][SS], wp[2][SS];
        interp_weights<double>(tau_star(), w[0], wp[0]);
        interp_weights<double>(1.0 - tau_star(), w[1], wp[1]);
        double est[2];
        for (int smp = 0; smp < 2; ++smp) {
            double z[M], zp[M], fz[M];
            for (int m = 0; m < M; ++m) {
                double acc = K[m] * w[smp][0];
                for (int r = 1; r < S; ++r) acc = acc + K[r * M + m] * w[smp][r];
                for (int qq = 0; qq < NSX; ++qq) acc = acc + KI[qq * M + m] * w[smp][S + qq];
                z[m] = acc * hi + yi[m];
                double accp = K[m] * wp[smp][0];
                for (int r = 1; r < S; ++r) accp += K[r * M + m] * wp[smp][r];
                for (int qq = 0; qq < NSX; ++qq) accp += KI[qq * M + m] * wp[smp][S + qq];
                zp[m] = accp;
            }
            bvp_f<double, double>(fz, z, p, ti + (smp ? 1.0 - tau_star() : tau_star()) * hi);
            double e = 0.0;
            for (int m = 0; m < M; ++m) e = fmax(e, fabs((zp[m] - fz[m]) / (fabs(fz[m]) + 1.0)));
            est[smp] = e;
        }
        ei = est[0] > est[1] ? est[0] : est[1];
        a.err[nb + i] = ei;
        bad = isnan(ei);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ei = fmax(ei, __shfl_xor_sync(FULL, ei, o));
        bad |= __shfl_xor_sync(FULL, int(bad), o) != 0;
    }
    if (lane_id() == 0) {
        if (bad) ei = __longlong_as_double(0x7ff0000000000000LL);
        atomicMax(&a.dnorm[q], norm_bits(ei));
    }
}

// ---- transfer (adaptivity.jl:6-13 from mirk.jl:366-371): one warp per instance -------------
// The new mesh is in buffer 1 (a.newN[q] points); the guess on it comes from the old
// interpolant (buffer 0, K, KI); with transfer_inplace node j reads the already updated
// value of node i_old < j as the reference's in-place update does. The new mesh, spacings
// and guess are then copied into buffer 0.
extern "C" __global__ void bl_transfer(const BvpLargeArgs a) {
    using namespace bvp;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= a.n_active) return;
    const int lane = lane_id();
    const int q = a.active[w];
    const int No = a.N[q], Nn = a.newN[q];
    const long long nb = a.node_off[q];
    const double* om = a.mesh + nb;
    const double* oh = a.h + nb;
    const double* oy = a.y + nb * M;
    double* nm = a.mesh + a.tot + nb;
    double* nh = a.h + a.tot + nb;
    double* ny = a.y + (a.tot + nb) * M;
    double* inc = a.inc + nb * M;
    int* io = a.iold + nb;
    for (int j = lane; j < Nn; j += 32) {
        const double t = nm[j];
        int lo = 0, hi = No;
        while (lo < hi) { const int mid = (lo + hi) >> 1; if (om[mid] < t) lo = mid + 1; else hi = mid; }
        int i = lo - 1;
        i = i < 0 ? 0 : (i > No - 2 ? No - 2 : i);
        const double dt = oh[i];
        double wv[SS], wpv[SS];
        interp_weights<double>((t - om[i]) / dt, wv, wpv);
        const double* Kg = a.K + (nb + i) * (S * M);
        const double* KIg = a.KI + (nb + i) * (NSXA * M);
        for (int m = 0; m < M; ++m) {
            double acc = Kg[m] * wv[0];
            for (int r = 1; r < S; ++r) acc += Kg[r * M + m] * wv[r];
            for (int qq = 0; qq < NSX; ++qq) acc += KIg[qq * M + m] * wv[S + qq];
            inc[(long long)j * M + m] = acc * dt;
            if (!a.transfer_inplace) ny[(long long)j * M + m] = acc * dt + oy[(long long)i * M + m];
        }
        io[j] = i;
    }
    __syncwarp();
    if (a.transfer_inplace) {
        for (int j = 0; j < Nn; ++j) {
            const int i = io[j];
            for (int m = lane; m < M; m += 32) {
                const double base = (i < j) ? ny[(long long)i * M + m] : oy[(long long)i * M + m];
                ny[(long long)j * M + m] = inc[(long long)j * M + m] + base;
            }
            __syncwarp();
        }
    }
    double* m0 = a.mesh + nb;
    double* h0 = a.h + nb;
    double* y0 = a.y + nb * M;
    for (int k = lane; k < Nn; k += 32) { m0[k] = nm[k]; if (k < Nn - 1) h0[k] = nh[k]; }
    for (int k = lane; k < Nn * M; k += 32) y0[k] = ny[k];
}

// ---- dense output u(t) / u'(t) from the final mesh, solution and stages (interpolation.jl:17-206):
//      one warp per instance, lanes over the query times -------------------------------------
extern "C" __global__ void bl_dense(const BvpLargeArgs a, int nq, const double* tq, int deriv, double* out) {
    using namespace bvp;
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (q >= a.n_inst) return;
    const int N = a.N[q];
    const long long nb = a.node_off[q];
    const double* mesh = a.mesh + nb;
    const double* y = a.y + nb * M;
    for (int j = lane_id(); j < nq; j += 32) {
        const double t = tq[(long long)q * nq + j];
        // EvalSol's interval rule (interpolation.jl:214-242, Core/src/utils.jl:119-121)
        int lo = 0, hi = N;
        while (lo < hi) { const int mid = (lo + hi) >> 1; if (mesh[mid] < t) lo = mid + 1; else hi = mid; }
        int i = lo - 1;
        i = i < 0 ? 0 : (i > N - 2 ? N - 2 : i);
        const double dt = a.h[nb + i];
        double w[SS], wp[SS];
        interp_weights<double>((t - mesh[i]) / dt, w, wp);
        const double* wv = deriv ? wp : w;
        const double* Kg = a.K + (nb + i) * (S * M);
        const double* KIg = a.KI + (nb + i) * (NSXA * M);
        double* o = out + ((long long)q * nq + j) * M;
        for (int m = 0; m < M; ++m) {
            double acc = Kg[m] * wv[0];
            for (int r = 1; r < S; ++r) acc += Kg[r * M + m] * wv[r];
            for (int qq = 0; qq < NSX; ++qq) acc += KIg[qq * M + m] * wv[S + qq];
            o[m] = deriv ? acc : acc * dt + y[(long long)i * M + m];
        }
    }
}

// ---- initial meshes, spacings and guesses from one packed upload into the arena ----------------
extern "C" __global__ void bl_scatter(const BvpLargeArgs a, const double* pm, const double* ph, const double* py,
                                      const long long* poff) {
    using namespace bvp;
    const int q = blockIdx.y;
    const long long p0 = poff[q];
    const int N = int(poff[q + 1] - p0);
    const long long nb = a.node_off[q];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N * M; k += gridDim.x * blockDim.x) {
        a.y[nb * M + k] = py[p0 * M + k];
        if (k < N) a.mesh[nb + k] = pm[p0 + k];
        if (k < N - 1) a.h[nb + k] = ph[p0 + k];
    }
}

extern "C" __global__ void bl_convert_params(const double* p, bvp::JT* pj, long long n) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        pj[k] = bvp::JT(p[k]);
}

extern "C" __global__ void bl_layout_probe(int* out) {
    out[0] = int(sizeof(BvpLargeArgs));
    out[1] = bvp::RECW;
    out[2] = bvp::WARP_BYTES;
    out[3] = bvp::JWARP_BYTES;
    out[7] = bvp::JPMAX;
    out[4] = bvp::S;
    out[5] = bvp::NSXA;
    out[6] = bvp::DENSE_BYTES;
}
