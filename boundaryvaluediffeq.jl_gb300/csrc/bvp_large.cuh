// Batched adaptive MIRK for larger state dimensions (9 <= M <= 32) on sm_103a: device code.
//
// NVRTC compiles this file instead of bvp_kernels.cuh when the problem's state dimension is
// above what one warp keeps in registers. The algorithm is the same (the reference's MIRK
// solve: collocation.jl:44-72, mirk.jl:286-388, adaptivity.jl:6-75, 250-461); the work is
// laid out differently:
//   bl_residual  one thread per (instance, interval): FP64 stages and collocation residual,
//                the BC rows on the instance's last thread; max |F| and sum F^2 per instance
//   bl_jacobian  one thread per (instance, interval, 8 tangent directions): the blocks
//                S_i = dr_i/dy_i, R_i = dr_i/dy_{i+1} by forward mode in BVP_JT, and the BC
//                blocks
//   bl_linsolve  one CTA per instance: each warp eliminates a chunk of intervals in shared
//                memory (Gaussian elimination with row pivoting on the 2M x M column block,
//                the warp owning two rows per lane), the chunk relations are combined
//                pairwise, a 2M x 2M system with the BC rows gives the end values, and the
//                warps back-substitute their chunks
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
constexpr int D = 2 * M;
constexpr int LA = BVP_LA;
using JT = BVP_JT;
constexpr int NCH = 8;                        // tangent directions per Jacobian thread
constexpr int NCHUNK = (D + NCH - 1) / NCH;   // thread slots per interval
constexpr int NCHB = (M + NCH - 1) / NCH;     // thread slots of the BC Jacobian
constexpr int RECW = 3 * M * M + M;
constexpr int WR = 2 * M;                     // elimination workspace rows
constexpr int WC = 3 * M + 1;                 // columns: δ_mid | δ_lo | δ_hi | rhs
constexpr int WLD = WC + (WC % 2 == 0 ? 1 : 0);   // odd row stride: conflict-free columns
static_assert(M <= 32 && M > 0, "M <= 32");

BVP_DEV int lane_id() { return threadIdx.x & 31; }
BVP_DEV unsigned long long norm_bits(double v) { return (unsigned long long)__double_as_longlong(v); }

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
        bvp_f<T, PT>(&K[rr * M], Y, p, PT(ti + TT(tab_c(rr)) * hi_t));
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

// ---- Jacobian blocks: threads over (interval, 8 tangent directions) ----------------------
extern "C" __global__ void __launch_bounds__(128) bl_jacobian(const BvpLargeArgs a) {
    using namespace bvp;
    using DC = Dual<JT, NCH>;
    const int q = a.active[blockIdx.y];
    const int N = a.N[q];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / NCHUNK, ch = t % NCHUNK;
    if (i > N - 1) return;
    const long long nb = a.node_off[q];
    const JT* pj = a.params_j + (long long)q * a.n_params;
    const JT* yj = a.yj + nb * M;
    if (i < N - 1) {
        DC yi[M], yi1[M], K[S * M], r[M];
        for (int m = 0; m < M; ++m) { yi[m] = DC(yj[i * M + m]); yi1[m] = DC(yj[(i + 1) * M + m]); }
#pragma unroll
        for (int d = 0; d < NCH; ++d) {
            const int g = ch * NCH + d;
            if (g < M) yi[g].d[d] = JT(1);
            else if (g < D) yi1[g - M].d[d] = JT(1);
        }
        phi_large<DC, JT, JT>(yi, yi1, K, r, pj, JT(a.mesh[nb + i]), JT(a.h[nb + i]));
        JT* Sg = a.Sb + (nb + i) * (M * M);
        JT* Rg = a.Rb + (nb + i) * (M * M);
        for (int rr = 0; rr < M; ++rr) {
#pragma unroll
            for (int d = 0; d < NCH; ++d) {
                const int g = ch * NCH + d;
                if (g < M) Sg[rr * M + g] = r[rr].d[d];
                else if (g < D) Rg[rr * M + g - M] = r[rr].d[d];
            }
        }
    } else if (ch < NCHB) {
        // BC blocks: columns ch*8.. of dbca/dy0 and dbcb/dyN
        DC ya[M], yb[M], ra[M], rb[M];
        for (int m = 0; m < M; ++m) { ya[m] = DC(yj[m]); yb[m] = DC(yj[(N - 1) * M + m]); ra[m] = DC(JT(0)); rb[m] = DC(JT(0)); }
#pragma unroll
        for (int d = 0; d < NCH; ++d) {
            const int g = ch * NCH + d;
            if (g < M) { ya[g].d[d] = JT(1); yb[g].d[d] = JT(1); }
        }
        bvp_bca<DC, JT>(ra, ya, pj);
        bvp_bcb<DC, JT>(rb, yb, pj);
        JT* G0 = a.G + (long long)q * 2 * M * M;
        JT* G1 = G0 + M * M;
        for (int k = 0; k < M; ++k) {
#pragma unroll
            for (int d = 0; d < NCH; ++d) {
                const int g = ch * NCH + d;
                if (g >= M) continue;
                if (k < LA) { G0[k * M + g] = ra[k].d[d]; G1[k * M + g] = JT(0); }
                else { G1[k * M + g] = rb[k - LA].d[d]; G0[k * M + g] = JT(0); }
            }
        }
    }
}

namespace bvp {

// Gaussian elimination with row pivoting on the first M columns of the warp's 2M x WC
// workspace W (lane l owns rows l and l + 32). Afterwards rows 0..M-1 hold the pivot rows
// [U | X | Y | g] (U upper triangular) and rows M..2M-1 the reduced equations
// [0 | A' | B' | g']. Returns false on a zero or non-finite pivot (uniform across the warp).
BVP_DEV bool warp_gepp(JT* W, int ncols) {
    const int lane = lane_id();
    bool ok = true;
    for (int k = 0; k < M; ++k) {
        JT v = JT(-1);
        int pr = 0x7fffffff;
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const int r = lane + 32 * h2;
            if (r >= k && r < WR) {
                const JT av = fabs(W[r * WLD + k]);
                if (av > v) { v = av; pr = r; }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const JT v2 = __shfl_xor_sync(FULL, v, o);
            const int p2 = __shfl_xor_sync(FULL, pr, o);
            if (v2 > v || (v2 == v && p2 < pr)) { v = v2; pr = p2; }
        }
        ok = ok && v > JT(0) && isfinite(v);
        if (pr != k && pr < WR) {
            for (int c = lane; c < ncols; c += 32) {
                const JT tmp = W[k * WLD + c];
                W[k * WLD + c] = W[pr * WLD + c];
                W[pr * WLD + c] = tmp;
            }
        }
        __syncwarp();
        const JT inv = JT(1) / W[k * WLD + k];
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const int r = lane + 32 * h2;
            if (r > k && r < WR) {
                const JT mlt = W[r * WLD + k] * inv;
                for (int c = k; c < ncols; ++c) W[r * WLD + c] -= mlt * W[k * WLD + c];
            }
        }
        __syncwarp();
    }
    return ok;
}

// x = U^{-1} (g - X lo - Y hi) from a record (U, X, Y, g), the warp cooperating (lane r: row r)
BVP_DEV void warp_back_solve(const JT* rg, const JT* lo, const JT* hi, JT* x_out) {
    const int lane = lane_id();
    JT t = JT(0);
    if (lane < M) {
        t = rg[3 * M * M + lane];
        for (int c = 0; c < M; ++c)
            t -= rg[M * M + lane * M + c] * lo[c] + rg[2 * M * M + lane * M + c] * hi[c];
    }
    for (int r = M - 1; r >= 0; --r) {
        const JT xr = __shfl_sync(FULL, t / (lane < M ? rg[lane * M + lane] : JT(1)), r);
        if (lane == r) t = xr;
        if (lane < r) t -= rg[lane * M + r] * xr;
    }
    if (lane < M) x_out[lane] = t;
    __syncwarp();
}

// store the pivot rows of W as an elimination record
BVP_DEV void store_record(const JT* W, JT* rec) {
    for (int e = lane_id(); e < M * M; e += 32) {
        const int r = e / M, c = e % M;
        rec[e] = W[r * WLD + c];
        rec[M * M + e] = W[r * WLD + M + c];
        rec[2 * M * M + e] = W[r * WLD + 2 * M + c];
    }
    for (int r = lane_id(); r < M; r += 32) rec[3 * M * M + r] = W[r * WLD + 3 * M];
    __syncwarp();
}

// relation rows M..2M-1 of W ([0 | A | B | g]) moved to rows 0..M-1 as the current relation
// in the layout [B | A | 0 | g] ready for the next elimination (δ_hi becomes δ_mid)
BVP_DEV void relation_to_top(JT* W) {
    for (int e = lane_id(); e < M * M; e += 32) {
        const int r = e / M, c = e % M;
        const JT A = W[(M + r) * WLD + M + c];
        const JT B = W[(M + r) * WLD + 2 * M + c];
        W[r * WLD + c] = B;
        W[r * WLD + M + c] = A;
        W[r * WLD + 2 * M + c] = JT(0);
    }
    for (int r = lane_id(); r < M; r += 32) W[r * WLD + 3 * M] = W[(M + r) * WLD + 3 * M];
    __syncwarp();
}

}  // namespace bvp

// ---- linear solve: one CTA per active instance ----------------------------------------------
// Dynamic shared memory: one WR x WLD workspace per warp (BVP_JT).
extern "C" __global__ void __launch_bounds__(256) bl_linsolve(const BvpLargeArgs a) {
    using namespace bvp;
    extern __shared__ __align__(16) unsigned char bl_smem[];
    JT* Wall = reinterpret_cast<JT*>(bl_smem);
    __shared__ int s_lo[8], s_hi[8];
    __shared__ int s_bad;
    const int q = a.active[blockIdx.x];
    const int N = a.N[q];
    const int nI = N - 1;
    const int warp = threadIdx.x >> 5, lane = lane_id();
    const int NWl = int(blockDim.x >> 5);
    const int NW = nI < NWl ? nI : NWl;             // warps with a chunk
    const long long nb = a.node_off[q];
    JT* W = Wall + warp * (WR * WLD);
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
        // relation of interval c0: S δ_c0 + R δ_c0+1 = -F, in the top rows as [R | S | 0 | -F]
        for (int e = lane; e < M * M; e += 32) {
            const int r = e / M, c = e % M;
            W[r * WLD + c] = Rb[(long long)c0 * M * M + e];
            W[r * WLD + M + c] = Sb[(long long)c0 * M * M + e];
            W[r * WLD + 2 * M + c] = JT(0);
        }
        for (int r = lane; r < M; r += 32) W[r * WLD + 3 * M] = JT(-F[(long long)c0 * M + r]);
        __syncwarp();
        for (int c = c0 + 1; c < c1; ++c) {
            // bottom rows: interval c, [S_c | 0 | R_c | -F_c]
            for (int e = lane; e < M * M; e += 32) {
                const int r = e / M, cc = e % M;
                W[(M + r) * WLD + cc] = Sb[(long long)c * M * M + e];
                W[(M + r) * WLD + M + cc] = JT(0);
                W[(M + r) * WLD + 2 * M + cc] = Rb[(long long)c * M * M + e];
            }
            for (int r = lane; r < M; r += 32) W[(M + r) * WLD + 3 * M] = JT(-F[(long long)c * M + r]);
            __syncwarp();
            ok &= warp_gepp(W, WC);
            store_record(W, rec + (long long)c * RECW);
            relation_to_top(W);
        }
        if (lane == 0) { s_lo[warp] = c0; s_hi[warp] = c1; }
    }
    __syncthreads();
    // 2. combine chunk relations pairwise: warp w (multiple of 2s) eliminates the node it shares
    //    with warp w + s; its relation then spans both chunks
    for (int s = 1; s < NW; s <<= 1) {
        if (warp < NW && (warp % (2 * s)) == 0 && warp + s < NW) {
            const JT* W2 = Wall + (warp + s) * (WR * WLD);
            // bottom rows: the partner's relation [B2 | A2 | 0 | g2] as [A2 | 0 | B2 | g2]
            for (int e = lane; e < M * M; e += 32) {
                const int r = e / M, cc = e % M;
                W[(M + r) * WLD + cc] = W2[r * WLD + M + cc];
                W[(M + r) * WLD + M + cc] = JT(0);
                W[(M + r) * WLD + 2 * M + cc] = W2[r * WLD + cc];
            }
            for (int r = lane; r < M; r += 32) W[(M + r) * WLD + 3 * M] = W2[r * WLD + 3 * M];
            __syncwarp();
            ok &= warp_gepp(W, WC);
            store_record(W, rec + (long long)s_hi[warp] * RECW);
            relation_to_top(W);
            if (lane == 0) s_hi[warp] = s_hi[warp + s];
        }
        __syncthreads();
    }
    // 3. warp 0: [dbca/dy0 rows | relation | dbcb/dyN rows] in δ_0, δ_N-1 (2M x 2M). The
    //    relation sits in warp 0's top rows as [B | A | 0 | g] (A on δ_0, B on δ_N-1); it is
    //    staged in warp 1's workspace in the column order δ_0 | δ_N-1 | rhs first.
    if (warp == 0) {
        JT* Wd = W;
        JT* Wt = Wall + 1 * (WR * WLD);
        const JT* G0 = a.G + (long long)q * 2 * M * M;
        const JT* G1 = G0 + M * M;
        const double* bc = a.bcres + (long long)q * M;
        for (int e = lane; e < M * (2 * M + 1); e += 32) {
            const int r = e / (2 * M + 1), c = e % (2 * M + 1);
            Wt[r * WLD + c] = c < M ? W[r * WLD + M + c] : (c < 2 * M ? W[r * WLD + c - M] : W[r * WLD + 3 * M]);
        }
        __syncwarp();
        for (int e = lane; e < LA * (2 * M + 1); e += 32) {
            const int r = e / (2 * M + 1), c = e % (2 * M + 1);
            Wd[r * WLD + c] = c < M ? G0[r * M + c] : (c < 2 * M ? JT(0) : JT(-bc[r]));
        }
        for (int e = lane; e < M * (2 * M + 1); e += 32) {
            const int r = e / (2 * M + 1), c = e % (2 * M + 1);
            Wd[(LA + r) * WLD + c] = Wt[r * WLD + c];
        }
        for (int e = lane; e < (M - LA) * (2 * M + 1); e += 32) {
            const int r = LA + e / (2 * M + 1), c = e % (2 * M + 1);
            Wd[(M + r) * WLD + c] = c < M ? JT(0) : (c < 2 * M ? G1[r * M + c - M] : JT(-bc[r]));
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
                    const JT av = fabs(Wd[r * WLD + k]);
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
                    const JT tmp = Wd[k * WLD + c];
                    Wd[k * WLD + c] = Wd[pr * WLD + c];
                    Wd[pr * WLD + c] = tmp;
                }
            }
            __syncwarp();
            const JT inv = JT(1) / Wd[k * WLD + k];
#pragma unroll
            for (int h2 = 0; h2 < 2; ++h2) {
                const int r = lane + 32 * h2;
                if (r > k && r < 2 * M) {
                    const JT mlt = Wd[r * WLD + k] * inv;
                    for (int c = k; c <= 2 * M; ++c) Wd[r * WLD + c] -= mlt * Wd[k * WLD + c];
                }
            }
            __syncwarp();
        }
        for (int k = 2 * M - 1; k >= 0; --k) {
            if (lane == 0) Wd[k * WLD + 2 * M] = Wd[k * WLD + 2 * M] / Wd[k * WLD + k];
            __syncwarp();
            for (int r = lane; r < k; r += 32) Wd[r * WLD + 2 * M] -= Wd[r * WLD + k] * Wd[k * WLD + 2 * M];
            __syncwarp();
        }
        for (int m = lane; m < M; m += 32) {
            dl[m] = Wd[m * WLD + 2 * M];
            dl[(long long)(N - 1) * M + m] = Wd[(M + m) * WLD + 2 * M];
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
            JT* xm = dl + (long long)mid * M;
            warp_back_solve(rec + (long long)mid * RECW, dl + (long long)lo * M, dl + (long long)hi * M, xm);
        }
        __syncthreads();
    }
    // 5. back substitution inside each chunk (the chunk ends are known)
    if (warp < NW) {
        const int lo = c0;
        for (int c = c1 - 1; c > c0; --c)
            warp_back_solve(rec + (long long)c * RECW, dl + (long long)lo * M, dl + (long long)(c + 1) * M,
                            dl + (long long)c * M);
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

extern "C" __global__ void bl_convert_params(const double* p, bvp::JT* pj, long long n) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        pj[k] = bvp::JT(p[k]);
}

extern "C" __global__ void bl_layout_probe(int* out) {
    out[0] = int(sizeof(BvpLargeArgs));
    out[1] = bvp::RECW;
    out[2] = bvp::WLD;
    out[3] = bvp::NCHUNK;
    out[4] = bvp::S;
    out[5] = bvp::NSXA;
}
