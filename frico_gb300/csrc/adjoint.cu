// Adjoint sensitivities of the antenna quantities FRICO reports: the input
// impedance Zin = V0 / sum_feed(l_i s_i I_i) (compute_port_values,
// src/emw_ana_antenna.cpp:76-105) and |E(P)|^2 of eval_fields
// (src/emw_postpro_common.cpp:31-90), with respect to every mesh vertex
// coordinate and the frequency. FRICO has no derivatives; this is the
// hand-written reverse mode of its own fill (src/emw_solver.cpp:45-142, degree-1
// Dunavant rule with the sub-triangle split), delta-gap RHS
// (src/emw_solver.cpp:352-378), current lumping (src/emw_solver.h:137-164) and
// field formula.
//
// With Z I = V, c the port vector (c_i = l_i s_i on feed edges) and
// E = A I the field at P:
//   dZin   = -(Zin^2 / V0) (dc^T I + lam^T (dV - dZ I)),       Z^T lam = c
//   d|E|^2 = 2 Re(E^H dA I + mu^T (dV - dZ I)),                Z^T mu  = A^T conj(E)
// lam and mu come from one transposed solve with the factors of the forward
// solve (transposed copies of the factors run through the same chained
// triangular solves; the mixed path refines against the FP64 Z^T). The only
// O(N^2) term, w^T dZ I = sum_ij w_j I_i dZ_ji, is a reverse pass over the
// fill on the GPU: one thread per (basis triangle, test triangle) pair
// recomputes the Green function and scatters the derivative of every entry
// into per-triangle centroid gradients and per-half-RWG free-vertex gradients;
// the split (sub-triangle) terms, O(N), go through a per-RWG kernel.
// Everything else is O(N) and runs on the host.
//
// Per term of Z_ji (basis point p on T_ia, test point q on T_jb, weight w):
//   t = K phi G,  K = l_i l_j s_a s_b w / (4 pi),  phi = (p - v_ia).(q - v_jb) / 4 - 1/k^2,
//   G = e^{-jkR}/R, R = |p - q|,  dG/dR = -(1/R + jk) G,  dG/dk = -jR G.
// Dunavant degree-1 points are centroids (d p / d v = 1/3 per vertex) and the
// sub-triangle points are (v_s + v_{s+1} + c)/3; the weight ratios w/A are
// constants (1 or 1/3), so areas carry no derivative.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

#include "common.cuh"

namespace frico {

namespace {

constexpr double kInv4Pi = 0.25 * M_1_PI;

// ------------------------------------------------------------------ transposed factors
template <typename C>
__global__ void k_transpose(const C* __restrict__ A, int64_t lda, int n, C* __restrict__ At, int64_t ldt) {
    __shared__ C t[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = bx + threadIdx.x, c = by + k;   // A(r, c)
        if (r < n && c < n) t[k][threadIdx.x] = A[int64_t(c) * lda + r];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = by + threadIdx.x, c = bx + k;   // At(r, c) = A(c, r)
        if (r < n && c < n) At[int64_t(c) * ldt + r] = t[threadIdx.x][k];
    }
}

// Inverted diagonal blocks of the transposed factors: the forward solve keeps
// Linv_b then Uinv_b (64 x 64, column-major); Z^T's lower pass needs
// (Uinv_b)^T and its upper pass (Linv_b)^T.
template <typename C>
__global__ void k_transpose_dinv(const C* __restrict__ D, int nb, C* __restrict__ Dt) {
    const int b = blockIdx.x;                 // 0 .. 2 nb - 1 of the output
    const int src = b < nb ? nb + b : b - nb;
    const C* s = D + int64_t(src) * 4096;
    C* d = Dt + int64_t(b) * 4096;
    for (int idx = threadIdx.x; idx < 4096; idx += blockDim.x) {
        const int r = idx & 63, c = idx >> 6;
        d[idx] = s[r * 64 + c];
    }
}

// X[perm[i], c] (+)= W[i, c]  (x = P w for Z = P L U)
template <typename C>
__global__ void k_scatter_add(int n, int nrhs, const int32_t* __restrict__ perm, const C* __restrict__ W,
                              double2* __restrict__ X, int first) {
    const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= int64_t(n) * nrhs) return;
    const int i = int(idx % n), c = int(idx / n);
    const double2 w = make_double2(double(W[idx].x), double(W[idx].y));
    double2* x = X + int64_t(c) * n + perm[i];
    *x = first ? w : cadd(*x, w);
}

template <typename C>
__global__ void k_to(int64_t cnt, const double2* __restrict__ a, C* __restrict__ b) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < cnt) b[i] = C{decltype(b[0].x)(a[i].x), decltype(b[0].x)(a[i].y)};
}

// R[:, c] = B[:, c] - Z^T X[:, c] (FP64), one warp per column of Z; nrhs <= 4.
__global__ void k_residual_t(const double2* __restrict__ Z, int64_t ldz, int n, const double2* __restrict__ X,
                             const double2* __restrict__ B, int nrhs, double2* __restrict__ R) {
    const int warp = int((blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (warp >= n) return;
    const double2* col = Z + int64_t(warp) * ldz;
    double2 acc[4] = {};
    for (int j = lane; j < n; j += 32) {
        const double2 z = col[j];
#pragma unroll
        for (int c = 0; c < 4; c++)
            if (c < nrhs) {
                const double2 x = X[int64_t(c) * n + j];
                acc[c].x = fma(z.x, x.x, fma(-z.y, x.y, acc[c].x));
                acc[c].y = fma(z.x, x.y, fma(z.y, x.x, acc[c].y));
            }
    }
#pragma unroll
    for (int c = 0; c < 4; c++)
        for (int o = 16; o > 0; o >>= 1) {
            acc[c].x += __shfl_xor_sync(0xffffffffu, acc[c].x, o);
            acc[c].y += __shfl_xor_sync(0xffffffffu, acc[c].y, o);
        }
    if (lane < nrhs) {
        double2 a = acc[0];
#pragma unroll
        for (int c = 1; c < 4; c++)
            if (lane == c) a = acc[c];
        R[int64_t(lane) * n + warp] = csub(B[int64_t(lane) * n + warp], a);
    }
}

// ------------------------------------------------------------------ reverse pass over the fill
struct AdjTables {
    const double* qp;        // [nt][4] degree-1 point (x, y, z, w)
    const double* qps;       // [nt][3][4] sub-triangle points
    const TriGeo* geo;       // areas
    const int32_t* tri_bf;   // [nt][3] signed (basis + 1) per slot, + on T+
    const int32_t* itm;      // [n]
    const int32_t* itp;
    const double* len;
    const double* vm;        // [n][3] free vertex of T-
    const double* vp;
    const double2* u;        // [n] basis-side weights (the currents I)
    const double2* w;        // [n] test-side weights (the adjoint solution)
    const int64_t* tri;      // [nt][3] vertex ids
    double k;
};

// Accumulators (double2 = complex): tri_gc[nt][3] centroid-point gradients,
// slot_gv[nt][3 slots][3] free-vertex gradients, vert_g[nv][3] direct vertex
// gradients (sub-triangle points), gk[1] d/dk.
struct AdjOut {
    double2* tri_gc;
    double2* slot_gv;
    double2* vert_g;
    double2* gk;
};

__device__ __forceinline__ void atomic_add_c(double2* a, double2 v) {
    atomicAdd(&a->x, v.x);
    atomicAdd(&a->y, v.y);
}

// one term K phi G with K the complex weight (u_i w_j s_a s_b l_i l_j w / 4 pi):
// A = K G, B = K phi G'/R. Returns the complex d/dk contribution.
struct TermGrad {
    double2 A, B, gk;
};

__device__ __forceinline__ TermGrad term_grad(double2 K, double phi, double R, double k) {
    double s, c;
    sincos(k * R, &s, &c);
    const double2 G = make_double2(c / R, -s / R);
    const double2 A = cmul(K, G);
    // G'/R = -(1/R + jk) G / R
    const double2 Gp = cmul(make_double2(-1.0 / (R * R), -k / R), G);
    const double2 B = cscale(cmul(K, Gp), phi);
    // d/dk: K (2/k^3 G - jR phi G)
    const double2 gk = cmul(A, make_double2(2.0 / (k * k * k), -R * phi));
    return {A, B, gk};
}

// Thread (T = basis triangle, T' = test triangle), non-split terms only: the
// pairs with T' in {T_i-, T_i+} are the split terms of k_adj_split. A warp
// holds 32 consecutive T' and walks its CTA's range of T.
__global__ void __launch_bounds__(256) k_adj_pairs(int nt, int t_per_cta, AdjTables tb, AdjOut out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tq = blockIdx.x * 32 + lane;          // test triangle T'
    const bool qok = tq < nt;
    double q[3] = {0, 0, 0}, wq = 0;
    int32_t bq[3] = {0, 0, 0};
    double vq[3][3] = {};
    double2 wj[3] = {};                              // test weights w_j s_b l_j
    if (qok) {
        for (int d = 0; d < 3; d++) q[d] = tb.qp[4 * tq + d];
        wq = tb.qp[4 * tq + 3] / tb.geo[tq].area;
        for (int sl = 0; sl < 3; sl++) {
            const int32_t b = tb.tri_bf[3 * tq + sl];
            bq[sl] = b;
            if (!b) continue;
            const int j = (b > 0 ? b : -b) - 1;
            const double* fv = (b > 0 ? tb.vp : tb.vm) + 3 * j;
            for (int d = 0; d < 3; d++) vq[sl][d] = fv[d];
            wj[sl] = cscale(tb.w[j], (b > 0 ? 1.0 : -1.0) * tb.len[j]);
        }
    }
    // T'-side accumulators: per slot sum(A e)/4, and sum(B) (R vector part)
    double2 gq_v[3][3] = {}, gq_c[3] = {}, gk = make_double2(0, 0);
    const double inv_k2 = 1.0 / (tb.k * tb.k);
    const int t_lo = blockIdx.y * t_per_cta, t_hi = min(nt, t_lo + t_per_cta);
    for (int tp = t_lo + warp; tp < t_hi; tp += 8) {
        double p[3];
        for (int d = 0; d < 3; d++) p[d] = tb.qp[4 * tp + d];
        const double wp = tb.qp[4 * tp + 3] / tb.geo[tp].area;
        double2 gp_v[3][3] = {}, gp_c[3] = {};
        if (qok && tq != tp) {
            const double vr[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
            const double R = sqrt(vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2]);
            for (int sa = 0; sa < 3; sa++) {
                const int32_t a = tb.tri_bf[3 * tp + sa];
                if (!a) continue;
                const int i = (a > 0 ? a : -a) - 1;
                const int other = a > 0 ? tb.itm[i] : tb.itp[i];
                if (other == tq) continue;   // T' = the other triangle of RWG i: split term
                const double* fv = (a > 0 ? tb.vp : tb.vm) + 3 * i;
                const double e[3] = {p[0] - fv[0], p[1] - fv[1], p[2] - fv[2]};
                const double2 ui = cscale(tb.u[i], (a > 0 ? 1.0 : -1.0) * tb.len[i] * wp * wq * kInv4Pi);
                for (int sb = 0; sb < 3; sb++) {
                    if (!bq[sb]) continue;
                    const double d_[3] = {q[0] - vq[sb][0], q[1] - vq[sb][1], q[2] - vq[sb][2]};
                    const double phi = 0.25 * (e[0] * d_[0] + e[1] * d_[1] + e[2] * d_[2]) - inv_k2;
                    const TermGrad g = term_grad(cmul(ui, wj[sb]), phi, R, tb.k);
                    gk = cadd(gk, g.gk);
                    for (int d = 0; d < 3; d++) {
                        // p: A d/4 + B vr; v_ia: -A d/4; q: A e/4 - B vr; v_jb: -A e/4 (as FMAs)
                        const double sd = 0.25 * d_[d], se = 0.25 * e[d], vd = vr[d];
                        gp_c[d].x = fma(g.A.x, sd, fma(g.B.x, vd, gp_c[d].x));
                        gp_c[d].y = fma(g.A.y, sd, fma(g.B.y, vd, gp_c[d].y));
                        gp_v[sa][d].x = fma(-g.A.x, sd, gp_v[sa][d].x);
                        gp_v[sa][d].y = fma(-g.A.y, sd, gp_v[sa][d].y);
                        gq_c[d].x = fma(g.A.x, se, fma(-g.B.x, vd, gq_c[d].x));
                        gq_c[d].y = fma(g.A.y, se, fma(-g.B.y, vd, gq_c[d].y));
                        gq_v[sb][d].x = fma(-g.A.x, se, gq_v[sb][d].x);
                        gq_v[sb][d].y = fma(-g.A.y, se, gq_v[sb][d].y);
                    }
                }
            }
        }
        // reduce the T-side sums over the warp's 32 test triangles
        for (int d = 0; d < 3; d++) {
            for (int o = 16; o > 0; o >>= 1) {
                gp_c[d].x += __shfl_xor_sync(0xffffffffu, gp_c[d].x, o);
                gp_c[d].y += __shfl_xor_sync(0xffffffffu, gp_c[d].y, o);
                for (int sa = 0; sa < 3; sa++) {
                    gp_v[sa][d].x += __shfl_xor_sync(0xffffffffu, gp_v[sa][d].x, o);
                    gp_v[sa][d].y += __shfl_xor_sync(0xffffffffu, gp_v[sa][d].y, o);
                }
            }
        }
        if (lane == 0) {
            for (int d = 0; d < 3; d++) {
                atomic_add_c(out.tri_gc + 3 * tp + d, gp_c[d]);
                for (int sa = 0; sa < 3; sa++) atomic_add_c(out.slot_gv + 9 * tp + 3 * sa + d, gp_v[sa][d]);
            }
        }
    }
    if (qok) {
        for (int d = 0; d < 3; d++) {
            atomic_add_c(out.tri_gc + 3 * tq + d, gq_c[d]);
            for (int sb = 0; sb < 3; sb++) atomic_add_c(out.slot_gv + 9 * tq + 3 * sb + d, gq_v[sb][d]);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        gk.x += __shfl_xor_sync(0xffffffffu, gk.x, o);
        gk.y += __shfl_xor_sync(0xffffffffu, gk.y, o);
    }
    if (lane == 0) atomic_add_c(out.gk, gk);
}

// Split terms: basis RWG i (thread), side a, test triangle T' in {T_i-, T_i+},
// every test half-RWG (j, b) on T', the three sub-triangle points of T'.
__global__ void k_adj_split(int n, AdjTables tb, AdjOut out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double inv_k2 = 1.0 / (tb.k * tb.k);
    double2 gk = make_double2(0, 0);
    for (int a = 0; a < 2; a++) {   // a = 0: T-, 1: T+
        const int tp = a ? tb.itp[i] : tb.itm[i];
        const double* fv = (a ? tb.vp : tb.vm) + 3 * i;
        double p[3];
        for (int d = 0; d < 3; d++) p[d] = tb.qp[4 * tp + d];
        const double wp = tb.qp[4 * tp + 3] / tb.geo[tp].area;
        const double e[3] = {p[0] - fv[0], p[1] - fv[1], p[2] - fv[2]};
        const double2 ui = cscale(tb.u[i], (a ? 1.0 : -1.0) * tb.len[i] * wp * kInv4Pi);
        // slot of (i, a) on tp
        int sa = 0;
        for (int s = 0; s < 3; s++)
            if (tb.tri_bf[3 * tp + s] == (a ? i + 1 : -(i + 1))) sa = s;
        double2 gp_c[3] = {}, gp_v[3] = {};
        for (int side = 0; side < 2; side++) {
            const int tq = side ? tb.itp[i] : tb.itm[i];
            const double area_q = tb.geo[tq].area;
            int64_t vid[3];
            for (int s = 0; s < 3; s++) vid[s] = tb.tri[3 * tq + s];
            for (int sb = 0; sb < 3; sb++) {
                const int32_t b = tb.tri_bf[3 * tq + sb];
                if (!b) continue;
                const int j = (b > 0 ? b : -b) - 1;
                const double* fq = (b > 0 ? tb.vp : tb.vm) + 3 * j;
                const double2 K0 = cmul(ui, cscale(tb.w[j], (b > 0 ? 1.0 : -1.0) * tb.len[j]));
                double2 gv_b[3] = {};
                for (int s = 0; s < 3; s++) {
                    const double* qs = tb.qps + 12 * tq + 4 * s;
                    const double d_[3] = {qs[0] - fq[0], qs[1] - fq[1], qs[2] - fq[2]};
                    const double vr[3] = {p[0] - qs[0], p[1] - qs[1], p[2] - qs[2]};
                    const double R = sqrt(vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2]);
                    const double phi = 0.25 * (e[0] * d_[0] + e[1] * d_[1] + e[2] * d_[2]) - inv_k2;
                    const TermGrad g = term_grad(cscale(K0, qs[3] / area_q), phi, R, tb.k);
                    gk = cadd(gk, g.gk);
                    for (int d = 0; d < 3; d++) {
                        const double2 ad = cscale(g.A, 0.25 * d_[d]), ae = cscale(g.A, 0.25 * e[d]);
                        const double2 bv = cscale(g.B, vr[d]);
                        gp_c[d] = cadd(gp_c[d], cadd(ad, bv));
                        gp_v[d] = csub(gp_v[d], ad);
                        gv_b[d] = csub(gv_b[d], ae);
                        // sub-point q_s = (v_s + v_{s+1} + c)/3: vertex weights 1/3 + 1/9, 1/3 + 1/9, 1/9
                        const double2 gqs = csub(ae, bv);
                        for (int vv = 0; vv < 3; vv++) {
                            const double wgt = (vv == s || vv == (s + 1) % 3 ? 1.0 / 3.0 : 0.0) + 1.0 / 9.0;
                            atomic_add_c(out.vert_g + 3 * vid[vv] + d, cscale(gqs, wgt));
                        }
                    }
                }
                for (int d = 0; d < 3; d++) atomic_add_c(out.slot_gv + 9 * tq + 3 * sb + d, gv_b[d]);
            }
        }
        for (int d = 0; d < 3; d++) {
            atomic_add_c(out.tri_gc + 3 * tp + d, gp_c[d]);
            atomic_add_c(out.slot_gv + 9 * tp + 3 * sa + d, gp_v[d]);
        }
    }
    atomic_add_c(out.gk, gk);
}

using cd = std::complex<double>;

}  // namespace

// Z^T X = B for the factors of the last solve (host in, host out), nrhs <= 4.
static int solve_transposed(frico_gpu_ctx* ctx, const std::vector<cd>& B, int nrhs, std::vector<cd>& X) {
    const int n = int(ctx->n);
    const int64_t cnt = int64_t(n) * nrhs;
    const int nb = (n + 63) / 64;
    cudaStream_t st = ctx->stream;
    const bool mixed = ctx->factor_prec == FRICO_PREC_MIXED;
    const size_t es = mixed ? sizeof(float2) : sizeof(double2);
    int rc;
    if ((rc = ensure(ctx, ctx->lut, es * size_t(n) * n))) return rc;
    if ((rc = ensure(ctx, ctx->dinv_t, es * size_t(2) * nb * 4096))) return rc;
    // workspace: B, X, R (c128) + W (c64 or c128) + norms
    if ((rc = ensure(ctx, ctx->adj_ws, sizeof(double2) * 4 * cnt + 64 * sizeof(double)))) return rc;
    double2* dB = (double2*)ctx->adj_ws.p;
    double2* dX = dB + cnt;
    double2* dR = dX + cnt;
    void* dW = dR + cnt;
    double* nrm = (double*)((double2*)dW + cnt);
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(dB, B.data(), sizeof(double2) * cnt, cudaMemcpyHostToDevice, st),
                         "adjoint rhs")))
        return rc;
    const dim3 tg((n + 31) / 32, (n + 31) / 32), tb(32, 8);
    if (mixed) {
        if ((rc = trsv_dinv64_fp32(ctx))) return rc;
        k_transpose<float2><<<tg, tb, 0, st>>>((const float2*)ctx->z32.p, n, n, (float2*)ctx->lut.p, n);
        k_transpose_dinv<float2><<<2 * nb, 256, 0, st>>>((const float2*)ctx->dinv.p, nb, (float2*)ctx->dinv_t.p);
    } else {
        k_transpose<double2><<<tg, tb, 0, st>>>((const double2*)ctx->z64.p, n, n, (double2*)ctx->lut.p, n);
        k_transpose_dinv<double2><<<2 * nb, 256, 0, st>>>((const double2*)ctx->dinv.p, nb, (double2*)ctx->dinv_t.p);
    }
    count_launch(ctx, 2);
    const unsigned g1 = unsigned((cnt + 255) / 256);
    const int32_t* perm = (const int32_t*)ctx->perm.p;
    if (!mixed) {
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(dW, dB, sizeof(double2) * cnt, cudaMemcpyDeviceToDevice, st),
                             "copy")))
            return rc;
        if ((rc = trsv_solve_with_fp64(ctx, (const double2*)ctx->lut.p, ctx->dinv_t, (double2*)dW, nrhs, n)))
            return rc;
        k_scatter_add<double2><<<g1, 256, 0, st>>>(n, nrhs, perm, (const double2*)dW, dX, 1);
        count_launch(ctx);
    } else {
        // complex64 transposed solves refined against the FP64 Z^T
        const double tol = ctx->opt.refine_tol > 0 ? ctx->opt.refine_tol : 1e-12;
        const int max_it = ctx->opt.max_refine_iters > 0 ? ctx->opt.max_refine_iters : 30;
        std::vector<double> bn(nrhs), rn(nrhs);
        for (int c = 0; c < nrhs; c++) {
            double s = 0;
            for (int i = 0; i < n; i++) s += std::norm(B[size_t(c) * n + i]);
            bn[c] = s > 0 ? std::sqrt(s) : 1.0;
        }
        const double2* src = dB;
        double prev = 1e300, rel = 1e300;
        std::vector<double2> hR(cnt);
        int it = 0;
        for (; it < max_it; it++) {
            k_to<float2><<<g1, 256, 0, st>>>(cnt, src, (float2*)dW);
            count_launch(ctx);
            if ((rc = trsv_solve_with_fp32(ctx, (const float2*)ctx->lut.p, ctx->dinv_t, (float2*)dW, nrhs, n)))
                return rc;
            k_scatter_add<float2><<<g1, 256, 0, st>>>(n, nrhs, perm, (const float2*)dW, dX, it == 0);
            k_residual_t<<<unsigned((n + 7) / 8), 256, 0, st>>>((const double2*)ctx->z64.p, n, n, dX, dB, nrhs, dR);
            count_launch(ctx, 2);
            if ((rc = cuda_check(ctx, cudaMemcpyAsync(hR.data(), dR, sizeof(double2) * cnt, cudaMemcpyDeviceToHost,
                                                      st), "adjoint residual")))
                return rc;
            if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "adjoint sync"))) return rc;
            rel = 0.0;
            bool finite = true;
            for (int c = 0; c < nrhs; c++) {
                double s = 0;
                for (int i = 0; i < n; i++) s += hR[size_t(c) * n + i].x * hR[size_t(c) * n + i].x +
                                                 hR[size_t(c) * n + i].y * hR[size_t(c) * n + i].y;
                const double v = std::sqrt(s) / bn[c];
                finite = finite && std::isfinite(v);
                rel = std::max(rel, v);
            }
            if (!finite) rel = std::numeric_limits<double>::quiet_NaN();
            src = dR;
            if (!std::isfinite(rel) || rel <= tol) {
                it++;
                break;
            }
            if (it >= 2 && rel > 0.5 * prev) {
                it++;
                break;
            }
            prev = rel;
        }
        (void)nrm;
        if (!(rel <= tol) && !(rel < 1e-9))
            return set_err(ctx, FRICO_GPU_ENOCONV, "adjoint: transposed refinement did not converge");
    }
    if ((rc = cuda_check(ctx, cudaGetLastError(), "adjoint solve kernels"))) return rc;
    X.resize(cnt);
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(X.data(), dX, sizeof(double2) * cnt, cudaMemcpyDeviceToHost, st),
                         "adjoint x")))
        return rc;
    if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "adjoint sync"))) return rc;
    return trsv_check(ctx);
}

// w^T dZ I for the current fill: per-coordinate complex gradient over the
// vertices (3 nv) and the d/dk term.
static int fill_vjp(frico_gpu_ctx* ctx, const std::vector<cd>& I, const std::vector<cd>& w, double k,
                    const std::vector<int64_t>& fv_m, const std::vector<int64_t>& fv_p,
                    std::vector<cd>& gx, cd& gk) {
    const int64_t n = ctx->n, nt = ctx->nt, nv = ctx->nv;
    cudaStream_t st = ctx->stream;
    const size_t acc = size_t(3 * nt + 9 * nt + 3 * nv + 1);
    int rc;
    if ((rc = ensure(ctx, ctx->adj_tab, sizeof(double2) * (2 * n + acc)))) return rc;
    double2* du = (double2*)ctx->adj_tab.p;
    double2* dw = du + n;
    double2* dacc = dw + n;
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(du, I.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, st), "u")))
        return rc;
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(dw, w.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, st), "w")))
        return rc;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(dacc, 0, sizeof(double2) * acc, st), "acc"))) return rc;
    AdjTables tb;
    tb.qp = (const double*)ctx->qp.p;
    tb.qps = (const double*)ctx->qps.p;
    tb.geo = (const TriGeo*)ctx->trigeo.p;
    tb.tri_bf = (const int32_t*)ctx->tri_bf.p;
    tb.itm = (const int32_t*)ctx->rwg_itm.p;
    tb.itp = (const int32_t*)ctx->rwg_itp.p;
    tb.len = (const double*)ctx->rwg_len.p;
    tb.vm = (const double*)ctx->rwg_vm.p;
    tb.vp = (const double*)ctx->rwg_vp.p;
    tb.u = du;
    tb.w = dw;
    tb.tri = (const int64_t*)ctx->tri.p;
    tb.k = k;
    AdjOut out;
    out.tri_gc = dacc;
    out.slot_gv = dacc + 3 * nt;
    out.vert_g = dacc + 12 * nt;
    out.gk = dacc + 12 * nt + 3 * nv;
    const int t_per_cta = 64;
    k_adj_pairs<<<dim3(unsigned((nt + 31) / 32), unsigned((nt + t_per_cta - 1) / t_per_cta)), 256, 0, st>>>(
        int(nt), t_per_cta, tb, out);
    k_adj_split<<<unsigned((n + 127) / 128), 128, 0, st>>>(int(n), tb, out);
    count_launch(ctx, 2);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "adjoint fill kernels"))) return rc;
    std::vector<cd> h(acc);
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(h.data(), dacc, sizeof(double2) * acc, cudaMemcpyDeviceToHost, st),
                         "adjoint acc")))
        return rc;
    if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "adjoint sync"))) return rc;
    const cd* tri_gc = h.data();
    const cd* slot_gv = tri_gc + 3 * nt;
    const cd* vert_g = slot_gv + 9 * nt;
    gk = vert_g[3 * nv];
    gx.assign(vert_g, vert_g + 3 * nv);
    const int32_t* tbf = nullptr;
    std::vector<int32_t> hbf(3 * nt);
    if ((rc = cuda_check(ctx, cudaMemcpy(hbf.data(), ctx->tri_bf.p, sizeof(int32_t) * 3 * nt, cudaMemcpyDeviceToHost),
                         "tri_bf")))
        return rc;
    tbf = hbf.data();
    for (int64_t t = 0; t < nt; t++) {
        for (int s = 0; s < 3; s++) {
            const int64_t v = ctx->h_tri[3 * t + s];
            for (int d = 0; d < 3; d++) gx[3 * v + d] += tri_gc[3 * t + d] / 3.0;   // degree-1 point = centroid
            const int32_t b = tbf[3 * t + s];
            if (!b) continue;
            const int64_t i = (b > 0 ? b : -b) - 1;
            const int64_t f = b > 0 ? fv_p[i] : fv_m[i];
            for (int d = 0; d < 3; d++) gx[3 * f + d] += slot_gv[9 * t + 3 * s + d];
        }
    }
    return FRICO_GPU_OK;
}

int adjoint(frico_gpu_ctx* ctx, double freq, int n_itf, const int32_t* itf_tags, frico_c128 V0c, const double* signs,
            const double* Pobs, int edge_mode, double* g_zre, double* g_zim, double* g_e2, frico_adjoint_result* res) {
    const int64_t n = ctx->n, nt = ctx->nt, nv = ctx->nv;
    int rc;
    if ((rc = frico_gpu_fill(ctx, freq, nullptr, 0))) return rc;
    if ((rc = frico_gpu_set_nrhs(ctx, 1))) return rc;
    if ((rc = frico_gpu_rhs_delta_gap(ctx, freq, 0, n_itf, itf_tags, V0c, signs))) return rc;
    std::vector<cd> I(n);
    int32_t info = 0;
    if ((rc = frico_gpu_solve(ctx, (frico_c128*)I.data(), n, &info))) return rc;

    const double omega = 2.0 * M_PI * freq;
    const double k = omega * std::sqrt(FRICO_MU0 * FRICO_EPS0);
    const double dk_df = 2.0 * M_PI * std::sqrt(FRICO_MU0 * FRICO_EPS0);
    const cd V0(V0c.re, V0c.im), J(0.0, 1.0);
    const std::vector<frico_rwg>& rw = ctx->h_rwg;
    const double* X = ctx->h_xyz.data();
    const int64_t* T = ctx->h_tri.data();
    auto vtx = [&](int64_t v, int d) { return X[3 * v + d]; };
    // free vertex and edge end points of every RWG (ids in the uploaded mesh)
    std::vector<int64_t> fv_m(n), fv_p(n), e0(n), e1(n);
    for (int64_t i = 0; i < n; i++) {
        for (int side = 0; side < 2; side++) {
            const int64_t t = side ? rw[i].itplus : rw[i].itminus;
            const double* pf = side ? rw[i].pplus : rw[i].pminus;
            int64_t f = -1;
            for (int s = 0; s < 3; s++) {
                const int64_t v = T[3 * t + s];
                if (vtx(v, 0) == pf[0] && vtx(v, 1) == pf[1] && vtx(v, 2) == pf[2]) f = v;
            }
            if (f < 0) return set_err(ctx, FRICO_GPU_EMESH, "adjoint: RWG free vertex is not a triangle vertex");
            (side ? fv_p : fv_m)[i] = f;
            if (side == 0) {
                int c = 0;
                for (int s = 0; s < 3; s++)
                    if (T[3 * t + s] != f) (c++ ? e1[i] : e0[i]) = T[3 * t + s];
            }
        }
    }
    // d l_i / d x at the edge end points (e1 - e0 direction)
    auto dl = [&](int64_t i, double g[3]) {
        double d[3];
        for (int a = 0; a < 3; a++) d[a] = vtx(e1[i], a) - vtx(e0[i], a);
        if (edge_mode == FRICO_EDGE_LENGTH_XY) d[2] = 0.0;
        const double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int a = 0; a < 3; a++) g[a] = l > 0 ? d[a] / l : 0.0;
    };
    // feed: c_i = l_i s_i, V_i = -j l_i V0 s_i / (omega mu0)
    std::vector<cd> c(n, 0.0), V(n, 0.0);
    for (int64_t i = 0; i < n; i++) {
        if (!rw[i].has_interface) continue;
        for (int q = 0; q < n_itf; q++)
            if (rw[i].interface_tag == itf_tags[q]) {
                const double s = signs ? signs[i] : 1.0;
                c[i] += rw[i].length * s;
                V[i] += cd(0.0, -rw[i].length / (omega * FRICO_MU0)) * V0 * s;
            }
    }
    cd Iport = 0.0;
    for (int64_t i = 0; i < n; i++) Iport += c[i] * I[i];
    const cd Zin = V0 / Iport;

    // field at P (eval_fields' E) with its per-triangle pieces
    const cd pre = -J * omega * FRICO_MU0;
    std::vector<cd> AJ(3 * nt, 0.0), D(nt, 0.0);
    std::vector<double> ctr(3 * nt);
    for (int64_t t = 0; t < nt; t++)
        for (int a = 0; a < 3; a++) ctr[3 * t + a] = (vtx(T[3 * t], a) + vtx(T[3 * t + 1], a) + vtx(T[3 * t + 2], a)) / 3.0;
    for (int64_t i = 0; i < n; i++)
        for (int side = 0; side < 2; side++) {
            const int64_t t = side ? rw[i].itplus : rw[i].itminus;
            const double* pf = side ? rw[i].pplus : rw[i].pminus;
            const double s = side ? 1.0 : -1.0;
            for (int a = 0; a < 3; a++) AJ[3 * t + a] += s * 0.5 * rw[i].length * (ctr[3 * t + a] - pf[a]) * I[i];
            D[t] += s * rw[i].length * I[i];
        }
    struct TriField { double vr[3], R; cd g, h; };
    std::vector<TriField> tf(nt);
    cd E[3] = {0.0, 0.0, 0.0};
    for (int64_t t = 0; t < nt; t++) {
        TriField& f = tf[t];
        for (int a = 0; a < 3; a++) f.vr[a] = Pobs[a] - ctr[3 * t + a];
        f.R = std::sqrt(f.vr[0] * f.vr[0] + f.vr[1] * f.vr[1] + f.vr[2] * f.vr[2]);
        const double kR = k * f.R;
        f.g = std::exp(cd(0.0, -kR)) / (4 * M_PI * f.R);
        f.h = (1.0 + J * kR) / (kR * kR);
        for (int a = 0; a < 3; a++) E[a] += pre * (AJ[3 * t + a] - D[t] * f.h * f.vr[a]) * f.g;
    }
    const double e2 = std::norm(E[0]) + std::norm(E[1]) + std::norm(E[2]);
    const cd u[3] = {std::conj(E[0]), std::conj(E[1]), std::conj(E[2])};
    // A^T conj(E): d(u.E)/dI_i
    std::vector<cd> ATu(n, 0.0);
    for (int64_t i = 0; i < n; i++)
        for (int side = 0; side < 2; side++) {
            const int64_t t = side ? rw[i].itplus : rw[i].itminus;
            const double* pf = side ? rw[i].pplus : rw[i].pminus;
            const double s = side ? 1.0 : -1.0;
            const TriField& f = tf[t];
            cd uaj = 0.0, uvr = 0.0;
            for (int a = 0; a < 3; a++) {
                uaj += u[a] * (s * 0.5 * rw[i].length * (ctr[3 * t + a] - pf[a]));
                uvr += u[a] * f.vr[a];
            }
            ATu[i] += pre * f.g * (uaj - s * rw[i].length * f.h * uvr);
        }

    // adjoint solve: Z^T [lam mu] = [c, A^T conj(E)]
    std::vector<cd> B(2 * n), LM;
    std::copy(c.begin(), c.end(), B.begin());
    std::copy(ATu.begin(), ATu.end(), B.begin() + n);
    if ((rc = solve_transposed(ctx, B, 2, LM))) return rc;
    std::vector<cd> lam(LM.begin(), LM.begin() + n), mu(LM.begin() + n, LM.end());

    // O(N^2): w^T dZ I for w = lam, mu
    std::vector<cd> gzl, gzm;
    cd gkl, gkm;
    if ((rc = fill_vjp(ctx, I, lam, k, fv_m, fv_p, gzl, gkl))) return rc;
    if ((rc = fill_vjp(ctx, I, mu, k, fv_m, fv_p, gzm, gkm))) return rc;

    // Zin: S = dc^T I + lam^T dV - lam^T dZ I, dZin = -(Zin^2 / V0) S
    // mu:  Q = E^H dA I + mu^T dV - mu^T dZ I,   d|E|^2 = 2 Re Q
    std::vector<cd> S(3 * nv, 0.0), Q(3 * nv, 0.0);
    for (int64_t v = 0; v < 3 * nv; v++) {
        S[v] = -gzl[v];
        Q[v] = -gzm[v];
    }
    cd Sf = -gkl * dk_df, Qf = -gkm * dk_df;
    // length terms: d/dl_i of c, V and Z (Z_ji ~ l_i l_j: dZ_ji/dl_i = Z_ji / l_i,
    // so w^T (dZ/dl_i) I = I_i (Z^T w)_i / l_i + w_i (Z I)_i / l_i)
    std::vector<cd> ZtL = c;   // Z^T lam = c
    for (int64_t i = 0; i < n; i++) {
        const double l = rw[i].length;
        if (!(l > 0)) continue;
        double g[3];
        dl(i, g);
        const cd dS = (c[i] / l) * I[i] + lam[i] * V[i] / l - (I[i] * ZtL[i] / l + lam[i] * V[i] / l);
        const cd dQ = mu[i] * V[i] / l - (I[i] * ATu[i] / l + mu[i] * V[i] / l);
        for (int a = 0; a < 3; a++) {
            S[3 * e1[i] + a] += dS * g[a];
            S[3 * e0[i] + a] -= dS * g[a];
            Q[3 * e1[i] + a] += dQ * g[a];
            Q[3 * e0[i] + a] -= dQ * g[a];
        }
    }
    // frequency: V ~ 1/omega
    for (int64_t i = 0; i < n; i++) {
        Sf += lam[i] * (-V[i] / freq);
        Qf += mu[i] * (-V[i] / freq);
    }
    // explicit field terms E^H dA I (I fixed)
    for (int64_t t = 0; t < nt; t++) {
        const TriField& f = tf[t];
        const double R = f.R, kR = k * R;
        cd uvr = 0.0, uaj = 0.0;
        for (int a = 0; a < 3; a++) {
            uvr += u[a] * f.vr[a];
            uaj += u[a] * AJ[3 * t + a];
        }
        const cd Qt = uaj - D[t] * f.h * uvr;
        const cd gp = -(1.0 / R + J * k) * f.g;                       // dg/dR
        const cd hp = -2.0 / (k * k * R * R * R) - J / (k * R * R);     // dh/dR
        // d(u.E_t)/d vR
        cd dvr[3];
        for (int a = 0; a < 3; a++)
            dvr[a] = pre * (gp * (f.vr[a] / R) * Qt + f.g * (-D[t] * hp * (f.vr[a] / R) * uvr - D[t] * f.h * u[a]));
        // centroid: vR = P - c, and AJ_t depends on c with coefficient D_t / 2
        for (int s = 0; s < 3; s++) {
            const int64_t v = T[3 * t + s];
            for (int a = 0; a < 3; a++) Q[3 * v + a] += (-dvr[a] + pre * f.g * (D[t] * 0.5) * u[a]) / 3.0;
        }
        // frequency: pre ~ omega, g and h through k
        const cd dg_dk = -J * R * f.g;
        const cd dh_dk = -2.0 / (k * k * k * R * R) - J / (k * k * R);
        Qf += (-J * FRICO_MU0 * 2.0 * M_PI) * f.g * Qt + pre * (dg_dk * Qt + f.g * (-D[t] * dh_dk * uvr)) * dk_df;
    }
    for (int64_t i = 0; i < n; i++)
        for (int side = 0; side < 2; side++) {
            const int64_t t = side ? rw[i].itplus : rw[i].itminus;
            const double* pf = side ? rw[i].pplus : rw[i].pminus;
            const double s = side ? 1.0 : -1.0;
            const int64_t f = side ? fv_p[i] : fv_m[i];
            const TriField& tr = tf[t];
            // free vertex inside AJ_t
            for (int a = 0; a < 3; a++) Q[3 * f + a] += pre * tr.g * (-s * 0.5 * rw[i].length * I[i]) * u[a];
            // l_i inside AJ_t and AdivJ_t
            const double l = rw[i].length;
            if (!(l > 0)) continue;
            cd uc = 0.0, uvr = 0.0;
            for (int a = 0; a < 3; a++) {
                uc += u[a] * (ctr[3 * t + a] - pf[a]);
                uvr += u[a] * tr.vr[a];
            }
            const cd dQl = pre * tr.g * (s * 0.5 * I[i] * uc - s * I[i] * tr.h * uvr);
            double g[3];
            dl(i, g);
            for (int a = 0; a < 3; a++) {
                Q[3 * e1[i] + a] += dQl * g[a];
                Q[3 * e0[i] + a] -= dQl * g[a];
            }
        }
    // port vector: dc^T I (c_i = l_i s_i) is in dS above via c_i / l_i I_i
    const cd zf = -(Zin * Zin) / V0;
    for (int64_t v = 0; v < 3 * nv; v++) {
        const cd dz = zf * S[v];
        if (g_zre) g_zre[v] = dz.real();
        if (g_zim) g_zim[v] = dz.imag();
        if (g_e2) g_e2[v] = 2.0 * Q[v].real();
    }
    if (res) {
        res->zin = frico_c128{Zin.real(), Zin.imag()};
        res->e2 = e2;
        for (int a = 0; a < 3; a++) res->e[a] = frico_c128{E[a].real(), E[a].imag()};
        const cd dzf = zf * Sf;
        res->dzin_re_df = dzf.real();
        res->dzin_im_df = dzf.imag();
        res->de2_df = 2.0 * Qf.real();
    }
    return FRICO_GPU_OK;
}

}  // namespace frico

extern "C" int frico_gpu_adjoint(frico_gpu_ctx* ctx, double freq, int32_t n_itf, const int32_t* itf_tags,
                                 frico_c128 V0, const double* signs, const double* P_obs, int32_t edge_length_mode,
                                 double* grad_zin_re, double* grad_zin_im, double* grad_e2,
                                 frico_adjoint_result* out) {
    using namespace frico;
    if (!ctx) return FRICO_GPU_EINVAL;
    if (int rc = cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice")) return rc;
    if (ctx->n <= 0) return set_err(ctx, FRICO_GPU_ESTATE, "adjoint: no mesh (call frico_gpu_set_mesh)");
    if (!(freq > 0) || n_itf <= 0 || !itf_tags || !P_obs)
        return set_err(ctx, FRICO_GPU_EINVAL, "adjoint: need freq > 0, feed tags and an observation point");
    if (edge_length_mode != FRICO_EDGE_LENGTH_XY && edge_length_mode != FRICO_EDGE_LENGTH_TRUE)
        return set_err(ctx, FRICO_GPU_EINVAL, "adjoint: bad edge_length_mode");
    if (ctx->opt.degree != 1 || ctx->opt.approx || ctx->opt.force_symmetry)
        return set_err(ctx, FRICO_GPU_EINVAL,
                       "adjoint: supports the default fill (degree-1 quadrature, no MOM3D approximation, "
                       "no forced symmetry)");
    return adjoint(ctx, freq, n_itf, itf_tags, V0, signs, P_obs, edge_length_mode, grad_zin_re, grad_zin_im,
                   grad_e2, out);
}
