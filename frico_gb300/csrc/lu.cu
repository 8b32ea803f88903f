// Dense complex LU with partial pivoting + triangular solves + mixed-precision
// iterative refinement. Replaces FRICO's solve_general (zgetrf_ + zgetrs_,
// src/lapack_wrappers.cpp:53-133) and solve_symmetric (:135-177, whose
// Bunch-Kaufman factors are not reproduced: the GPU factors the symmetric Z
// with the same LU, and parity is on the solution).
//
// Blocked right-looking LU, block width nb = 64, column-major in place:
//   panel    one cooperative kernel over the (n-k0) x nb panel, rows split
//            across CTAs and held in shared memory; per column one bounded
//            grid barrier publishes every CTA's pivot candidate (max |re|+|im|
//            as LAPACK izamax, lowest row on ties) together with the
//            candidate row, so swap + scale + rank-1 update need no second sync.
//   laswp    the panel's interchanges applied to the other columns.
//   trsm     U12 = L11^-1 A12 (unit lower, shared-memory forward substitution).
//   gemm     A22 -= L21 U12, register-tiled SIMT complex GEMM.
// Pivots are stored 1-based as LAPACK's ipiv.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "common.cuh"

namespace frico {

static const int kNB = 64;          // LU block width
static const int kMaxPanelCTAs = 1024;
static const long long kBarrierTimeoutCycles = 4000000000LL;  // ~2 s at 2 GHz

template <typename R> struct PanelWS {
    unsigned* bar;        // [0] count, [1] generation
    R* cand_val;          // [2][kMaxPanelCTAs]
    int* cand_row;        // [2][kMaxPanelCTAs]
    cplx<R>* cand_data;   // [2][kMaxPanelCTAs][nb]
    cplx<R>* krow;        // [2][nb]
};

// Grid-wide barrier for a cooperative launch. The wait is bounded: on timeout
// the CTA records FRICO_DEV_ERR_TIMEOUT and returns false, so a lost CTA turns
// into an error status instead of a hung GPU.
__device__ bool grid_barrier(unsigned* bar, DeviceStatus* st, int where) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned* vgen = bar + 1;
        unsigned gen = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long t0 = clock64();
            while (*vgen == gen) {
                if (clock64() - t0 > kBarrierTimeoutCycles) {
                    ok = 0;
                    if (atomicCAS(&st->err, 0, FRICO_DEV_ERR_TIMEOUT) == 0) st->where = where;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        if (*(volatile int*)&st->err != 0) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Block-wide argmax of |re|+|im| over column c of the CTA's rows [rs, nr);
// ties go to the lowest row. Returns value (-1 if empty) and local row.
template <typename R>
__device__ void block_argmax(const cplx<R>* col, int rs, int nr, R* out_val, int* out_row) {
    __shared__ R sv[32];
    __shared__ int sr[32];
    R bv = R(-1);
    int br = 0x7fffffff;
    for (int r = rs + threadIdx.x; r < nr; r += blockDim.x) {
        R v = cabs1(col[r]);
        if (v > bv) { bv = v; br = r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        R ov = __shfl_down_sync(0xffffffffu, bv, o);
        int orr = __shfl_down_sync(0xffffffffu, br, o);
        if (ov > bv || (ov == bv && orr < br)) { bv = ov; br = orr; }
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { sv[w] = bv; sr[w] = br; }
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        bv = l < nw ? sv[l] : R(-1);
        br = l < nw ? sr[l] : 0x7fffffff;
        for (int o = 16; o > 0; o >>= 1) {
            R ov = __shfl_down_sync(0xffffffffu, bv, o);
            int orr = __shfl_down_sync(0xffffffffu, br, o);
            if (ov > bv || (ov == bv && orr < br)) { bv = ov; br = orr; }
        }
        if (l == 0) { *out_val = bv; *out_row = br; }
    }
    __syncthreads();
}

template <typename R>
__global__ void __launch_bounds__(256) k_panel(cplx<R>* A, int64_t lda, int n, int k0, int jb,
                                              int rows_per, int32_t* ipiv, PanelWS<R> ws,
                                              DeviceStatus* st) {
    using C = cplx<R>;
    extern __shared__ __align__(16) unsigned char smraw[];
    C* sm = (C*)smraw;             // [jb][rows_per]
    C* prow = sm + size_t(jb) * rows_per;
    C* krow = prow + jb;
    __shared__ R s_val;
    __shared__ int s_row, s_p, s_g;
    const int g = blockIdx.x, tid = threadIdx.x, G = gridDim.x;
    const int r0 = k0 + g * rows_per;
    const int nr = max(0, min(n, r0 + rows_per) - r0);

    for (int idx = tid; idx < nr * jb; idx += blockDim.x) {
        int r = idx % nr, c = idx / nr;
        sm[c * rows_per + r] = A[int64_t(k0 + c) * lda + r0 + r];
    }
    __syncthreads();

    auto publish = [&](int c, int par) {
        int k = k0 + c;
        int rs = max(0, k - r0);
        block_argmax<R>(sm + c * rows_per, rs, nr, &s_val, &s_row);
        if (tid == 0) {
            ws.cand_val[par * kMaxPanelCTAs + g] = s_val;
            ws.cand_row[par * kMaxPanelCTAs + g] = s_val >= R(0) ? r0 + s_row : 0x7fffffff;
        }
        if (s_val >= R(0))
            for (int cc = tid; cc < jb; cc += blockDim.x)
                ws.cand_data[(size_t(par) * kMaxPanelCTAs + g) * jb + cc] = sm[cc * rows_per + s_row];
        if (k >= r0 && k < r0 + nr)
            for (int cc = tid; cc < jb; cc += blockDim.x) ws.krow[par * jb + cc] = sm[cc * rows_per + (k - r0)];
    };

    publish(0, 0);
    if (!grid_barrier(ws.bar, st, k0)) return;

    for (int c = 0; c < jb; c++) {
        const int k = k0 + c, par = c & 1;
        if (tid < 32) {
            R bv = R(-1);
            int brow = 0x7fffffff, bg = 0;
            for (int q = tid; q < G; q += 32) {
                R v = __ldcg(&ws.cand_val[par * kMaxPanelCTAs + q]);
                int rr = __ldcg(&ws.cand_row[par * kMaxPanelCTAs + q]);
                if (v > bv || (v == bv && rr < brow)) { bv = v; brow = rr; bg = q; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                R ov = __shfl_down_sync(0xffffffffu, bv, o);
                int orr = __shfl_down_sync(0xffffffffu, brow, o);
                int og = __shfl_down_sync(0xffffffffu, bg, o);
                if (ov > bv || (ov == bv && orr < brow)) { bv = ov; brow = orr; bg = og; }
            }
            if (tid == 0) { s_p = brow; s_g = bg; }
        }
        __syncthreads();
        const int p = s_p, wg = s_g;
        for (int cc = tid; cc < jb; cc += blockDim.x) {
            prow[cc] = __ldcg(&ws.cand_data[(size_t(par) * kMaxPanelCTAs + wg) * jb + cc]);
            krow[cc] = __ldcg(&ws.krow[par * jb + cc]);
        }
        __syncthreads();
        if (k >= r0 && k < r0 + nr)
            for (int cc = tid; cc < jb; cc += blockDim.x) sm[cc * rows_per + (k - r0)] = prow[cc];
        if (p != k && p >= r0 && p < r0 + nr)
            for (int cc = tid; cc < jb; cc += blockDim.x) sm[cc * rows_per + (p - r0)] = krow[cc];
        if (g == 0 && tid == 0) ipiv[k] = p + 1;
        __syncthreads();
        C piv = prow[c];
        C inv;
        if (piv.x == R(0) && piv.y == R(0)) {
            inv = cmake(R(0), R(0));
            if (g == 0 && tid == 0) atomicCAS(&st->info, 0, k + 1);
        } else {
            inv = cdiv(cmake(R(1), R(0)), piv);
        }
        const int rs = max(0, k + 1 - r0);
        for (int r = rs + tid; r < nr; r += blockDim.x) sm[c * rows_per + r] = cmul(sm[c * rows_per + r], inv);
        __syncthreads();
        const int nrr = nr - rs, ncols = jb - c - 1;
        if (nrr > 0)
            for (int idx = tid; idx < nrr * ncols; idx += blockDim.x) {
                int r = rs + idx % nrr, cc = c + 1 + idx / nrr;
                sm[cc * rows_per + r] = cfms(sm[cc * rows_per + r], sm[c * rows_per + r], prow[cc]);
            }
        __syncthreads();
        if (c + 1 < jb) {
            publish(c + 1, par ^ 1);
            if (!grid_barrier(ws.bar, st, k + 1)) return;
        }
    }
    for (int idx = tid; idx < nr * jb; idx += blockDim.x) {
        int r = idx % nr, c = idx / nr;
        A[int64_t(k0 + c) * lda + r0 + r] = sm[c * rows_per + r];
    }
}

// Row interchanges k <-> ipiv[k]-1, k in [k0, k0+jb), on the columns outside
// the panel (LAPACK zlaswp applied left and right).
template <typename C>
__global__ void k_laswp(C* A, int64_t lda, int n, int k0, int jb, const int32_t* ipiv) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int ncols = n - jb;
    if (t >= ncols) return;
    int col = t < k0 ? t : t + jb;
    C* a = A + int64_t(col) * lda;
    for (int k = k0; k < k0 + jb; k++) {
        int p = ipiv[k] - 1;
        if (p != k) {
            C x = a[k];
            a[k] = a[p];
            a[p] = x;
        }
    }
}

// U12 = L11^{-1} A12; a CTA owns 32 columns, 8 row groups of 32 threads.
template <typename C>
__global__ void __launch_bounds__(256) k_trsm_lower_unit(C* A, int64_t lda, int n, int k0, int jb) {
    extern __shared__ __align__(16) unsigned char smraw[];
    C* L = (C*)smraw;           // [jb][jb] column-major
    C* B = L + jb * jb;         // [32][jb] column-major per column
    const int c0 = k0 + jb + blockIdx.x * 32;
    const int nc = min(32, n - c0);
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) {
        int r = idx % jb, c = idx / jb;
        L[idx] = A[int64_t(k0 + c) * lda + k0 + r];
    }
    for (int idx = threadIdx.x; idx < jb * nc; idx += blockDim.x) {
        int r = idx % jb, c = idx / jb;
        B[c * jb + r] = A[int64_t(c0 + c) * lda + k0 + r];
    }
    __syncthreads();
    const int lc = threadIdx.x & 31, rg = threadIdx.x >> 5;
    for (int q = 0; q < jb; q++) {
        if (lc < nc) {
            C xq = B[lc * jb + q];
            for (int r = q + 1 + rg; r < jb; r += 8) B[lc * jb + r] = cfms(B[lc * jb + r], L[q * jb + r], xq);
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < jb * nc; idx += blockDim.x) {
        int r = idx % jb, c = idx / jb;
        A[int64_t(c0 + c) * lda + k0 + r] = B[c * jb + r];
    }
}

// C[m x nn] -= A[m x kk] * B[kk x nn], all column-major with leading dim lda.
// 64x64 CTA tile, 16 k-slab, 256 threads, each thread 4x4 complex outputs
// (rows tx + 16*i, cols ty + 16*j: conflict-free shared-memory reads).
template <typename R>
__global__ void __launch_bounds__(256) k_gemm_update(cplx<R>* Cm, const cplx<R>* Am, const cplx<R>* Bm,
                                                     int64_t lda, int m, int nn, int kk) {
    using C = cplx<R>;
    __shared__ C As[16][64];
    __shared__ C Bs[16][64];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int bm = blockIdx.x * 64, bn = blockIdx.y * 64;
    C acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = cmake(R(0), R(0));
    for (int k0 = 0; k0 < kk; k0 += 16) {
        for (int idx = threadIdx.x; idx < 16 * 64; idx += 256) {
            int r = idx & 63, c = idx >> 6;  // A tile: 64 rows x 16 cols
            int gr = bm + r, gc = k0 + c;
            As[c][r] = (gr < m && gc < kk) ? Am[int64_t(gc) * lda + gr] : cmake(R(0), R(0));
            int br = idx & 15, bc = idx >> 4;  // B tile: 16 rows x 64 cols
            int gbr = k0 + br, gbc = bn + bc;
            Bs[br][bc] = (gbr < kk && gbc < nn) ? Bm[int64_t(gbc) * lda + gbr] : cmake(R(0), R(0));
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; q++) {
            C a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[q][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[q][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    acc[i][j].x += a[i].x * b[j].x - a[i].y * b[j].y;
                    acc[i][j].y += a[i].x * b[j].y + a[i].y * b[j].x;
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int gr = bm + tx + 16 * i, gc = bn + ty + 16 * j;
            if (gr < m && gc < nn) {
                C* p = Cm + int64_t(gc) * lda + gr;
                *p = csub(*p, acc[i][j]);
            }
        }
}

// ---------------------------------------------------------------- solves
// perm = the row permutation of the whole factorisation (LAPACK ipiv applied
// in order to the identity): (P b)[r] = b[perm[r]].
__global__ void k_perm_from_ipiv(int n, const int32_t* ipiv, int32_t* perm) {
    extern __shared__ int32_t sp[];
    for (int i = threadIdx.x; i < n; i += blockDim.x) sp[i] = i;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < n; k++) {
            int p = ipiv[k] - 1;
            int t = sp[k];
            sp[k] = sp[p];
            sp[p] = t;
        }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

template <typename CI, typename CO>
__global__ void k_gather_rows(int n, int nrhs, const int32_t* perm, const CI* B, int64_t ldb, CO* W,
                              int64_t ldw) {
    int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= int64_t(n) * nrhs) return;
    int r = int(idx % n), c = int(idx / n);
    CI v = B[c * ldb + perm[r]];
    W[c * ldw + r] = {decltype(W[0].x)(v.x), decltype(W[0].x)(v.y)};
}

static const int kTB = 64;   // triangular-solve block
static const int kTR = 8;    // RHS columns per pass

// Forward substitution with the unit lower factor, block rows [kb, kb+nb):
// every CTA solves the diagonal block in shared memory, CTA 0 stores it, and
// each CTA then updates 256 rows below the block.
template <typename C>
__global__ void __launch_bounds__(256) k_trsv_lower(const C* LU, int64_t lda, int n, int kb, int nb,
                                                   C* W, int64_t ldw, int nrhs) {
    __shared__ C Ld[kTB * kTB];
    __shared__ C X[kTB * kTR];
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        int r = idx % nb, c = idx / nb;
        Ld[c * kTB + r] = LU[int64_t(kb + c) * lda + kb + r];
    }
    const int r = kb + nb + blockIdx.x * blockDim.x + threadIdx.x;
    for (int c0 = 0; c0 < nrhs; c0 += kTR) {
        const int nc = min(kTR, nrhs - c0);
        __syncthreads();
        for (int idx = threadIdx.x; idx < nb * nc; idx += blockDim.x) {
            int rr = idx % nb, c = idx / nb;
            X[c * kTB + rr] = W[int64_t(c0 + c) * ldw + kb + rr];
        }
        __syncthreads();
        for (int q = 0; q < nb; q++) {
            int cnt = (nb - q - 1) * nc;
            for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
                int rr = q + 1 + idx % (nb - q - 1), c = idx / (nb - q - 1);
                X[c * kTB + rr] = cfms(X[c * kTB + rr], Ld[q * kTB + rr], X[c * kTB + q]);
            }
            __syncthreads();
        }
        if (blockIdx.x == 0)
            for (int idx = threadIdx.x; idx < nb * nc; idx += blockDim.x) {
                int rr = idx % nb, c = idx / nb;
                W[int64_t(c0 + c) * ldw + kb + rr] = X[c * kTB + rr];
            }
        if (r < n) {
            C acc[kTR];
            for (int c = 0; c < nc; c++) acc[c] = W[int64_t(c0 + c) * ldw + r];
            for (int q = 0; q < nb; q++) {
                C l = LU[int64_t(kb + q) * lda + r];
                for (int c = 0; c < nc; c++) acc[c] = cfms(acc[c], l, X[c * kTB + q]);
            }
            for (int c = 0; c < nc; c++) W[int64_t(c0 + c) * ldw + r] = acc[c];
        }
    }
}

// Back substitution with the upper factor for block rows [kb, kb+nb), then the
// rows above the block.
template <typename C>
__global__ void __launch_bounds__(256) k_trsv_upper(const C* LU, int64_t lda, int n, int kb, int nb,
                                                   C* W, int64_t ldw, int nrhs) {
    __shared__ C Ud[kTB * kTB];
    __shared__ C X[kTB * kTR];
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        int r = idx % nb, c = idx / nb;
        Ud[c * kTB + r] = LU[int64_t(kb + c) * lda + kb + r];
    }
    const int r = blockIdx.x * blockDim.x + threadIdx.x;  // rows above kb
    for (int c0 = 0; c0 < nrhs; c0 += kTR) {
        const int nc = min(kTR, nrhs - c0);
        __syncthreads();
        for (int idx = threadIdx.x; idx < nb * nc; idx += blockDim.x) {
            int rr = idx % nb, c = idx / nb;
            X[c * kTB + rr] = W[int64_t(c0 + c) * ldw + kb + rr];
        }
        __syncthreads();
        for (int q = nb - 1; q >= 0; q--) {
            if (threadIdx.x < nc) {
                int c = threadIdx.x;
                X[c * kTB + q] = cdiv(X[c * kTB + q], Ud[q * kTB + q]);
            }
            __syncthreads();
            int cnt = q * nc;
            for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
                int rr = idx % q, c = idx / q;
                X[c * kTB + rr] = cfms(X[c * kTB + rr], Ud[q * kTB + rr], X[c * kTB + q]);
            }
            __syncthreads();
        }
        if (blockIdx.x == 0)
            for (int idx = threadIdx.x; idx < nb * nc; idx += blockDim.x) {
                int rr = idx % nb, c = idx / nb;
                W[int64_t(c0 + c) * ldw + kb + rr] = X[c * kTB + rr];
            }
        if (r < kb) {
            C acc[kTR];
            for (int c = 0; c < nc; c++) acc[c] = W[int64_t(c0 + c) * ldw + r];
            for (int q = 0; q < nb; q++) {
                C u = LU[int64_t(kb + q) * lda + r];
                for (int c = 0; c < nc; c++) acc[c] = cfms(acc[c], u, X[c * kTB + q]);
            }
            for (int c = 0; c < nc; c++) W[int64_t(c0 + c) * ldw + r] = acc[c];
        }
    }
}

// R = B - Z X in FP64 (refinement residual), one thread per row, X staged in
// shared memory 128 columns at a time.
__global__ void __launch_bounds__(256) k_residual(const double2* Z, int64_t ldz, int n, const double2* X,
                                                 const double2* B, double2* Rr, int64_t ld, int nrhs) {
    __shared__ double2 xs[128 * kTR];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    for (int c0 = 0; c0 < nrhs; c0 += kTR) {
        const int nc = min(kTR, nrhs - c0);
        double2 acc[kTR];
        for (int c = 0; c < kTR; c++) acc[c] = make_double2(0, 0);
        for (int i0 = 0; i0 < n; i0 += 128) {
            const int ni = min(128, n - i0);
            __syncthreads();
            for (int idx = threadIdx.x; idx < ni * nc; idx += blockDim.x) {
                int ii = idx % ni, c = idx / ni;
                xs[c * 128 + ii] = X[int64_t(c0 + c) * ld + i0 + ii];
            }
            __syncthreads();
            if (r < n)
                for (int ii = 0; ii < ni; ii++) {
                    double2 z = Z[int64_t(i0 + ii) * ldz + r];
                    for (int c = 0; c < nc; c++) {
                        double2 x = xs[c * 128 + ii];
                        acc[c].x += z.x * x.x - z.y * x.y;
                        acc[c].y += z.x * x.y + z.y * x.x;
                    }
                }
        }
        if (r < n)
            for (int c = 0; c < nc; c++) {
                double2 b = B[int64_t(c0 + c) * ld + r];
                Rr[int64_t(c0 + c) * ld + r] = make_double2(b.x - acc[c].x, b.y - acc[c].y);
            }
    }
}

// out[c] = sum_r |V[r,c]|^2, one CTA per column (fixed summation order).
template <typename C>
__global__ void k_colnorm2(int n, const C* V, int64_t ld, double* out) {
    __shared__ double s[32];
    const C* v = V + int64_t(blockIdx.x) * ld;
    double acc = 0.0;
    for (int r = threadIdx.x; r < n; r += blockDim.x) acc += double(v[r].x) * v[r].x + double(v[r].y) * v[r].y;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? s[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[blockIdx.x] = acc;
    }
}

__global__ void k_add_c64_to_c128(int64_t count, const float2* d, double2* x, int init) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= count) return;
    double2 v = make_double2(d[i].x, d[i].y);
    x[i] = init ? v : make_double2(x[i].x + v.x, x[i].y + v.y);
}

// ---------------------------------------------------------------- host side
// With opt.profile_kernels, every trailing-update GEMM is bracketed by a pair
// of CUDA events on the context stream; prof_collect() sums their times.
static cudaEvent_t* prof_pair(frico_gpu_ctx* ctx) {
    if (!ctx->opt.profile_kernels) return nullptr;
    if (ctx->prof_used + 2 > ctx->prof_events.size()) {
        for (int k = 0; k < 64; k++) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            ctx->prof_events.push_back(e);
        }
    }
    cudaEvent_t* p = &ctx->prof_events[ctx->prof_used];
    ctx->prof_used += 2;
    return p;
}

static void prof_collect(frico_gpu_ctx* ctx) {
    if (!ctx->prof_used) return;
    cudaEventSynchronize(ctx->prof_events[ctx->prof_used - 1]);
    for (size_t k = 0; k + 1 < ctx->prof_used; k += 2) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ctx->prof_events[k], ctx->prof_events[k + 1]) == cudaSuccess) {
            ctx->stats.gemm_ms += ms;
            ctx->stats.gemm_launches += 1;
        }
    }
    ctx->prof_used = 0;
}

template <typename R>
static int lu_factor_impl(frico_gpu_ctx* ctx, cplx<R>* A) {
    using C = cplx<R>;
    const int n = int(ctx->n);
    const int64_t lda = ctx->n;
    cudaStream_t st = ctx->stream;
    int rc;
    if ((rc = ensure(ctx, ctx->ipiv, sizeof(int32_t) * n))) return rc;
    if ((rc = ensure(ctx, ctx->perm, sizeof(int32_t) * n))) return rc;
    if ((rc = ensure(ctx, ctx->status, sizeof(DeviceStatus)))) return rc;
    const size_t ws_bytes = 256 + sizeof(R) * 2 * kMaxPanelCTAs + sizeof(int) * 2 * kMaxPanelCTAs +
                            sizeof(C) * 2 * kMaxPanelCTAs * kNB + sizeof(C) * 2 * kNB + 64;
    if ((rc = ensure(ctx, ctx->panel_ws, ws_bytes))) return rc;
    char* wp = (char*)ctx->panel_ws.p;
    PanelWS<R> ws;
    ws.bar = (unsigned*)wp;
    ws.cand_val = (R*)(wp + 256);
    ws.cand_row = (int*)(ws.cand_val + 2 * kMaxPanelCTAs);
    ws.cand_data = (C*)(((uintptr_t)(ws.cand_row + 2 * kMaxPanelCTAs) + 15) & ~uintptr_t(15));
    ws.krow = ws.cand_data + 2 * kMaxPanelCTAs * kNB;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->panel_ws.p, 0, 256, st), "memset ws"))) return rc;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(DeviceStatus), st), "memset status")))
        return rc;
    DeviceStatus* dst = (DeviceStatus*)ctx->status.p;

    int dev_sms = 0, max_smem = 0;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    {
        // dynamic limit = opt-in limit minus the kernel's static shared memory
        cudaFuncAttributes fa;
        if ((rc = cuda_check(ctx, cudaFuncGetAttributes(&fa, k_panel<R>), "panel attributes"))) return rc;
        max_smem -= int(fa.sharedSizeBytes);
        if ((rc = cuda_check(ctx, cudaFuncSetAttribute(k_panel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      max_smem), "panel smem attribute")))
            return rc;
    }
    const size_t trsm_smem = sizeof(C) * (kNB * kNB + 32 * kNB);
    cudaFuncSetAttribute(k_trsm_lower_unit<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(trsm_smem));

    for (int k0 = 0; k0 < n; k0 += kNB) {
        const int jb = std::min(kNB, n - k0);
        const int m = n - k0;
        // CTAs: at least 32 rows each, at most one per SM, shared memory bound.
        int G = std::max(1, std::min(dev_sms, (m + 31) / 32));
        int rows_per = (m + G - 1) / G;
        size_t smem = sizeof(C) * (size_t(rows_per) * jb + 2 * jb);
        while (smem > size_t(max_smem) && G < dev_sms) {
            G++;
            rows_per = (m + G - 1) / G;
            smem = sizeof(C) * (size_t(rows_per) * jb + 2 * jb);
        }
        if (smem > size_t(max_smem)) return set_err(ctx, FRICO_GPU_EINVAL, "matrix too large for panel kernel");
        G = (m + rows_per - 1) / rows_per;
        int maxb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, k_panel<R>, 256, smem);
        if (maxb * dev_sms < G) return set_err(ctx, FRICO_GPU_ECUDA, "panel kernel cannot be co-resident");
        int32_t* ipiv = (int32_t*)ctx->ipiv.p;
        int64_t lda_ = lda;
        int n_ = n, k0_ = k0, jb_ = jb, rp_ = rows_per;
        void* args[] = {&A, &lda_, &n_, &k0_, &jb_, &rp_, &ipiv, &ws, &dst};
        rc = cuda_check(ctx, cudaLaunchCooperativeKernel((void*)k_panel<R>, dim3(G), dim3(256), args, smem, st),
                        "k_panel");
        if (rc) return rc;
        count_launch(ctx);
        if (n - jb > 0) {
            k_laswp<C><<<(n - jb + 255) / 256, 256, 0, st>>>(A, lda, n, k0, jb, ipiv);
            count_launch(ctx);
        }
        const int rest = n - k0 - jb;
        if (rest > 0) {
            k_trsm_lower_unit<C><<<(rest + 31) / 32, 256, trsm_smem, st>>>(A, lda, n, k0, jb);
            C* Cm = A + int64_t(k0 + jb) * lda + k0 + jb;
            const C* Am = A + int64_t(k0) * lda + k0 + jb;
            const C* Bm = A + int64_t(k0 + jb) * lda + k0;
            dim3 gg((rest + 63) / 64, (rest + 63) / 64);
            cudaEvent_t* ev = prof_pair(ctx);
            if (ev) cudaEventRecord(ev[0], st);
            k_gemm_update<R><<<gg, 256, 0, st>>>(Cm, Am, Bm, lda, rest, rest, jb);
            if (ev) {
                cudaEventRecord(ev[1], st);
                ctx->stats.gemm_flops += 8.0 * double(rest) * double(rest) * double(jb);
            }
            count_launch(ctx, 2);
        }
        if ((rc = cuda_check(ctx, cudaGetLastError(), "lu step"))) return rc;
    }
    k_perm_from_ipiv<<<1, 1024, sizeof(int32_t) * n, st>>>(n, (const int32_t*)ctx->ipiv.p, (int32_t*)ctx->perm.p);
    count_launch(ctx);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "k_perm_from_ipiv"))) return rc;
    prof_collect(ctx);
    DeviceStatus hs;
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, st), "status")))
        return rc;
    if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "lu sync"))) return rc;
    if (hs.err == FRICO_DEV_ERR_TIMEOUT) {
        char buf[128];
        snprintf(buf, sizeof buf, "panel barrier timed out at row %d", hs.where);
        return set_err(ctx, FRICO_GPU_ETIMEOUT, buf);
    }
    ctx->info = hs.info;
    return FRICO_GPU_OK;
}

int lu_factor_fp64(frico_gpu_ctx* ctx) { return lu_factor_impl<double>(ctx, (double2*)ctx->z64.p); }
int lu_factor_fp32(frico_gpu_ctx* ctx) { return lu_factor_impl<float>(ctx, (float2*)ctx->z32.p); }

// Solve in place on W (already row-permuted): L then U.
template <typename C>
static int trsv_all(frico_gpu_ctx* ctx, const C* LU, C* W, int nrhs, int64_t ldw) {
    const int n = int(ctx->n);
    cudaStream_t st = ctx->stream;
    for (int kb = 0; kb < n; kb += kTB) {
        int nb = std::min(kTB, n - kb);
        int below = n - kb - nb;
        int grid = std::max(1, (below + 255) / 256);
        k_trsv_lower<C><<<grid, 256, 0, st>>>(LU, n, n, kb, nb, W, ldw, nrhs);
        count_launch(ctx);
    }
    int last = ((n - 1) / kTB) * kTB;
    for (int kb = last; kb >= 0; kb -= kTB) {
        int nb = std::min(kTB, n - kb);
        int grid = std::max(1, (kb + 255) / 256);
        k_trsv_upper<C><<<grid, 256, 0, st>>>(LU, n, n, kb, nb, W, ldw, nrhs);
        count_launch(ctx);
    }
    return cuda_check(ctx, cudaGetLastError(), "trsv");
}

// X = A^{-1} B (FP64 factors in z64), B n x nrhs (device), result into B.
int lu_solve_fp64(frico_gpu_ctx* ctx, double2* B, int nrhs, int64_t ldb) {
    int rc;
    const int64_t n = ctx->n;
    if ((rc = ensure(ctx, ctx->rwork, sizeof(double2) * n * nrhs))) return rc;
    double2* W = (double2*)ctx->rwork.p;
    int64_t cnt = n * nrhs;
    k_gather_rows<double2, double2><<<unsigned((cnt + 255) / 256), 256, 0, ctx->stream>>>(
        int(n), nrhs, (const int32_t*)ctx->perm.p, B, ldb, W, n);
    count_launch(ctx);
    if ((rc = trsv_all<double2>(ctx, (const double2*)ctx->z64.p, W, nrhs, n))) return rc;
    for (int c = 0; c < nrhs; c++)
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(B + c * ldb, W + c * n, sizeof(double2) * n,
                                                  cudaMemcpyDeviceToDevice, ctx->stream), "copy X")))
            return rc;
    return FRICO_GPU_OK;
}

// Mixed precision: X solves Z64 X = B with complex64 LU factors (z32) and FP64
// residuals r = B - Z64 X (classical iterative refinement).
int refine_solve(frico_gpu_ctx* ctx) {
    int rc;
    const int64_t n = ctx->n;
    const int nrhs = ctx->nrhs;
    const int64_t cnt = n * nrhs;
    cudaStream_t st = ctx->stream;
    if ((rc = ensure(ctx, ctx->sol, sizeof(double2) * cnt))) return rc;
    if ((rc = ensure(ctx, ctx->rwork, sizeof(double2) * cnt))) return rc;
    if ((rc = ensure(ctx, ctx->dwork32, sizeof(float2) * cnt))) return rc;
    if ((rc = ensure(ctx, ctx->norms, sizeof(double) * 2 * nrhs))) return rc;
    const double2* B = (const double2*)ctx->rhs.p;
    double2* X = (double2*)ctx->sol.p;
    double2* Rr = (double2*)ctx->rwork.p;
    float2* W = (float2*)ctx->dwork32.p;
    double* nrm = (double*)ctx->norms.p;
    const float2* LU = (const float2*)ctx->z32.p;
    const int max_it = ctx->opt.max_refine_iters > 0 ? ctx->opt.max_refine_iters : 30;
    const double tol = ctx->opt.refine_tol > 0 ? ctx->opt.refine_tol : 1e-12;
    std::vector<double> hn(2 * nrhs);
    k_colnorm2<double2><<<nrhs, 256, 0, st>>>(int(n), B, n, nrm + nrhs);
    count_launch(ctx);
    const double2* src = B;
    double prev = 1e300, rel = 1e300;
    int it = 0;
    for (; it < max_it; it++) {
        k_gather_rows<double2, float2><<<unsigned((cnt + 255) / 256), 256, 0, st>>>(
            int(n), nrhs, (const int32_t*)ctx->perm.p, src, n, W, n);
        if ((rc = trsv_all<float2>(ctx, LU, W, nrhs, n))) return rc;
        k_add_c64_to_c128<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(cnt, W, X, it == 0);
        k_residual<<<unsigned((n + 255) / 256), 256, 0, st>>>((const double2*)ctx->z64.p, n, int(n), X, B, Rr,
                                                             n, nrhs);
        k_colnorm2<double2><<<nrhs, 256, 0, st>>>(int(n), Rr, n, nrm);
        count_launch(ctx, 4);
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * 2 * nrhs,
                                                  cudaMemcpyDeviceToHost, st), "norms")))
            return rc;
        if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "refine sync"))) return rc;
        rel = 0.0;
        for (int c = 0; c < nrhs; c++) {
            double bn = hn[nrhs + c] > 0 ? std::sqrt(hn[nrhs + c]) : 1.0;
            rel = std::max(rel, std::sqrt(hn[c]) / bn);
        }
        src = Rr;
        if (rel <= tol) { it++; break; }
        if (it >= 2 && rel > 0.5 * prev) { it++; break; }  // stagnation
        prev = rel;
    }
    ctx->stats.refine_iters = it;
    ctx->stats.refine_residual = rel;
    if (!(rel <= tol) && !(rel < 1e-9)) {
        char buf[128];
        snprintf(buf, sizeof buf, "refinement stopped at residual %.3e after %d sweeps", rel, it);
        return set_err(ctx, FRICO_GPU_ENOCONV, buf);
    }
    return FRICO_GPU_OK;
}

}  // namespace frico
