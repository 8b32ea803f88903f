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
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <cstdio>

#include "common.cuh"

namespace frico {

static const int kNB = 64;          // LU block width
static const int kMaxPanelCTAs = 1024;

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
__device__ bool grid_barrier(unsigned* bar, DeviceStatus* st, int where, long long lim) {
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
                if (clock64() - t0 > lim) {
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
                                              DeviceStatus* st, long long lim) {
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
    if (!grid_barrier(ws.bar, st, k0, lim)) return;

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
            // thread = (row lane of 64, column group of 4): no integer division
            for (int cc = c + 1 + (tid >> 6); cc < jb; cc += 4) {
                const C u = prow[cc];
                for (int r = rs + (tid & 63); r < nr; r += 64)
                    sm[cc * rows_per + r] = cfms(sm[cc * rows_per + r], sm[c * rows_per + r], u);
            }
        __syncthreads();
        if (c + 1 < jb) {
            publish(c + 1, par ^ 1);
            if (!grid_barrier(ws.bar, st, k + 1, lim)) return;
        }
    }
    for (int idx = tid; idx < nr * jb; idx += blockDim.x) {
        int r = idx % nr, c = idx / nr;
        A[int64_t(k0 + c) * lda + r0 + r] = sm[c * rows_per + r];
    }
}

// Panel leaf on one thread-block cluster (<= 16 CTAs). The rows [k0, n) of
// columns [k0, k0+jb) are split across the cluster's CTAs and stay in shared
// memory for the whole leaf. Per column: each CTA publishes its pivot
// candidate (value, row, the row itself) and, if it owns row k, row k in its
// own shared memory (two parity slots); one hardware cluster barrier; then
// every CTA reads the candidates of all CTAs through distributed shared
// memory, picks the pivot (max |re|+|im|, lowest row on ties, as izamax),
// swaps, scales and applies the rank-1 update to its rows. Parity slots make
// one barrier per column sufficient: slot c&1 is rewritten only at column c+2,
// after every CTA has passed barrier c+1.
template <typename R>
__global__ void __launch_bounds__(256) k_panel_cluster(cplx<R>* A, int64_t lda, int n, int k0, int jb, int rows_per,
                                                      int32_t* ipiv, DeviceStatus* st) {
    using C = cplx<R>;
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char smraw[];
    C* sm = (C*)smraw;                         // [jb][rows_per]
    C* cdata = sm + size_t(jb) * rows_per;     // [2][jb] candidate row
    C* kdata = cdata + 2 * jb;                 // [2][jb] row k (owner only)
    C* prow = kdata + 2 * jb;                  // [jb] pivot row (local copy)
    C* krow = prow + jb;                       // [jb] old row k (local copy)
    __shared__ R cval[2];
    __shared__ int crow[2];
    __shared__ R s_val;
    __shared__ int s_row, s_p, s_g;
    const int g = int(cluster.block_rank()), tid = threadIdx.x, G = int(cluster.num_blocks());
    const int r0 = k0 + g * rows_per;
    const int nr = max(0, min(n, r0 + rows_per) - r0);

    for (int idx = tid; idx < nr * jb; idx += blockDim.x) {
        int r = idx % nr, c = idx / nr;
        sm[c * rows_per + r] = A[int64_t(k0 + c) * lda + r0 + r];
    }
    __syncthreads();

    auto publish = [&](int c, int par) {
        const int k = k0 + c;
        block_argmax<R>(sm + c * rows_per, max(0, k - r0), nr, &s_val, &s_row);
        if (tid == 0) {
            cval[par] = s_val;
            crow[par] = s_val >= R(0) ? r0 + s_row : 0x7fffffff;
        }
        if (s_val >= R(0))
            for (int cc = tid; cc < jb; cc += blockDim.x) cdata[par * jb + cc] = sm[cc * rows_per + s_row];
        if (k >= r0 && k < r0 + nr)
            for (int cc = tid; cc < jb; cc += blockDim.x) kdata[par * jb + cc] = sm[cc * rows_per + (k - r0)];
    };

    publish(0, 0);
    for (int c = 0; c < jb; c++) {
        const int k = k0 + c, par = c & 1;
        cluster.sync();
        if (tid < 32) {
            R bv = R(-1);
            int brow = 0x7fffffff, bg = 0;
            if (tid < G) {
                R* rv = cluster.map_shared_rank(cval, tid);
                int* rr = cluster.map_shared_rank(crow, tid);
                bv = rv[par];
                brow = rr[par];
                bg = tid;
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
        const int kown = (k - k0) / rows_per;
        {
            const C* rc = cluster.map_shared_rank(cdata, wg) + par * jb;
            const C* rk = cluster.map_shared_rank(kdata, kown) + par * jb;
            for (int cc = tid; cc < jb; cc += blockDim.x) {
                prow[cc] = rc[cc];
                krow[cc] = rk[cc];
            }
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
            // thread = (row lane of 64, column group of 4): no integer division
            for (int cc = c + 1 + (tid >> 6); cc < jb; cc += 4) {
                const C u = prow[cc];
                for (int r = rs + (tid & 63); r < nr; r += 64)
                    sm[cc * rows_per + r] = cfms(sm[cc * rows_per + r], sm[c * rows_per + r], u);
            }
        __syncthreads();
        if (c + 1 < jb) publish(c + 1, par ^ 1);
    }
    for (int idx = tid; idx < nr * jb; idx += blockDim.x) {
        int r = idx % nr, c = idx / nr;
        A[int64_t(k0 + c) * lda + r0 + r] = sm[c * rows_per + r];
    }
    cluster.sync();   // no CTA leaves while others may still read its shared memory
}

// Row interchanges k <-> ipiv[k]-1 for k in [p0, p1), applied to columns [c0, c1).
template <typename C>
__global__ void k_laswp_range(C* A, int64_t lda, int c0, int c1, int p0, int p1, const int32_t* ipiv) {
    int col = c0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= c1) return;
    C* a = A + int64_t(col) * lda;
    for (int k = p0; k < p1; k++) {
        int p = ipiv[k] - 1;
        if (p != k) {
            C x = a[k];
            a[k] = a[p];
            a[p] = x;
        }
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
// B is stored row-major with the 32 columns contiguous, so the 32 lanes of a
// warp (one column each) touch 32 consecutive words; L reads are broadcasts.
template <typename C>
__global__ void __launch_bounds__(256) k_trsm_lower_unit(C* A, int64_t lda, int k0, int jb, int cb, int ce) {
    extern __shared__ __align__(16) unsigned char smraw[];
    C* L = (C*)smraw;           // [jb][jb] column-major
    C* B = L + jb * jb;         // [jb rows][32 cols]
    const int c0 = cb + blockIdx.x * 32;
    const int nc = min(32, ce - c0);
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) {
        int r = idx % jb, c = idx / jb;
        L[idx] = A[int64_t(k0 + c) * lda + k0 + r];
    }
    for (int idx = threadIdx.x; idx < jb * nc; idx += blockDim.x) {
        int r = idx % jb, c = idx / jb;
        B[r * 32 + c] = A[int64_t(c0 + c) * lda + k0 + r];
    }
    __syncthreads();
    const int lc = threadIdx.x & 31, rg = threadIdx.x >> 5;
    for (int q = 0; q < jb; q++) {
        if (lc < nc) {
            C xq = B[q * 32 + lc];
            for (int r = q + 1 + rg; r < jb; r += 8) B[r * 32 + lc] = cfms(B[r * 32 + lc], L[q * jb + r], xq);
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < jb * nc; idx += blockDim.x) {
        int r = idx % jb, c = idx / jb;
        A[int64_t(c0 + c) * lda + k0 + r] = B[r * 32 + c];
    }
}

// C[m x nn] -= A[m x kk] * B[kk x nn], all column-major with leading dim lda.
// 64x64 CTA tile, 16 k-slab, 256 threads, each thread 4x4 complex outputs
// (rows tx + 16*i, cols ty + 16*j: conflict-free shared-memory reads).
template <typename R>
__global__ void __launch_bounds__(256) k_gemm_update(cplx<R>* Cm, int64_t ldc, const cplx<R>* Am, int64_t lda,
                                                     const cplx<R>* Bm, int64_t ldb, int m, int nn, int kk) {
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
            Bs[br][bc] = (gbr < kk && gbc < nn) ? Bm[int64_t(gbc) * ldb + gbr] : cmake(R(0), R(0));
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
                    cmac(acc[i][j], a[i], b[j]);
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
                C* p = Cm + int64_t(gc) * ldc + gr;
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

static const int kTR = 8;    // RHS columns per residual pass

// Column chunks of the residual / matvec kernels: about 4 CTAs per SM in all, chunks of
// at least 32 columns (smaller systems get more chunks rather than idle SMs: the FP64
// pipe, not the bandwidth, bounds these products on this part).
static int residual_chunks(int n, int sms, int rblocks) {
    return std::max(1, std::min(n / 32, (4 * sms + rblocks - 1) / rblocks));
}

// Partial products of the FP64 refinement residual. The FP64 pipe is narrow on
// this part, so the work is spread over rows (256 per CTA) and over column
// chunks (blockIdx.y): part[(y * nrhs + c) * n + r] = sum_{i in chunk y} Z[r, i] X[i, c].
__global__ void __launch_bounds__(256) k_residual_part(const double2* __restrict__ Z, int64_t ldz, int n,
                                                      const double2* __restrict__ X, int64_t ld, int nrhs,
                                                      int chunk, double2* __restrict__ part) {
    __shared__ double2 xs[128 * kTR];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    for (int c0 = 0; c0 < nrhs; c0 += kTR) {
        const int nc = min(kTR, nrhs - c0);
        double2 acc[kTR];
#pragma unroll
        for (int c = 0; c < kTR; c++) acc[c] = make_double2(0, 0);
        for (int i0 = j0; i0 < j1; i0 += 128) {
            const int ni = min(128, j1 - i0);
            __syncthreads();
            for (int idx = threadIdx.x; idx < ni * nc; idx += blockDim.x) {
                int ii = idx % ni, c = idx / ni;
                xs[c * 128 + ii] = X[int64_t(c0 + c) * ld + i0 + ii];
            }
            __syncthreads();
            if (r < n) {
                const double2* zp = Z + int64_t(i0) * ldz + r;
                if (nc == 1) {
#pragma unroll 8
                    for (int ii = 0; ii < ni; ii++) {
                        double2 z = zp[int64_t(ii) * ldz];
                        double2 x = xs[ii];
                        cmac(acc[0], z, x);
                    }
                } else {
                    for (int ii = 0; ii < ni; ii++) {
                        double2 z = zp[int64_t(ii) * ldz];
#pragma unroll
                        for (int c = 0; c < kTR; c++)
                            if (c < nc) {
                                double2 x = xs[c * 128 + ii];
                                cmac(acc[c], z, x);
                            }
                    }
                }
            }
        }
        if (r < n)
#pragma unroll
            for (int c = 0; c < kTR; c++)
                if (c < nc) part[(int64_t(blockIdx.y) * nrhs + c0 + c) * n + r] = acc[c];
    }
}

// The same partial products in double-float arithmetic on the FP32 pipe, which
// is many times wider than the FP64 one on this part. Every FP64 value d is
// split by integer operations into FP32 h + l: h = d with its significand
// truncated to 24 bits, l = the remaining 29 bits rounded down to 23 (|d - h - l|
// <= 2^-47 |d|). A product a b = (a1 + a2)(b1 + b2) is a1 b1 as an FP32 value
// p plus its exact rounding error (one FMA) plus the cross terms a1 b2 + a2 b1
// (a2 b2 < 2^-47 |a b| is dropped); p enters the running sum s by an exact
// two-sum whose error goes to the compensation t with the small terms. (s, t)
// is renormalised every 4 terms and flushed into FP64 every 32, so the
// accumulated error stays below about 32 * 2^-47 of the sum of |Z[r, i] X[i]|
// over a flush block (FP64 summation: 2^-53 per term).
// An exponent outside [-100, 127] (values beyond about 1e-30 .. 3e38, or not
// finite) sets st->df_range; the caller then recomputes with k_residual_part.
// (split_df, df_mac and df_renorm are in common.cuh.)
// NC right-hand sides per pass (1, 2, 4 or 8: register use grows with NC);
// 8 entries of Z are loaded ahead of their use. Of every 8 entries, the last
// kResidualF64<NC> go through the FP64 pipe instead (four DFMAs into the FP64
// sum), which the double-float arithmetic leaves idle: a DFMA warp-instruction
// takes about 80 cycles of a sub-partition's FP64 pipe on this part, a
// double-float product about 12 issue slots, so the two finish together near
// 2 of 8 entries for one right-hand side and 1 of 8 for eight (the split of Z
// is shared by the right-hand sides, the DFMAs are not).
template <int NC> constexpr int kResidualF64 = NC <= 2 ? 2 : 1;

template <int NC>
__global__ void __launch_bounds__(256) k_residual_part_df(const double2* __restrict__ Z, int64_t ldz, int n,
                                                         const double2* __restrict__ X, int64_t ld, int nrhs,
                                                         int chunk, double2* __restrict__ part, DeviceStatus* st) {
    constexpr int F64 = kResidualF64<NC>, DF = 8 - F64;   // entries per 8 through FP64 / double-float
    __shared__ float4 xs[128 * NC];   // (re hi, re lo, im hi, im lo) of X[i0 + ii, c0 + c]
    __shared__ double2 xd[128 * NC];  // the same in FP64
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    int bad = 0;
    for (int c0 = 0; c0 < nrhs; c0 += NC) {
        const int nc = min(NC, nrhs - c0);
        double2 acc[NC];
        float sr[NC], tr[NC], si[NC], ti[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) {
            acc[c] = make_double2(0, 0);
            sr[c] = tr[c] = si[c] = ti[c] = 0.f;
        }
        for (int i0 = j0; i0 < j1; i0 += 128) {
            const int ni = min(128, j1 - i0);
            __syncthreads();
            for (int idx = threadIdx.x; idx < ni * nc; idx += blockDim.x) {
                const int ii = idx % ni, c = idx / ni;
                const double2 x = X[int64_t(c0 + c) * ld + i0 + ii];
                float4 q;
                split_df(x.x, q.x, q.y, bad);
                split_df(x.y, q.z, q.w, bad);
                xs[c * 128 + ii] = q;
                xd[c * 128 + ii] = x;
            }
            __syncthreads();
            if (r < n) {
                const double2* zp = Z + int64_t(i0) * ldz + r;
#pragma unroll 1
                for (int b0 = 0; b0 < ni; b0 += 32) {
                    const int be = min(b0 + 32, ni);
#pragma unroll 1
                    for (int ii = b0; ii < be; ii += 8) {
                        double2 zz[8];
#pragma unroll
                        for (int u = 0; u < 8; u++)
                            zz[u] = ii + u < be ? zp[int64_t(ii + u) * ldz] : make_double2(0, 0);
#pragma unroll
                        for (int u = 0; u < 8; u++) {
                            if (ii + u >= be) break;
                            if (u >= DF) {   // FP64 pipe
#pragma unroll
                                for (int c = 0; c < NC; c++)
                                    if (NC == 1 || c < nc) cmac(acc[c], zz[u], xd[c * 128 + ii + u]);
                                continue;
                            }
                            float zr1, zr2, zi1, zi2;
                            split_df(zz[u].x, zr1, zr2, bad);
                            split_df(zz[u].y, zi1, zi2, bad);
#pragma unroll
                            for (int c = 0; c < NC; c++)
                                if (NC == 1 || c < nc) {
                                    const float4 x = xs[c * 128 + ii + u];
                                    df_mac(sr[c], tr[c], zr1, zr2, x.x, x.y);     // Re += zr xr - zi xi
                                    df_mac(sr[c], tr[c], -zi1, -zi2, x.z, x.w);
                                    df_mac(si[c], ti[c], zr1, zr2, x.z, x.w);     // Im += zr xi + zi xr
                                    df_mac(si[c], ti[c], zi1, zi2, x.x, x.y);
                                    if (u == 3 || u == DF - 1) {
                                        df_renorm(sr[c], tr[c]);
                                        df_renorm(si[c], ti[c]);
                                    }
                                }
                        }
                    }
#pragma unroll
                    for (int c = 0; c < NC; c++)
                        if (NC == 1 || c < nc) {
                            acc[c].x += double(sr[c]) + double(tr[c]);
                            acc[c].y += double(si[c]) + double(ti[c]);
                            sr[c] = tr[c] = si[c] = ti[c] = 0.f;
                        }
                }
            }
        }
        if (r < n)
#pragma unroll
            for (int c = 0; c < NC; c++)
                if (c < nc) part[(int64_t(blockIdx.y) * nrhs + c0 + c) * n + r] = acc[c];
    }
    if (bad) atomicOr(&st->df_range, 1);
}

// R = B - sum over chunks of the partial products (fixed chunk order).
__global__ void k_residual_reduce(int n, int nrhs, int nchunks, const double2* __restrict__ part,
                                  const double2* __restrict__ B, int64_t ld, double2* __restrict__ Rr) {
    int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= int64_t(n) * nrhs) return;
    int r = int(idx % n), c = int(idx / n);
    double2 acc = make_double2(0, 0);
    for (int y = 0; y < nchunks; y++) acc = cadd(acc, part[(int64_t(y) * nrhs + c) * n + r]);
    double2 b = B[int64_t(c) * ld + r];
    Rr[int64_t(c) * ld + r] = make_double2(b.x - acc.x, b.y - acc.y);
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
cudaEvent_t* prof_event_pair(frico_gpu_ctx* ctx) {
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

void prof_event_collect(frico_gpu_ctx* ctx) {
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

// Host-side launcher for one factorisation: recursive panel (zgetrf2-style
// halving down to a leaf that fits one thread-block cluster), interchanges,
// triangular solve and trailing GEMM.
template <typename R> struct LuDriver {
    using C = cplx<R>;
    frico_gpu_ctx* ctx;
    C* A;
    int64_t lda;
    int n;
    cudaStream_t st;
    PanelWS<R> ws;
    DeviceStatus* dst;
    int dev_sms = 0, coop_smem = 0, cl_smem = 0, cl_max = 8;
    size_t trsm_smem = 0;
    bool use_tc = false;

    int init() {
        int rc;
        cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device);
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
        cudaFuncAttributes fa;
        if ((rc = cuda_check(ctx, cudaFuncGetAttributes(&fa, k_panel<R>), "panel attributes"))) return rc;
        coop_smem = optin - int(fa.sharedSizeBytes);
        if ((rc = cuda_check(ctx, cudaFuncSetAttribute(k_panel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      coop_smem), "panel smem attribute")))
            return rc;
        if ((rc = cuda_check(ctx, cudaFuncGetAttributes(&fa, k_panel_cluster<R>), "cluster attributes"))) return rc;
        cl_smem = optin - int(fa.sharedSizeBytes);
        if ((rc = cuda_check(ctx, cudaFuncSetAttribute(k_panel_cluster<R>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize, cl_smem),
                             "cluster smem attribute")))
            return rc;
        cl_max = 8;
        if (cudaFuncSetAttribute(k_panel_cluster<R>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess)
            cl_max = 16;
        else
            cudaGetLastError();
        // largest cluster that can actually be placed with a full shared-memory budget
        for (; cl_max > 1; cl_max /= 2) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(cl_max);
            cfg.blockDim = dim3(256);
            cfg.dynamicSmemBytes = size_t(cl_smem);
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = cl_max;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int num = 0;
            if (cudaOccupancyMaxActiveClusters(&num, k_panel_cluster<R>, &cfg) == cudaSuccess && num > 0) break;
            cudaGetLastError();
        }
        trsm_smem = sizeof(C) * (kNB * kNB + 32 * kNB);
        const int eng = ctx->opt.gemm_engine;
        use_tc = sizeof(R) == 4 && eng != FRICO_GEMM_SIMT && gemm_tc_available(ctx);
        if ((eng == FRICO_GEMM_TC || eng == FRICO_GEMM_TC_F16) && sizeof(R) == 4 && !use_tc)
            return set_err(ctx, FRICO_GPU_EINVAL, "tensor-core GEMM engine not available on this device");
        // never below what the unpivoted complex64 path needs (128-wide blocks, trsm_lower_unit_f32):
        // the attribute belongs to the kernel on this device, not to this factorisation
        const size_t attr = sizeof(R) == 4 ? std::max(trsm_smem, sizeof(C) * (128 * 128 + 32 * 128)) : trsm_smem;
        return cuda_check(ctx, cudaFuncSetAttribute(k_trsm_lower_unit<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    int(attr)), "trsm smem attribute");
    }

    // Widest leaf (<= w, power of two >= 8) the cluster kernel can hold for m rows; 0 if none.
    int leaf_width(int m, int w, int* cl, int* rows_per) const {
        int CL = std::max(1, std::min(cl_max, (m + 63) / 64));
        int rp = (m + CL - 1) / CL;
        for (int lw = std::min(w, sizeof(R) == 4 ? 32 : 16); lw >= 8; lw /= 2) {
            size_t smem = sizeof(C) * (size_t(rp) * lw + 6 * lw);
            if (smem <= size_t(cl_smem)) {
                *cl = (m + rp - 1) / rp;
                *rows_per = rp;
                return lw;
            }
        }
        return 0;
    }

    int leaf_cluster(int k0, int w, int CL, int rows_per) {
        size_t smem = sizeof(C) * (size_t(rows_per) * w + 6 * w);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL);
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CL;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int32_t* ipiv = (int32_t*)ctx->ipiv.p;
        count_launch(ctx);
        return cuda_check(ctx, cudaLaunchKernelEx(&cfg, k_panel_cluster<R>, A, lda, n, k0, w, rows_per, ipiv, dst),
                          "k_panel_cluster");
    }

    int leaf_coop(int k0, int w) {
        const int m = n - k0;
        int G = std::max(1, std::min(dev_sms, (m + 31) / 32));
        int rows_per = (m + G - 1) / G;
        size_t smem = sizeof(C) * (size_t(rows_per) * w + 2 * w);
        while (smem > size_t(coop_smem) && G < dev_sms) {
            G++;
            rows_per = (m + G - 1) / G;
            smem = sizeof(C) * (size_t(rows_per) * w + 2 * w);
        }
        if (smem > size_t(coop_smem)) return set_err(ctx, FRICO_GPU_EINVAL, "matrix too large for panel kernel");
        G = (m + rows_per - 1) / rows_per;
        int maxb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, k_panel<R>, 256, smem);
        if (maxb * dev_sms < G) return set_err(ctx, FRICO_GPU_ECUDA, "panel kernel cannot be co-resident");
        int32_t* ipiv = (int32_t*)ctx->ipiv.p;
        int64_t lda_ = lda;
        int n_ = n, k0_ = k0, w_ = w, rp_ = rows_per;
        PanelWS<R> ws_ = ws;
        DeviceStatus* dst_ = dst;
        long long lim = wait_limit(ctx);
        void* args[] = {&A, &lda_, &n_, &k0_, &w_, &rp_, &ipiv, &ws_, &dst_, &lim};
        count_launch(ctx);
        return cuda_check(ctx, cudaLaunchCooperativeKernel((void*)k_panel<R>, dim3(G), dim3(256), args, smem, st),
                          "k_panel");
    }

    void laswp(int c0, int c1, int p0, int p1) {
        if (c1 <= c0 || p1 <= p0) return;
        k_laswp_range<C><<<(c1 - c0 + 127) / 128, 128, 0, st>>>(A, lda, c0, c1, p0, p1, (const int32_t*)ctx->ipiv.p);
        count_launch(ctx);
    }

    // A[k0:k0+w, cb:ce] <- L11^{-1} A[k0:k0+w, cb:ce], L11 unit lower at (k0, k0)
    void trsm(int k0, int w, int cb, int ce) {
        if (ce <= cb) return;
        k_trsm_lower_unit<C><<<(ce - cb + 31) / 32, 256, trsm_smem, st>>>(A, lda, k0, w, cb, ce);
        count_launch(ctx);
    }

    // A[r0:r0+m, c0:c0+nn] -= A[r0:r0+m, k0:k0+kk] * A[k0:k0+kk, c0:c0+nn]
    int gemm(int r0, int c0, int m, int nn, int k0, int kk, bool profile) {
        if (m <= 0 || nn <= 0) return FRICO_GPU_OK;
        C* Cm = A + int64_t(c0) * lda + r0;
        const C* Am = A + int64_t(k0) * lda + r0;
        const C* Bm = A + int64_t(c0) * lda + k0;
        dim3 gg((m + 63) / 64, (nn + 63) / 64);
        cudaEvent_t* ev = profile ? prof_event_pair(ctx) : nullptr;
        if (ev) {
            ctx->stats.gemm_flops += 8.0 * double(m) * double(nn) * double(kk);
            ctx->stats.gemm_bytes += sizeof(C) * (2.0 * double(m) * double(nn) + double(m + nn) * kk);
        }
        if (sizeof(R) == 4 && profile && use_tc && m >= 128 && nn >= 128) {
            // outer trailing update on the tensor cores (events bracket the MMA kernel)
            int rc = gemm_update_tc(ctx, (float2*)Cm, lda, (const float2*)Am, lda, (const float2*)Bm, lda, m, nn,
                                    kk, ev);
            if (rc) return rc;
            return FRICO_GPU_OK;
        }
        if (ev) cudaEventRecord(ev[0], st);
        k_gemm_update<R><<<gg, 256, 0, st>>>(Cm, lda, Am, lda, Bm, lda, m, nn, kk);
        if (ev) cudaEventRecord(ev[1], st);
        count_launch(ctx);
        return FRICO_GPU_OK;
    }

    // Factor columns [k0, k0+w) of rows [k0, n), interchanges applied inside the panel.
    int panel(int k0, int w) {
        const int m = n - k0;
        int CL = 0, rp = 0;
        int lw = leaf_width(m, w, &CL, &rp);
        if (lw == 0) return leaf_coop(k0, w);
        if (w <= lw) return leaf_cluster(k0, w, CL, rp);
        const int w1 = w / 2, w2 = w - w1;
        int rc;
        if ((rc = panel(k0, w1))) return rc;
        laswp(k0 + w1, k0 + w, k0, k0 + w1);
        trsm(k0, w1, k0 + w1, k0 + w);
        if ((rc = gemm(k0 + w1, k0 + w1, m - w1, w2, k0, w1, false))) return rc;
        if ((rc = panel(k0 + w1, w2))) return rc;
        laswp(k0, k0 + w1, k0 + w1, k0 + w);
        return FRICO_GPU_OK;
    }
};

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

    LuDriver<R> drv;
    drv.ctx = ctx;
    drv.A = A;
    drv.lda = lda;
    drv.n = n;
    drv.st = st;
    drv.ws = ws;
    drv.dst = dst;
    if ((rc = drv.init())) return rc;
    int32_t* ipiv = (int32_t*)ctx->ipiv.p;
    for (int k0 = 0; k0 < n; k0 += kNB) {
        const int jb = std::min(kNB, n - k0);
        if ((rc = drv.panel(k0, jb))) return rc;
        // the panel's interchanges on the columns left and right of it
        if (k0 > 0) drv.laswp(0, k0, k0, k0 + jb);
        if (k0 + jb < n) drv.laswp(k0 + jb, n, k0, k0 + jb);
        const int rest = n - k0 - jb;
        if (rest > 0) {
            drv.trsm(k0, jb, k0 + jb, n);
            if ((rc = drv.gemm(k0 + jb, k0 + jb, rest, rest, k0, jb, true))) return rc;
        }
        if ((rc = cuda_check(ctx, cudaGetLastError(), "lu step"))) return rc;
    }
    k_perm_from_ipiv<<<1, 1024, sizeof(int32_t) * n, st>>>(n, (const int32_t*)ctx->ipiv.p, (int32_t*)ctx->perm.p);
    count_launch(ctx);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "k_perm_from_ipiv"))) return rc;
    prof_event_collect(ctx);
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
    if (hs.info != 0) return FRICO_GPU_OK;   // singular: no solve will follow
    // clear the status word for the solves, then invert the diagonal blocks
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(DeviceStatus), st), "status reset")))
        return rc;
    return sizeof(R) == 8 ? trsv_prepare_fp64(ctx) : trsv_prepare_fp32(ctx);
}

int lu_factor_fp64(frico_gpu_ctx* ctx) { return lu_factor_impl<double>(ctx, (double2*)ctx->z64.p); }
int lu_factor_fp32(frico_gpu_ctx* ctx) { return lu_factor_impl<float>(ctx, (float2*)ctx->z32.p); }

// A[k0:k0+jb, cb:ce] <- L11^{-1} A[k0:k0+jb, cb:ce] (unit lower L11 at (k0, k0)), jb <= 128.
int trsm_lower_unit_f32(frico_gpu_ctx* ctx, float2* A, int64_t lda, int k0, int jb, int cb, int ce) {
    if (ce <= cb) return FRICO_GPU_OK;
    const size_t smem = sizeof(float2) * (size_t(jb) * jb + 32 * jb);
    if (jb > 128) return set_err(ctx, FRICO_GPU_EINVAL, "trsm_lower_unit_f32: block wider than 128");
    if (int rc = device_once(ctx, kOnceTrsmLower, [](frico_gpu_ctx* c) {
            return cuda_check(c, cudaFuncSetAttribute(k_trsm_lower_unit<float2>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      int(sizeof(float2) * (128 * 128 + 32 * 128))),
                              "trsm smem attribute");
        }))
        return rc;
    k_trsm_lower_unit<float2><<<(ce - cb + 31) / 32, 256, smem, ctx->stream>>>(A, lda, k0, jb, cb, ce);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_trsm_lower_unit");
}

int gemm_update_simt32(frico_gpu_ctx* ctx, float2* C, int64_t ldc, const float2* L, int64_t ldl, const float2* U,
                       int64_t ldu, int m, int n, int k) {
    if (m <= 0 || n <= 0) return FRICO_GPU_OK;
    dim3 gg((m + 63) / 64, (n + 63) / 64);
    k_gemm_update<float><<<gg, 256, 0, ctx->stream>>>(C, ldc, L, ldl, U, ldu, m, n, k);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_gemm_update");
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
    if ((rc = trsv_solve_fp64(ctx, W, nrhs, n))) return rc;
    if ((rc = trsv_check(ctx))) return rc;
    for (int c = 0; c < nrhs; c++)
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(B + c * ldb, W + c * n, sizeof(double2) * n,
                                                  cudaMemcpyDeviceToDevice, ctx->stream), "copy X")))
            return rc;
    return FRICO_GPU_OK;
}

__global__ void k_add_c128(int64_t count, const double2* __restrict__ d, double2* __restrict__ x) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < count) x[i] = cadd(x[i], d[i]);
}

// One step of FP64 iterative refinement of the FP64 drop-in's solution X (n x nrhs,
// ld n) of Zk X = B, Zk the matrix the resident factors came from (kept before the
// in-place factorisation): R = B - Zk X, X += (LU)^{-1} R. The chained solves apply
// explicit inverses of their 64 x 64 diagonal blocks, which is not backward stable
// when those blocks are ill-conditioned (the EFIE at low frequency); one step brings
// the backward error to that of a substitution solve such as LAPACK's zgetrs.
int refine_fp64_once(frico_gpu_ctx* ctx, const double2* Zk, const double2* B, double2* X) {
    const int64_t n = ctx->n;
    const int nrhs = ctx->nrhs;
    const int64_t cnt = n * nrhs;
    cudaStream_t st = ctx->stream;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const unsigned rblocks = unsigned((n + 255) / 256);
    int nchunks = residual_chunks(int(n), sms, int(rblocks));
    const int chunk = int((n + nchunks - 1) / nchunks);
    nchunks = int((n + chunk - 1) / chunk);
    int rc;
    if ((rc = ensure(ctx, ctx->rwork32, sizeof(double2) * size_t(nchunks) * nrhs * n))) return rc;
    if ((rc = ensure(ctx, ctx->res64, sizeof(double2) * cnt))) return rc;
    double2* part = (double2*)ctx->rwork32.p;
    double2* R = (double2*)ctx->res64.p;
    k_residual_part<<<dim3(rblocks, nchunks), 256, 0, st>>>(Zk, n, int(n), X, n, nrhs, chunk, part);
    k_residual_reduce<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(int(n), nrhs, nchunks, part, B, n, R);
    count_launch(ctx, 2);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "fp64 refinement residual"))) return rc;
    if ((rc = lu_solve_fp64(ctx, R, nrhs, n))) return rc;
    k_add_c128<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(cnt, R, X);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "fp64 refinement update");
}

__global__ void k_matvec_reduce(int64_t cnt, int nchunks, const double2* __restrict__ part,
                                double2* __restrict__ Y) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= cnt) return;
    double2 acc = make_double2(0, 0);
    for (int y = 0; y < nchunks; y++) acc = cadd(acc, part[int64_t(y) * cnt + i]);
    Y[i] = acc;
}

// Y (n x nrhs, ld n) = Z64 X (X: n x nrhs, ld n), with the residual kernel's
// row x column-chunk split; df: the products in double-float on the FP32 pipe
// (k_residual_part_df, about 1e-13 relative; an operand outside its exponent
// range sets the status word's df_range, and the caller repeats the product with
// df = false). Workspace: ctx->rwork32.
int matvec_z64(frico_gpu_ctx* ctx, const double2* X, int nrhs, double2* Y, bool df) {
    const int64_t n = ctx->n;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const unsigned rblocks = unsigned((n + 255) / 256);
    int nchunks = residual_chunks(int(n), sms, int(rblocks));
    const int chunk = int((n + nchunks - 1) / nchunks);
    nchunks = int((n + chunk - 1) / chunk);
    int rc;
    if ((rc = ensure(ctx, ctx->rwork32, sizeof(double2) * size_t(nchunks) * nrhs * n))) return rc;
    double2* part = (double2*)ctx->rwork32.p;
    const double2* Z64 = (const double2*)ctx->z64.p;
    DeviceStatus* dst = (DeviceStatus*)ctx->status.p;
    const dim3 grid(rblocks, nchunks);
    cudaStream_t st = ctx->stream;
    if (df && nrhs == 1)
        k_residual_part_df<1><<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part, dst);
    else if (df && nrhs == 2)
        k_residual_part_df<2><<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part, dst);
    else if (df && nrhs <= 4)
        k_residual_part_df<4><<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part, dst);
    else if (df)
        k_residual_part_df<kTR><<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part, dst);
    else
        k_residual_part<<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part);
    const int64_t cnt = n * nrhs;
    k_matvec_reduce<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(cnt, nchunks, part, Y);
    count_launch(ctx, 2);
    return cuda_check(ctx, cudaGetLastError(), "matvec");
}

int matvec_fp64(frico_gpu_ctx* ctx, const double2* X, int nrhs, double2* Y) {
    return matvec_z64(ctx, X, nrhs, Y, false);
}

// Out (n x nrhs, ld n) = M^{-1} In for the complex64 factors (z32, perm): rows
// gathered by the pivot order and cast, the two chained triangular solves,
// cast back. In has leading dimension ld_in. Workspace: ctx->dwork32.
int precond_apply_fp32(frico_gpu_ctx* ctx, const double2* In, int64_t ld_in, int nrhs, double2* Out) {
    const int64_t n = ctx->n, cnt = n * nrhs;
    int rc;
    if ((rc = ensure(ctx, ctx->dwork32, sizeof(float2) * cnt))) return rc;
    float2* W = (float2*)ctx->dwork32.p;
    k_gather_rows<double2, float2><<<unsigned((cnt + 255) / 256), 256, 0, ctx->stream>>>(
        int(n), nrhs, (const int32_t*)ctx->perm.p, In, ld_in, W, n);
    count_launch(ctx);
    if ((rc = trsv_solve_fp32(ctx, W, nrhs, n))) return rc;
    k_add_c64_to_c128<<<unsigned((cnt + 255) / 256), 256, 0, ctx->stream>>>(cnt, W, Out, 1);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "precond");
}

int gmres_refine(frico_gpu_ctx* ctx, double2* X, const double2* B, double2* R, const double* bnorm, double tol,
                 int max_iters, int* iters_out, double* rel_out);   // gmres.cu

// Mixed precision: X solves Z64 X = B with complex64 LU factors (z32) and FP64
// residuals r = B - Z64 X (classical iterative refinement). When the sweeps
// contract too slowly (ill-conditioned Z: kappa * eps32 near 1), the same
// factors precondition a GMRES on the FP64 system instead (gmres.cu).
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
    // residual split: 256 rows x `chunk` columns per CTA, ~4 CTAs per SM
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const unsigned rblocks = unsigned((n + 255) / 256);
    int nchunks = residual_chunks(int(n), sms, int(rblocks));
    const int chunk = int((n + nchunks - 1) / nchunks);
    nchunks = int((n + chunk - 1) / chunk);
    if ((rc = ensure(ctx, ctx->rwork32, sizeof(double2) * size_t(nchunks) * nrhs * n))) return rc;
    double2* part = (double2*)ctx->rwork32.p;
    k_colnorm2<double2><<<nrhs, 256, 0, st>>>(int(n), B, n, nrm + nrhs);
    count_launch(ctx);
    const double2* src = B;
    double prev = 1e300, rel = 1e300;
    DeviceStatus* dst = (DeviceStatus*)ctx->status.p;
    bool use_df = ctx->opt.residual_mode == FRICO_RESIDUAL_AUTO;
    if (use_df && (rc = cuda_check(ctx, cudaMemsetAsync(&dst->df_range, 0, sizeof(int), st), "df flag"))) return rc;
    // R = B - Z X and its column norms (double-float or FP64 products), then the norms to the host
    auto residual = [&](bool df) -> int {
        const double2* Z64 = (const double2*)ctx->z64.p;
        const dim3 grid = dim3(rblocks, nchunks);
        if (df && nrhs == 1)
            k_residual_part_df<1><<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part, dst);
        else if (df && nrhs == 2)
            k_residual_part_df<2><<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part, dst);
        else if (df && nrhs <= 4)
            k_residual_part_df<4><<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part, dst);
        else if (df)
            k_residual_part_df<kTR><<<grid, 256, 0, st>>>(Z64, n, int(n), X, n, nrhs, chunk, part, dst);
        else
            k_residual_part<<<dim3(rblocks, nchunks), 256, 0, st>>>((const double2*)ctx->z64.p, n, int(n), X, n,
                                                                   nrhs, chunk, part);
        k_residual_reduce<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(int(n), nrhs, nchunks, part, B, n, Rr);
        k_colnorm2<double2><<<nrhs, 256, 0, st>>>(int(n), Rr, n, nrm);
        count_launch(ctx, 3);
        int r2 = cuda_check(ctx, cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * 2 * nrhs, cudaMemcpyDeviceToHost, st),
                            "norms");
        if (!r2) r2 = cuda_check(ctx, cudaStreamSynchronize(st), "refine sync");
        return r2;
    };
    int it = 0;
    for (; it < max_it; it++) {
        k_gather_rows<double2, float2><<<unsigned((cnt + 255) / 256), 256, 0, st>>>(
            int(n), nrhs, (const int32_t*)ctx->perm.p, src, n, W, n);
        if ((rc = trsv_solve_fp32(ctx, W, nrhs, n))) return rc;
        k_add_c64_to_c128<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(cnt, W, X, it == 0);
        count_launch(ctx, 2);
        if ((rc = residual(use_df))) return rc;
        DeviceStatus hs;
        if ((rc = trsv_check(ctx, &hs))) return rc;
        if (use_df && hs.df_range) {   // an entry outside the double-float range: FP64 from here on
            use_df = false;
            if ((rc = residual(false))) return rc;
        }
        rel = 0.0;
        bool finite = true;
        for (int c = 0; c < nrhs; c++) {
            double bn = hn[nrhs + c] > 0 ? std::sqrt(hn[nrhs + c]) : 1.0;
            const double v = std::sqrt(hn[c]) / bn;
            finite = finite && std::isfinite(v);
            rel = std::max(rel, v);
        }
        if (!finite) rel = std::numeric_limits<double>::quiet_NaN();   // one bad column fails the solve
        src = Rr;
        if (!std::isfinite(rel)) { it++; break; }
        if (rel <= tol) { it++; break; }
        if (it >= 2 && rel > 0.5 * prev) { it++; break; }  // stagnation
        // slow contraction: more than 6 further sweeps at this rate -> Krylov
        if (it >= 1 && rel < prev && std::log(tol / rel) / std::log(rel / prev) > 6.0) { it++; break; }
        prev = rel;
    }
    if (std::isfinite(rel) && rel > tol && ctx->opt.refine_mode != FRICO_REFINE_CLASSIC) {
        // GMRES with its own budget: 2 x max_refine_iters iterations, at least one full
        // Krylov space of 120
        std::vector<double> bn(nrhs);
        for (int c = 0; c < nrhs; c++) bn[c] = hn[nrhs + c] > 0 ? std::sqrt(hn[nrhs + c]) : 1.0;
        int git = 0;
        double grel = rel;
        if ((rc = gmres_refine(ctx, X, B, Rr, bn.data(), tol, std::max(120, 2 * max_it), &git, &grel))) return rc;
        it += git;
        rel = grel;
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
