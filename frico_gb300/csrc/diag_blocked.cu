// Diagonal blocks of the no-pivot complex64 LU, blocked: the 128 x 128 block is
// factored in four 32-column panels instead of 128 barrier-separated rank-1
// steps, then inverted by 32 x 32 blocks.
//
// Per panel p (columns c0 = 32 p .. c0 + 31 of the working block W, 512 threads):
//   1. one warp factors the 32 x 32 diagonal block D (lane = column; pivots and
//      multipliers broadcast by shuffles, no barrier), keeping 1 / U_cc;
//   2. six warps solve the panels at once: L rows (x U_D = w, one thread per row
//      below D) and U columns (L_D x = w, one thread per column right of D);
//   3. all sixteen warps update the trailing block with the rank-32 product,
//      register-tiled (6 x 3, 4 x 2, 2 x 1 outputs per thread).
// Four barriers per panel instead of 32 steps of one barrier each. Both CTAs
// factor the block (the same arithmetic, so the same LU), then each builds one
// inverse by 32 x 32 blocks:
//   CTA 0: X = U^{-1} in the form X U = I (what L21 = A21 U^{-1} needs):
//     X_jj U_jj = I row by row, then in rounds s = 1..3, all row blocks i at once,
//     X[i][i+s] = -(sum_{k=i}^{i+s-1} X[i][k] U[k][i+s]) X_{i+s,i+s};
//   CTA 1: Y = L^{-1} in the form L Y = I (what U12 = L^{-1} A12 needs):
//     L_jj Y_jj = I column by column, then Y[i+s][i] = -Y_{i+s,i+s} sum_{k=i}^{i+s-1} L[i+s][k] Y[k][i].
// Outputs as the single-sweep kernel of lu_nopiv.cu writes them: the LU (CTA 0),
// U^{-1} and its B^ operand hi / lo (CTA 0), L^{-1} and its A* operand hi / lo
// (CTA 1), a zero or non-finite pivot in st->info (first one, CTA 0).
#include <cuda_runtime.h>

#include <cstdio>

#include "common.cuh"

namespace frico {

namespace dblk {

constexpr int kN = 128;          // block size
constexpr int kLD = 129;         // shared leading dimension (odd: strided columns hit distinct banks)
constexpr int kThreads = 512;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float2 shfl2(float2 v, int src) {
    return make_float2(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src));
}
__device__ __forceinline__ bool finite2(float2 a) { return isfinite(a.x) && isfinite(a.y); }
__device__ __forceinline__ float2 crcp(float2 p, bool& bad) {
    bad = (p.x == 0.f && p.y == 0.f) || !finite2(p);
    const float d = p.x * p.x + p.y * p.y;
    return bad ? make_float2(0.f, 0.f) : make_float2(p.x / d, -p.y / d);
}
__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }
__device__ __forceinline__ void put_split(float* hp, float* lp, int64_t pair, float2 a) {
    const float2 h = make_float2(tf32_hi(a.x), tf32_hi(a.y));
    reinterpret_cast<float2*>(hp)[pair] = h;
    reinterpret_cast<float2*>(lp)[pair] = make_float2(a.x - h.x, a.y - h.y);
}

// 1. LU of the 32 x 32 block at (c0, c0), one warp, lane = column c0 + lane.
// rdiag[c] = 1 / U_cc (0 for a zero or non-finite pivot, reported once in info).
__device__ __noinline__ void lu32(float2* W, int c0, int lane, float2* rdiag, bool report, DeviceStatus* st,
                                     int kbase) {
    float2 v[32];
#pragma unroll
    for (int r = 0; r < 32; r++) v[r] = W[(c0 + lane) * kLD + c0 + r];
#pragma unroll
    for (int c = 0; c < 32; c++) {
        bool bad;
        const float2 inv = crcp(shfl2(v[c], c), bad);
        if (lane == 0) {
            rdiag[c] = inv;
            if (report && bad) atomicCAS(&st->info, 0, kbase + c + 1);
        }
#pragma unroll
        for (int r = c + 1; r < 32; r++) {
            if (lane == c) v[r] = cmul(v[r], inv);   // multiplier: L's column c
            const float2 m = shfl2(v[r], c);
            if (lane > c) v[r] = cfms(v[r], m, v[c]);
        }
    }
#pragma unroll
    for (int r = 0; r < 32; r++) W[(c0 + lane) * kLD + c0 + r] = v[r];
}

// 2a. Row i below the diagonal block: x U_D = w (forward over the panel's columns).
__device__ __noinline__ void lrow(float2* W, int c0, int i, const float2* rdiag) {
    float2 w[32];
#pragma unroll
    for (int k = 0; k < 32; k++) w[k] = W[(c0 + k) * kLD + i];
#pragma unroll
    for (int k = 0; k < 32; k++) {
        w[k] = cmul(w[k], rdiag[k]);
#pragma unroll
        for (int j = k + 1; j < 32; j++) w[j] = cfms(w[j], w[k], W[(c0 + j) * kLD + c0 + k]);
    }
#pragma unroll
    for (int k = 0; k < 32; k++) W[(c0 + k) * kLD + i] = w[k];
}

// 2b. Column j right of the diagonal block: L_D x = w (L_D unit lower).
__device__ __noinline__ void ucol(float2* W, int c0, int j) {
    float2 w[32];
#pragma unroll
    for (int r = 0; r < 32; r++) w[r] = W[j * kLD + c0 + r];
#pragma unroll
    for (int k = 0; k < 32; k++)
#pragma unroll
        for (int r = k + 1; r < 32; r++) w[r] = cfms(w[r], W[(c0 + k) * kLD + c0 + r], w[k]);
#pragma unroll
    for (int r = 0; r < 32; r++) W[j * kLD + c0 + r] = w[r];
}

// 3. W[i][j] -= sum_k L[i][k] U[k][j] over the trailing block (m = 96 - 32 P rows and
// columns from c0 + 32), thread (tx, ty) of a 32 x 16 grid: rows ty + 16 a, columns tx + 32 b.
template <int P>
__device__ __forceinline__ void trailing(float2* W, int tx, int ty) {
    constexpr int c0 = 32 * P, m = 96 - 32 * P, RA = m / 16, CB = m / 32, base = c0 + 32;
    float2 acc[RA][CB];
#pragma unroll
    for (int a = 0; a < RA; a++)
#pragma unroll
        for (int b = 0; b < CB; b++) acc[a][b] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k < 32; k++) {
        float2 l[RA], u[CB];
#pragma unroll
        for (int a = 0; a < RA; a++) l[a] = W[(c0 + k) * kLD + base + ty + 16 * a];
#pragma unroll
        for (int b = 0; b < CB; b++) u[b] = W[(base + tx + 32 * b) * kLD + c0 + k];
#pragma unroll
        for (int a = 0; a < RA; a++)
#pragma unroll
            for (int b = 0; b < CB; b++) {
                acc[a][b].x += l[a].x * u[b].x - l[a].y * u[b].y;
                acc[a][b].y += l[a].x * u[b].y + l[a].y * u[b].x;
            }
    }
#pragma unroll
    for (int a = 0; a < RA; a++)
#pragma unroll
        for (int b = 0; b < CB; b++) {
            float2& w = W[(base + tx + 32 * b) * kLD + base + ty + 16 * a];
            w = csub(w, acc[a][b]);
        }
}

// Inverse of one 32 x 32 diagonal block, one thread per row (upper, X U = I) or per
// column (unit lower, L Y = I); results into the inverse's block (ldx).
__device__ __noinline__ void xdiag_row(const float2* W, int c0, int r, const float2* rdiag, float2* X) {
    float2 w[32];
#pragma unroll
    for (int c = 0; c < 32; c++) w[c] = make_float2(c == r ? 1.f : 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 32; k++) {
        w[k] = cmul(w[k], rdiag[k]);
#pragma unroll
        for (int c = k + 1; c < 32; c++) w[c] = cfms(w[c], w[k], W[(c0 + c) * kLD + c0 + k]);
    }
#pragma unroll
    for (int c = 0; c < 32; c++) X[c * 33 + r] = w[c];   // the packed diagonal block (leading dimension 33)
}

__device__ __noinline__ void ydiag_col(const float2* W, int c0, int j, float2* Y) {
    float2 w[32];
#pragma unroll
    for (int r = 0; r < 32; r++) w[r] = make_float2(r == j ? 1.f : 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 32; k++)
#pragma unroll
        for (int r = k + 1; r < 32; r++) w[r] = cfms(w[r], W[(c0 + k) * kLD + c0 + r], w[k]);
#pragma unroll
    for (int r = 0; r < 32; r++) Y[j * 33 + r] = w[r];   // the packed diagonal block (leading dimension 33)
}

// The inverse is kept block-packed in shared memory: only the ten 32 x 32 blocks of its
// triangle, each column-major with leading dimension 33. Block (a, b), a <= b the smaller
// of the two block indices, is block number 4 a - a (a - 1) / 2 + b - a.
constexpr int kBLD = 33, kBlk = 32 * kBLD;
__device__ __forceinline__ int bidx(int a, int b) { return 4 * a - (a * (a - 1)) / 2 + (b - a); }
// element (row R, column C) of X (upper) or Y (lower)
__device__ __forceinline__ float2& xs_at(float2* Xs, bool upper, int R, int C) {
    const int blk = upper ? bidx(R >> 5, C >> 5) : bidx(C >> 5, R >> 5);
    return Xs[blk * kBlk + (C & 31) * kBLD + (R & 31)];
}

}  // namespace dblk

// The blocked diagonal-block kernel (see the top of this file). src: the block
// (leading dimension lds), read in place; dlu: the LU (ldd); Uinv, Linv: 128 x 128
// column-major; the split operands in sp (TF32 hi / lo).
__global__ void __launch_bounds__(dblk::kThreads) k_diag_lu_blk(const float2* __restrict__ src, int64_t lds,
                                                                float2* dlu, int64_t ldd, int k0, int jb,
                                                                float2* Uinv, float2* Linv, DeviceStatus* st,
                                                                TcDiagSplit sp) {
    using namespace dblk;
    extern __shared__ __align__(16) unsigned char smraw[];
    float2* W = (float2*)smraw;                 // [c * kLD + r], the working block, then its LU
    float2* Xs = W + kN * kLD;                  // the inverse being built, block-packed (xs_at)
    float2* rd = Xs + 10 * kBlk;                // [4][32] 1 / U_cc of each diagonal block
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const bool upper = blockIdx.x == 0;
    for (int idx = t; idx < kN * kN; idx += kThreads) {
        const int r = idx & (kN - 1), c = idx >> 7;
        W[c * kLD + r] = (r < jb && c < jb) ? src[int64_t(c) * lds + r] : make_float2(r == c ? 1.f : 0.f, 0.f);
    }
    __syncthreads();
    const int tx = t & 31, ty = t >> 5;
#pragma unroll 1
    for (int p = 0; p < 4; p++) {
        const int c0 = 32 * p;
        if (warp == 0) lu32(W, c0, lane, rd + 32 * p, upper, st, k0 + c0);
        __syncthreads();
        if (p == 3) break;
        const int nr = 96 - c0;                  // rows below / columns right of D
        if (t >= 32 && t < 32 + nr) lrow(W, c0, c0 + 32 + (t - 32), rd + 32 * p);
        else if (t >= 128 && t < 128 + nr) ucol(W, c0, c0 + 32 + (t - 128));
        __syncthreads();
        if (p == 0) trailing<0>(W, tx, ty);
        else if (p == 1) trailing<1>(W, tx, ty);
        else trailing<2>(W, tx, ty);
        __syncthreads();
    }
    // ---- inverses by 32 x 32 blocks, into Xs (column-major, kLD)
    for (int idx = t; idx < 10 * kBlk; idx += kThreads) Xs[idx] = make_float2(0.f, 0.f);
    __syncthreads();
    if (t < 128) {
        const int b = t >> 5, q = t & 31;
        if (upper) xdiag_row(W, 32 * b, q, rd + 32 * b, Xs + bidx(b, b) * kBlk);
        else ydiag_col(W, 32 * b, q, Xs + bidx(b, b) * kBlk);
    }
    __syncthreads();
    // rounds s = 1..3: every block pair (i, i + s) at once. Thread (r = t & 31, cp = t >> 5):
    // row r, columns 2 cp and 2 cp + 1 of each output block (g = block pair of the round).
#pragma unroll 1
    for (int s = 1; s < 4; s++) {
        const int nblk = 4 - s;
        // T = sum over the s blocks between; each thread keeps its outputs for up to 3 blocks
        float2 T[3][2];
        const int r = t & 31, cp = t >> 5;
#pragma unroll
        for (int g = 0; g < 3; g++) {
            T[g][0] = T[g][1] = make_float2(0.f, 0.f);
            if (g >= nblk) continue;
            const int i = g, j = g + s;   // block pair
            for (int kb = i; kb < j; kb++) {
#pragma unroll 8
                for (int kk = 0; kk < 32; kk++) {
                    const int k = 32 * kb + kk;
                    if (upper) {
                        // X[i][kb] U[kb][j]: row 32 i + r of X, column 32 j + c of U
                        const float2 a = xs_at(Xs, true, 32 * i + r, k);
                        const float2 b0 = W[(32 * j + 2 * cp) * kLD + k], b1 = W[(32 * j + 2 * cp + 1) * kLD + k];
                        T[g][0] = cadd(T[g][0], cmul(a, b0));
                        T[g][1] = cadd(T[g][1], cmul(a, b1));
                    } else {
                        // L[j][kb] Y[kb][i]: row 32 j + r of L, column 32 i + c of Y
                        const float2 a = W[k * kLD + 32 * j + r];
                        const float2 b0 = xs_at(Xs, false, k, 32 * i + 2 * cp), b1 = xs_at(Xs, false, k, 32 * i + 2 * cp + 1);
                        T[g][0] = cadd(T[g][0], cmul(a, b0));
                        T[g][1] = cadd(T[g][1], cmul(a, b1));
                    }
                }
            }
        }
        __syncthreads();
        // stage T in the inverse's own (still zero) target blocks, then multiply by the diagonal inverse
#pragma unroll
        for (int g = 0; g < 3; g++) {
            if (g >= nblk) continue;
            const int i = g, j = g + s;
            if (upper) {
                xs_at(Xs, true, 32 * i + r, 32 * j + 2 * cp) = T[g][0];
                xs_at(Xs, true, 32 * i + r, 32 * j + 2 * cp + 1) = T[g][1];
            } else {
                xs_at(Xs, false, 32 * j + r, 32 * i + 2 * cp) = T[g][0];
                xs_at(Xs, false, 32 * j + r, 32 * i + 2 * cp + 1) = T[g][1];
            }
        }
        __syncthreads();
        float2 O[3][2];
#pragma unroll
        for (int g = 0; g < 3; g++) {
            O[g][0] = O[g][1] = make_float2(0.f, 0.f);
            if (g >= nblk) continue;
            const int i = g, j = g + s;
#pragma unroll 8
            for (int kk = 0; kk < 32; kk++) {
                if (upper) {
                    // X[i][j] = -T X_jj: T row r (staged at X[i][j]), X_jj column c
                    const float2 a = xs_at(Xs, true, 32 * i + r, 32 * j + kk);
                    const float2 b0 = xs_at(Xs, true, 32 * j + kk, 32 * j + 2 * cp);
                    const float2 b1 = xs_at(Xs, true, 32 * j + kk, 32 * j + 2 * cp + 1);
                    O[g][0] = csub(O[g][0], cmul(a, b0));
                    O[g][1] = csub(O[g][1], cmul(a, b1));
                } else {
                    // Y[j][i] = -Y_jj T: Y_jj row r, T column c (staged at Y[j][i])
                    const float2 a = xs_at(Xs, false, 32 * j + r, 32 * j + kk);
                    const float2 b0 = xs_at(Xs, false, 32 * j + kk, 32 * i + 2 * cp);
                    const float2 b1 = xs_at(Xs, false, 32 * j + kk, 32 * i + 2 * cp + 1);
                    O[g][0] = csub(O[g][0], cmul(a, b0));
                    O[g][1] = csub(O[g][1], cmul(a, b1));
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int g = 0; g < 3; g++) {
            if (g >= nblk) continue;
            const int i = g, j = g + s;
            if (upper) {
                xs_at(Xs, true, 32 * i + r, 32 * j + 2 * cp) = O[g][0];
                xs_at(Xs, true, 32 * i + r, 32 * j + 2 * cp + 1) = O[g][1];
            } else {
                xs_at(Xs, false, 32 * j + r, 32 * i + 2 * cp) = O[g][0];
                xs_at(Xs, false, 32 * j + r, 32 * i + 2 * cp + 1) = O[g][1];
            }
        }
        __syncthreads();
    }
    // ---- outputs (identity past jb in the inverses, as the single-sweep kernel writes them)
    if (upper) {
        for (int idx = t; idx < kN * kN; idx += kThreads) {
            const int r = idx & (kN - 1), c = idx >> 7;
            if (r < jb && c < jb) dlu[int64_t(c) * ldd + r] = W[c * kLD + r];
            const float2 v = r <= c ? xs_at(Xs, true, r, c) : make_float2(0.f, 0.f);
            Uinv[c * kN + r] = v;
            if (sp.uh) put_split((float*)sp.uh, (float*)sp.ul, int64_t(c) * kN + r, v);
        }
    } else {
        for (int idx = t; idx < kN * kN; idx += kThreads) {
            const int r = idx & (kN - 1), c = idx >> 7;
            Linv[c * kN + r] = r >= c ? xs_at(Xs, false, r, c) : make_float2(0.f, 0.f);
        }
        if (sp.lh)
            for (int idx = t; idx < kN * kN; idx += kThreads) {   // A* rows 2r, 2r + 1 at K = 2c, 2c + 1
                const int c = idx & (kN - 1), r = idx >> 7;
                const float2 v = r >= c ? xs_at(Xs, false, r, c) : make_float2(0.f, 0.f);
                const int64_t o0 = int64_t(2 * r) * kN + c, o1 = o0 + kN;   // pair units, rows of 256 values
                put_split((float*)sp.lh, (float*)sp.ll, o0, make_float2(v.x, -v.y));
                put_split((float*)sp.lh, (float*)sp.ll, o1, make_float2(v.y, v.x));
            }
    }
}

size_t diag_lu_blk_smem() { return sizeof(float2) * (size_t(dblk::kN) * dblk::kLD + 10 * dblk::kBlk + 4 * 32); }

int launch_diag_lu_blk(frico_gpu_ctx* ctx, cudaStream_t st, const float2* src, int64_t lds, float2* dlu, int64_t ldd,
                       int k0, int jb, float2* Uinv, float2* Linv, DeviceStatus* dst, const TcDiagSplit& sp) {
    k_diag_lu_blk<<<2, dblk::kThreads, diag_lu_blk_smem(), st>>>(src, lds, dlu, ldd, k0, jb, Uinv, Linv, dst, sp);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_diag_lu_blk");
}

int diag_lu_blk_setup(frico_gpu_ctx* ctx) {
    return cuda_check(ctx, cudaFuncSetAttribute(k_diag_lu_blk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                int(diag_lu_blk_smem())),
                      "k_diag_lu_blk smem");
}

}  // namespace frico
