// Blocked complex LU without row interchanges, for the mixed-precision path.
//
// The complex64 factors of the mixed path only precondition an iterative
// refinement whose residual is computed against the FP64 Z, so the pivoting
// strategy affects the number of refinement sweeps, not the accuracy of the
// result. EFIE impedance matrices (RWG, Dunavant quadrature) factor stably
// without interchanges (growth 2.3 on the 7680-unknown sphere), and dropping
// the pivot search removes the n sequential cluster-wide argmax steps of the
// partial-pivoting panel. The caller falls back to partial pivoting when a
// pivot is zero / not finite (info != 0) or the refinement does not converge.
//
// Per block column k0 (width nb = 128):
//   k_diag_lu      two CTAs, one elimination sweep each: LU and L11^{-1} of the
//                  nb x nb diagonal block, and U11^{-1} as the rows of U appear
//   k_trsm_right   L21 = A21 U11^{-1}, 64 rows per CTA
//   k_trsm_lower_unit (lu.cu)   U12 = L11^{-1} A12
//   trailing update A22 -= L21 U12 (tensor cores when available)
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "common.cuh"

namespace frico {

static const int kNP = 128;   // block width of the no-pivot LU

template <typename C> __device__ __forceinline__ bool cfinite(C a) { return isfinite(a.x) && isfinite(a.y); }

// Diagonal block kernel: 256 threads as a 16 x 16 grid; thread (tx, ty) keeps
// rows ty + 16 i and columns tx + 16 j (i, j < 8) of a 128 x 128 working
// matrix W in registers. Every elimination step is a rank-1 update of the
// registers from one column and one row published in shared memory
// (double-buffered, so one barrier per step). Step c lies in phase P = c / 16;
// each phase is unrolled for its own P and updates only the live tiles.
//
// Both CTAs run the same 128 elimination steps (no interchanges) with the same
// arithmetic on the not yet eliminated part (rows and columns > c), so they
// see the same pivots and the same U; each keeps a different inverse in the
// part of W that elimination has freed:
//  CTA 1 (LOWER): row elimination of [W | I], the columns <= c of the identity
//    half in place of the eliminated columns of W. With m_r = W[r][c] / W[c][c]:
//      W[r][j] -= m_r W[c][j] (r > c, j != c),   W[r][c] = -m_r,
//    ending with U on and above the diagonal and L^{-1} (unit diagonal
//    implied) below it; the multipliers m are L.
//  CTA 0: U^{-1} = X by a right-looking inversion as the rows of U appear. The
//    rows r <= c hold T (columns > c) and X (columns <= c); T starts as the
//    identity row when row c of U is final, then
//      X[r][c] = T[r][c] / U[c][c] (r <= c),  T[r][j] -= X[r][c] U[c][j] (j > c),
//    the same rank-1 form as the elimination of the rows below.
static const int kDLD = kNP + 1;   // shared leading dimension (conflict-free tile reads)
static const int kDiagThreads = 256;

// Steps c = 16 P .. 16 P + 15. LOWER: the multipliers (L) go to S[c * kDLD + r], r > c.
template <int P, bool LOWER, typename C>
__device__ __forceinline__ void diag_sweep_phase(C (&v)[8][8], C* S, C* vb, int tx, int ty, int k0,
                                                 DeviceStatus* st) {
    using R = decltype(v[0][0].x);
#pragma unroll 1
    for (int cl = 0; cl < 16; cl++) {
        const int c = 16 * P + cl;
        C* lb = vb + (c & 1) * 2 * kNP;   // column c (all rows)
        C* ub = lb + kNP;                 // row c (all columns)
        if (tx == cl) {
#pragma unroll
            for (int i = 0; i < 8; i++) lb[ty + 16 * i] = v[i][P];
        }
        if (ty == cl) {
#pragma unroll
            for (int j = 0; j < 8; j++) ub[tx + 16 * j] = v[P][j];
        }
        __syncthreads();
        const C p = ub[c];
        const bool bad = (p.x == R(0) && p.y == R(0)) || !cfinite(p);
        const R rd = R(1) / (p.x * p.x + p.y * p.y);
        const C inv = bad ? cmake(R(0), R(0)) : cmake(p.x * rd, -p.y * rd);
        if (LOWER && bad && threadIdx.x == 0) atomicCAS(&st->info, 0, k0 + c + 1);
        if (LOWER) {
            C m[8], u[8];
#pragma unroll
            for (int i = P; i < 8; i++) m[i] = (i > P || ty > cl) ? cmul(lb[ty + 16 * i], inv) : cmake(R(0), R(0));
#pragma unroll
            for (int j = 0; j < 8; j++) u[j] = ub[tx + 16 * j];
#pragma unroll
            for (int i = P; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) v[i][j] = cfms(v[i][j], m[i], u[j]);
            if (tx == cl) {
#pragma unroll
                for (int i = P; i < 8; i++)
                    if (i > P || ty > cl) {
                        v[i][P] = cmake(-m[i].x, -m[i].y);
                        S[c * kDLD + ty + 16 * i] = m[i];
                    }
            }
        } else {
            // f = multiplier (rows > c), X[r][c] (rows < c), 1 / U[c][c] (row c)
            C f[8], u[8];
#pragma unroll
            for (int i = 0; i < 8; i++) f[i] = (i == P && ty == cl) ? inv : cmul(lb[ty + 16 * i], inv);
#pragma unroll
            for (int j = P; j < 8; j++) u[j] = (j > P || tx > cl) ? ub[tx + 16 * j] : cmake(R(0), R(0));
            if (ty == cl) {   // row c of U becomes the identity row of T
#pragma unroll
                for (int j = P; j < 8; j++)
                    if (j > P || tx > cl) v[P][j] = cmake(R(0), R(0));
            }
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = P; j < 8; j++) v[i][j] = cfms(v[i][j], f[i], u[j]);
            if (tx == cl) {   // column c of X
#pragma unroll
                for (int i = 0; i <= P; i++)
                    if (i < P || ty <= cl) v[i][P] = f[i];
            }
        }
    }
}

template <bool LOWER, typename C>
__device__ __forceinline__ void diag_sweep(C (&v)[8][8], C* S, C* vb, int tx, int ty, int k0, DeviceStatus* st) {
    diag_sweep_phase<0, LOWER>(v, S, vb, tx, ty, k0, st);
    diag_sweep_phase<1, LOWER>(v, S, vb, tx, ty, k0, st);
    diag_sweep_phase<2, LOWER>(v, S, vb, tx, ty, k0, st);
    diag_sweep_phase<3, LOWER>(v, S, vb, tx, ty, k0, st);
    diag_sweep_phase<4, LOWER>(v, S, vb, tx, ty, k0, st);
    diag_sweep_phase<5, LOWER>(v, S, vb, tx, ty, k0, st);
    diag_sweep_phase<6, LOWER>(v, S, vb, tx, ty, k0, st);
    diag_sweep_phase<7, LOWER>(v, S, vb, tx, ty, k0, st);
}

template <typename C> constexpr size_t diag_lu_smem() { return sizeof(C) * (size_t(kNP) * kDLD + 4 * kNP); }

// LU (no interchanges) of the jb x jb diagonal block at (k0, k0) of the
// matrix, read from src (leading dimension lds) and written to dlu (ldd);
// U11^{-1} to Uinv and L11^{-1} (unit lower) to Linv, both 128 x 128
// column-major (the GEMMs read their jb x jb part with leading dimension 128,
// the chained solves the whole block). A block narrower than 128 is padded
// with the identity. A zero or non-finite pivot sets st->info (first one).
// CTA 1 writes the LU and L^{-1}, CTA 0 U^{-1}; both read src, so dlu must not
// alias it: either src is a copy of the block (the SIMT path, dlu = the block
// in A) or src is the block in A and dlu a staging slot that k_uinv_blocks
// copies into A after the factorisation (the tensor-core path, whose later
// steps never read the diagonal blocks of A).
// With usplit / lsplit (complex64 only): U^{-1} also as the hi/lo B^ operand
// of L21 = A21 U^{-1} (row j = column j of U^{-1}, 256 values: the hi/lo of the
// column-major array itself), L^{-1} as the A* operand of U12 = L^{-1} A12
// (rows 2r = (re, -im), 2r + 1 = (im, re) of row r, 256 values each); TF32 in
// float pairs or (sp.h) FP16 in half pairs, each inverse scaled by the power of
// two u (l) that puts its largest entry in [2^8, 2^9), with 1 / (s u) and
// 1 / (l s) (s = *sp.sc) to sp.res_l21 and sp.res_u12 for the GEMMs' results.
__device__ __forceinline__ float2 tf32_hi2(float2 v) {
    return make_float2(__uint_as_float(__float_as_uint(v.x) & 0xFFFFE000u),
                       __uint_as_float(__float_as_uint(v.y) & 0xFFFFE000u));
}

// Largest |re|, |im| over the CTA (every thread of the CTA calls it; red: 32 floats).
__device__ __forceinline__ float cta_absmax(float m, float* red) {
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = 0.f;
    for (int w = 0; w < int(blockDim.x >> 5); w++) m = fmaxf(m, red[w]);
    __syncthreads();
    return m;
}

// The power of two that puts m in [2^8, 2^9) (1 for zero or non-finite m).
__device__ __forceinline__ float pow2_for(float m) {
    int ex = 0;
    if (m > 0.f && isfinite(m)) {
        const int eb = int((__float_as_uint(m) >> 23) & 0xFF);   // 2^(eb-127) <= m < 2^(eb-126)
        ex = min(60, max(-60, 135 - max(eb, 1)));
    }
    return __uint_as_float(uint32_t(127 + ex) << 23);
}

// Pair a (already scaled for FP16) as hi/lo operands at pair index o.
__device__ __forceinline__ void put_split2(void* hp, void* lp, int64_t o, float2 a, bool h) {
    if (h) {
        const __half2 hi = __floats2half2_rn(a.x, a.y);
        const float2 hf = __half22float2(hi);
        ((__half2*)hp)[o] = hi;
        ((__half2*)lp)[o] = __floats2half2_rn(a.x - hf.x, a.y - hf.y);
    } else {
        const float2 hi = tf32_hi2(a);
        ((float2*)hp)[o] = hi;
        ((float2*)lp)[o] = make_float2(a.x - hi.x, a.y - hi.y);
    }
}

template <typename C, bool F16>
__global__ void __launch_bounds__(kDiagThreads) k_diag_lu(const C* __restrict__ src, int64_t lds, C* dlu,
                                                         int64_t ldd, int k0, int jb, C* Uinv, C* Linv,
                                                         DeviceStatus* st, TcDiagSplit sp) {
    using R = decltype(src[0].x);
    extern __shared__ __align__(16) unsigned char smraw[];
    C* S = (C*)smraw;              // S[c * kDLD + r]
    C* vb = S + kNP * kDLD;        // 4 x kNP published rows / columns
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const bool lower = blockIdx.x == 1;
#pragma unroll 16
    for (int it = 0; it < kNP * kNP / kDiagThreads; it++) {
        const int idx = threadIdx.x + kDiagThreads * it, r = idx & (kNP - 1), c = idx >> 7;
        S[c * kDLD + r] = (r < jb && c < jb) ? src[c * lds + r] : cmake(R(r == c ? 1 : 0), R(0));
    }
    __syncthreads();
    C v[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) v[i][j] = S[(tx + 16 * j) * kDLD + ty + 16 * i];
    if (lower) {
        diag_sweep<true>(v, S, vb, tx, ty, k0, st);
        // U (upper triangle and diagonal of W) next to L (multipliers, strict lower of S)
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++)
                if (ty + 16 * i <= tx + 16 * j) S[(tx + 16 * j) * kDLD + ty + 16 * i] = v[i][j];
        __syncthreads();
#pragma unroll 16
        for (int it = 0; it < kNP * kNP / kDiagThreads; it++) {
            const int idx = threadIdx.x + kDiagThreads * it, r = idx & (kNP - 1), c = idx >> 7;
            if (r < jb && c < jb) dlu[c * ldd + r] = S[c * kDLD + r];
        }
        __syncthreads();   // S takes L^{-1} (strict lower of W)
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++)
                if (ty + 16 * i > tx + 16 * j) S[(tx + 16 * j) * kDLD + ty + 16 * i] = v[i][j];
        __syncthreads();
#pragma unroll 8
        for (int it = 0; it < kNP * kNP / kDiagThreads; it++) {   // full 128 x 128, identity past jb
            const int idx = threadIdx.x + kDiagThreads * it, r = idx & (kNP - 1), c = idx >> 7;
            Linv[c * kNP + r] = r > c ? S[c * kDLD + r] : cmake(R(r == c ? 1 : 0), R(0));
        }
        if (sp.lh) {
            float ls = 1.f;
            if constexpr (F16) {   // l from the largest entry of L^{-1} (unit diagonal included)
                __shared__ float red[32];
                float m = 1.f;
#pragma unroll
                for (int i = 0; i < 8; i++)
#pragma unroll
                    for (int j = 0; j < 8; j++)
                        if (ty + 16 * i > tx + 16 * j)
                            m = fmaxf(m, fmaxf(fabsf(float(v[i][j].x)), fabsf(float(v[i][j].y))));
                ls = pow2_for(cta_absmax(m, red));
                if (threadIdx.x == 0) *sp.res_u12 = 1.f / (ls * *sp.sc);   // powers of two: exact
            }
#pragma unroll 4
            for (int it = 0; it < kNP * kNP / kDiagThreads; it++) {   // A* rows 2r, 2r + 1 at K = 2c, 2c + 1
                const int idx = threadIdx.x + kDiagThreads * it, c = idx & (kNP - 1), r = idx >> 7;
                const C v = r > c ? S[c * kDLD + r] : cmake(R(r == c ? 1 : 0), R(0));
                float2 a0 = make_float2(float(v.x), -float(v.y)), a1 = make_float2(float(v.y), float(v.x));
                if constexpr (F16) {
                    a0 = make_float2(a0.x * ls, a0.y * ls);
                    a1 = make_float2(a1.x * ls, a1.y * ls);
                }
                const int64_t o0 = int64_t(2 * r) * kNP + c, o1 = o0 + kNP;   // pair units, rows of 256 values
                put_split2(sp.lh, sp.ll, o0, a0, F16);
                put_split2(sp.lh, sp.ll, o1, a1, F16);
            }
        }
    } else {
        diag_sweep<false>(v, S, vb, tx, ty, k0, st);
        __syncthreads();   // S no longer read: it takes U^{-1} (upper triangle and diagonal of W)
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++)
                if (ty + 16 * i <= tx + 16 * j) S[(tx + 16 * j) * kDLD + ty + 16 * i] = v[i][j];
        __syncthreads();
        float us = 1.f;
        if constexpr (F16) {   // u from the largest entry of U^{-1}
            __shared__ float red[32];
            float m = 0.f;
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (ty + 16 * i <= tx + 16 * j)
                        m = fmaxf(m, fmaxf(fabsf(float(v[i][j].x)), fabsf(float(v[i][j].y))));
            us = pow2_for(cta_absmax(m, red));
            if (threadIdx.x == 0) *sp.res_l21 = 1.f / (*sp.sc * us);   // powers of two: exact
        }
#pragma unroll 8
        for (int it = 0; it < kNP * kNP / kDiagThreads; it++) {
            const int idx = threadIdx.x + kDiagThreads * it, r = idx & (kNP - 1), c = idx >> 7;
            const C v = r <= c ? S[c * kDLD + r] : cmake(R(0), R(0));
            Uinv[c * kNP + r] = v;
            if (sp.uh) {
                float2 a = make_float2(float(v.x), float(v.y));
                if constexpr (F16) a = make_float2(a.x * us, a.y * us);
                put_split2(sp.uh, sp.ul, c * kNP + r, a, F16);
            }
        }
    }
}

// U^{-1} of every diagonal block by back substitution, for the chained
// triangular solves: the inverse from the elimination sweep satisfies
// X U = I to working accuracy (what L21 = A21 U11^{-1} needs), the one below
// U X = I (what the block solve x = U11^{-1} b needs); on ill-conditioned
// blocks the two differ by far more than rounding. One CTA per block, after
// the factorisation.
// Backward column sweeps, steps i = 16 P + 15 .. 16 P:
//   X[i,:] /= U[i][i];  X[k,:] -= U[k][i] X[i,:]  (k < i).
// X[i][j] = 0 for j < i, so only tile columns >= P and rows <= P are live.
template <int P, typename C>
__device__ __forceinline__ void uinv_phase(C (&x)[8][8], const C* S, C* vb, const C* rdiag, int tx, int ty,
                                           int& step) {
    using R = decltype(x[0][0].x);
#pragma unroll 1
    for (int il = 15; il >= 0; il--) {
        const int i = 16 * P + il;
        C* b = vb + (step++ & 1) * kNP;
        if (ty == il) {
#pragma unroll
            for (int j = P; j < 8; j++) b[tx + 16 * j] = x[P][j];
        }
        __syncthreads();
        const C inv = rdiag[i];
        C xr[8], cf[8];
#pragma unroll
        for (int j = P; j < 8; j++) xr[j] = cmul(b[tx + 16 * j], inv);
#pragma unroll
        for (int k = 0; k <= P; k++) cf[k] = (k < P || ty < il) ? S[i * kDLD + ty + 16 * k] : cmake(R(0), R(0));
#pragma unroll
        for (int k = 0; k <= P; k++)
#pragma unroll
            for (int j = P; j < 8; j++) x[k][j] = cfms(x[k][j], cf[k], xr[j]);
        if (ty == il) {
#pragma unroll
            for (int j = P; j < 8; j++) x[P][j] = xr[j];
        }
    }
}

template <typename C> constexpr size_t uinv_smem() { return sizeof(C) * (size_t(kNP) * kDLD + 3 * kNP); }

// Block b = blockIdx.x: U of the diagonal block at (128 b, 128 b) (identity past
// n), its inverse to Uinv + b 128^2 (128 x 128 column-major). The block's LU is
// read from A (stage == nullptr) or from the staging slot stage + b 128^2
// (ld 128), which is then also copied into A.
template <typename C>
__global__ void __launch_bounds__(256) k_uinv_blocks(C* A, int64_t lda, int n, const C* __restrict__ stage,
                                                     C* Uinv) {
    using R = decltype(A[0].x);
    extern __shared__ __align__(16) unsigned char smraw[];
    C* S = (C*)smraw;              // S[c * kDLD + r]
    C* vb = S + kNP * kDLD;        // 2 x kNP published rows
    C* rdiag = vb + 2 * kNP;
    const int k0 = blockIdx.x * kNP, jb = min(kNP, n - k0);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const C* blk = stage ? stage + size_t(blockIdx.x) * kNP * kNP : A + int64_t(k0) * lda + k0;
    const int64_t ldb = stage ? kNP : lda;
    for (int idx = threadIdx.x; idx < kNP * kNP; idx += 256) {
        const int r = idx & (kNP - 1), c = idx >> 7;
        C a = cmake(R(r == c ? 1 : 0), R(0));
        if (r < jb && c < jb) {
            const C lu = blk[c * ldb + r];
            if (stage) A[int64_t(k0 + c) * lda + k0 + r] = lu;
            a = r <= c ? lu : cmake(R(0), R(0));
        }
        S[c * kDLD + r] = a;
    }
    __syncthreads();
    if (threadIdx.x < kNP) {
        const C p = S[threadIdx.x * kDLD + threadIdx.x];
        const R d = p.x * p.x + p.y * p.y;
        rdiag[threadIdx.x] = d > R(0) ? cmake(p.x / d, -p.y / d) : cmake(R(0), R(0));
    }
    C x[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) x[i][j] = cmake(R(ty + 16 * i == tx + 16 * j ? 1 : 0), R(0));
    int step = 0;
    uinv_phase<7>(x, S, vb, rdiag, tx, ty, step);
    uinv_phase<6>(x, S, vb, rdiag, tx, ty, step);
    uinv_phase<5>(x, S, vb, rdiag, tx, ty, step);
    uinv_phase<4>(x, S, vb, rdiag, tx, ty, step);
    uinv_phase<3>(x, S, vb, rdiag, tx, ty, step);
    uinv_phase<2>(x, S, vb, rdiag, tx, ty, step);
    uinv_phase<1>(x, S, vb, rdiag, tx, ty, step);
    uinv_phase<0>(x, S, vb, rdiag, tx, ty, step);
    __syncthreads();   // U no longer read
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (ty + 16 * i <= tx + 16 * j) S[(tx + 16 * j) * kDLD + ty + 16 * i] = x[i][j];
    __syncthreads();
    C* out = Uinv + size_t(blockIdx.x) * kNP * kNP;
#pragma unroll 8
    for (int it = 0; it < kNP * kNP / 256; it++) {
        const int idx = threadIdx.x + 256 * it, r = idx & (kNP - 1), c = idx >> 7;
        out[c * kNP + r] = r <= c ? S[c * kDLD + r] : cmake(R(0), R(0));
    }
}

// A[r0 + 64*blockIdx.x ..., k0:k0+jb] <- that block times U11^{-1}.
// Thread (row, column group of 32): 32 outputs accumulated in registers.
template <typename C>
__global__ void __launch_bounds__(256) k_trsm_right(C* A, int64_t lda, int r0, int r1, int k0, int jb,
                                                   const C* __restrict__ Uinv) {
    using R = decltype(A[0].x);
    extern __shared__ __align__(16) unsigned char smraw[];
    C* u = (C*)smraw;            // Uinv[c * jb + r]
    C* blk = u + jb * jb;        // blk[q * 64 + row]
    const int rb = r0 + blockIdx.x * 64;
    const int nr = min(64, r1 - rb);
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) u[idx] = Uinv[(idx / jb) * kNP + idx % jb];
    for (int idx = threadIdx.x; idx < 64 * jb; idx += blockDim.x) {
        int row = idx & 63, q = idx >> 6;
        blk[q * 64 + row] = row < nr ? A[int64_t(k0 + q) * lda + rb + row] : cmake(R(0), R(0));
    }
    __syncthreads();
    const int row = threadIdx.x & 63, cg = threadIdx.x >> 6;   // 4 groups
    for (int c0 = cg * 32; c0 < jb; c0 += 128) {
        C acc[32];
#pragma unroll
        for (int j = 0; j < 32; j++) acc[j] = cmake(R(0), R(0));
        for (int q = 0; q < jb; q++) {
            const C x = blk[q * 64 + row];
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const C w = u[(c0 + j) * jb + q];   // broadcast
                cmac(acc[j], x, w);
            }
        }
        if (row < nr)
#pragma unroll
            for (int j = 0; j < 32; j++)
                if (c0 + j < jb) A[int64_t(k0 + c0 + j) * lda + rb + row] = acc[j];
    }
}

// ------------------------------------------------------------------ host side
template <typename C> __global__ void k_ipiv_identity(int n, int32_t* ipiv, int32_t* perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        ipiv[i] = i + 1;
        perm[i] = i;
    }
}

int trsm_lower_unit_f32(frico_gpu_ctx* ctx, float2* A, int64_t lda, int k0, int jb, int cb, int ce);  // lu.cu

template <typename C> __global__ void k_copy_block(const C* __restrict__ A, int64_t lda, int k0, int jb, C* dst) {
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < jb * jb; idx += gridDim.x * blockDim.x) {
        const int r = idx % jb, c = idx / jb;
        dst[c * kNP + r] = A[int64_t(k0 + c) * lda + k0 + r];
    }
}

// The two-CTA factor + inverses of the diagonal block at k0. With stage, the
// kernel reads the block from A and writes its LU to stage (ld 128; copied into
// A by k_uinv_blocks); without, the block is first copied to blk and its LU
// written back into A.
static int launch_diag_lu(frico_gpu_ctx* ctx, cudaStream_t st, float2* A, int64_t lda, int k0, int jb,
                          float2* Uinv, float2* Linv, float2* blk, float2* stage, DeviceStatus* dst,
                          const TcDiagSplit* sp = nullptr) {
    float2* Akk = A + int64_t(k0) * lda + k0;
    const float2* src = Akk;
    int64_t lds = lda, ldd = lda;
    float2* dlu = Akk;
    if (stage) {
        dlu = stage;
        ldd = kNP;
    } else {
        k_copy_block<float2><<<16, 256, 0, st>>>(A, lda, k0, jb, blk);
        count_launch(ctx);
        src = blk;
        lds = kNP;
    }
    TcDiagSplit none{};
    if (sp && sp->h)
        k_diag_lu<float2, true><<<2, kDiagThreads, diag_lu_smem<float2>(), st>>>(src, lds, dlu, ldd, k0, jb, Uinv,
                                                                                 Linv, dst, *sp);
    else
        k_diag_lu<float2, false><<<2, kDiagThreads, diag_lu_smem<float2>(), st>>>(src, lds, dlu, ldd, k0, jb, Uinv,
                                                                                  Linv, dst, sp ? *sp : none);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_diag_lu");
}

// U^{-1} of all diagonal blocks for the chained solves (replacing the sweep's);
// with stage, the staged LU blocks are copied into A on the way.
static int launch_uinv_blocks(frico_gpu_ctx* ctx, cudaStream_t st, float2* A, int64_t lda, int n,
                              const float2* stage, float2* Uinv0) {
    k_uinv_blocks<float2><<<(n + kNP - 1) / kNP, 256, uinv_smem<float2>(), st>>>(A, lda, n, stage, Uinv0);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_uinv_blocks");
}

// The launch sequence of a factorisation depends only on N and on the buffers it
// uses: the first call with a given key runs eagerly (and performs any one-time
// setup), the second captures the sequence into a CUDA graph, later calls
// replay it. Host-side counters (launches, GEMM flops) are restored from the
// capture on replay. With profile_kernels the sequence always runs eagerly
// (per-GEMM timing events are host-recorded).
template <typename F> static int run_lu_graph(frico_gpu_ctx* ctx, F&& enqueue) {
    LuGraph& g = ctx->lu_graph;
    if (ctx->opt.profile_kernels) return enqueue();
    const uintptr_t key[12] = {uintptr_t(ctx->n), uintptr_t(ctx->z32.p), uintptr_t(ctx->dinv128.p),
                               uintptr_t(ctx->panel_ws.p), uintptr_t(ctx->tc_ws.p), uintptr_t(ctx->status.p),
                               uintptr_t(ctx->ipiv.p), uintptr_t(ctx->perm.p), uintptr_t(ctx->stream2),
                               uintptr_t(ctx->tc_ws.bytes), uintptr_t(ctx->opt.gemm_engine),
                               uintptr_t(wait_limit(ctx))};
    const bool same = std::equal(key, key + 12, g.key);
    cudaStream_t st = ctx->stream;
    if (same && g.exec) {
        ctx->stats.kernel_launches += g.launches;
        ctx->stats.gemm_flops += g.gemm_flops;
        ctx->stats.gemm_bytes += g.gemm_bytes;
        ctx->prof_used = g.prof_used;
        return cuda_check(ctx, cudaGraphLaunch(g.exec, st), "lu graph launch");
    }
    if (!same) {   // first call with this key: run eagerly
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        std::copy(key, key + 12, g.key);
        return enqueue();
    }
    const int64_t l0 = ctx->stats.kernel_launches;
    const double f0 = ctx->stats.gemm_flops, b0 = ctx->stats.gemm_bytes;
    int rc = cuda_check(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (rc) return rc;
    rc = enqueue();
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return rc ? rc : cuda_check(ctx, e, "end capture");
    }
    rc = cuda_check(ctx, cudaGraphInstantiate(&g.exec, graph, 0), "graph instantiate");
    cudaGraphDestroy(graph);
    if (rc) {
        g.exec = nullptr;
        return rc;
    }
    g.launches = ctx->stats.kernel_launches - l0;
    g.gemm_flops = ctx->stats.gemm_flops - f0;
    g.gemm_bytes = ctx->stats.gemm_bytes - b0;
    g.prof_used = ctx->prof_used;
    return cuda_check(ctx, cudaGraphLaunch(g.exec, st), "lu graph launch");
}

// Second stream (high priority) and two events of the look-ahead, made once per context.
static int lookahead_streams(frico_gpu_ctx* ctx) {
    if (ctx->stream2) return FRICO_GPU_OK;
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    int rc = cuda_check(ctx, cudaStreamCreateWithPriority(&ctx->stream2, cudaStreamNonBlocking, hi), "stream2");
    for (int i = 0; !rc && i < 2; i++)
        rc = cuda_check(ctx, cudaEventCreateWithFlags(&ctx->la_ev[i], cudaEventDisableTiming), "look-ahead event");
    return rc;
}

int lu_factor_nopiv_fp32(frico_gpu_ctx* ctx) {
    using C = float2;
    C* A = (C*)ctx->z32.p;
    const int n = int(ctx->n);
    const int64_t lda = ctx->n;
    cudaStream_t st = ctx->stream;
    int rc;
    if ((rc = ensure(ctx, ctx->ipiv, sizeof(int32_t) * n))) return rc;
    if ((rc = ensure(ctx, ctx->perm, sizeof(int32_t) * n))) return rc;
    if ((rc = ensure(ctx, ctx->status, sizeof(DeviceStatus)))) return rc;
    const int nbk = (n + kNP - 1) / kNP;
    const bool tc = ctx->opt.gemm_engine != FRICO_GEMM_SIMT && gemm_tc_available(ctx);
    // tensor cores: one staging slot per diagonal block's LU; SIMT: one copy of the block being factored
    if ((rc = ensure(ctx, ctx->panel_ws, sizeof(C) * (tc ? size_t(nbk) : 1) * kNP * kNP + 256))) return rc;
    if ((rc = ensure(ctx, ctx->dinv128, sizeof(C) * 4 * size_t(nbk) * kNP * kNP))) return rc;
    ctx->dinv128_valid = false;
    DeviceStatus* dst = (DeviceStatus*)ctx->status.p;
    C* Blk = (C*)ctx->panel_ws.p;   // copy of the diagonal block being factored (SIMT) or the staging slots
    auto stage_of = [&](int k0) { return Blk + size_t(k0 / kNP) * kNP * kNP; };
    // inverted diagonal blocks, kept for the chained solves: L^-1 of block b, U^-1 of block b
    auto Linv_of = [&](int k0) { return (C*)ctx->dinv128.p + size_t(k0 / kNP) * kNP * kNP; };
    auto Uinv_of = [&](int k0) { return (C*)ctx->dinv128.p + size_t(nbk + k0 / kNP) * kNP * kNP; };
    if ((rc = device_once(ctx, kOnceNopivLu, [](frico_gpu_ctx* c) {
             int r = cuda_check(c, cudaFuncSetAttribute(k_diag_lu<float2, false>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        int(diag_lu_smem<float2>())), "diag smem");
             if (r) return r;
             r = cuda_check(c, cudaFuncSetAttribute(k_diag_lu<float2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    int(diag_lu_smem<float2>())), "diag smem");
             if (r) return r;
             r = cuda_check(c, cudaFuncSetAttribute(k_uinv_blocks<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    int(uinv_smem<float2>())), "uinv smem");
             if (r) return r;
             return cuda_check(c, cudaFuncSetAttribute(k_trsm_right<float2>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       int(sizeof(float2) * (kNP * kNP + 64 * kNP))),
                               "trsm_right smem");
         })))
        return rc;
    if ((ctx->opt.gemm_engine == FRICO_GEMM_TC || ctx->opt.gemm_engine == FRICO_GEMM_TC_F16) && !tc)
        return set_err(ctx, FRICO_GPU_EINVAL, "tensor-core GEMM engine not available on this device");
    if (tc) {
        // every buffer the factorisation touches is sized before the first launch, so that
        // the launch sequence can be captured once and replayed as a CUDA graph
        if ((rc = ensure(ctx, ctx->tc_ws, tc_panel_ws_bytes(n)))) return rc;
        if ((rc = lookahead_streams(ctx))) return rc;
        auto enqueue = [&]() -> int {
            int rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(DeviceStatus), st), "status");
            if (rc) return rc;
            k_ipiv_identity<C><<<(n + 255) / 256, 256, 0, st>>>(n, (int32_t*)ctx->ipiv.p, (int32_t*)ctx->perm.p);
            count_launch(ctx);
            if ((rc = lookahead_streams(ctx))) return rc;
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
            cudaStream_t s2 = ctx->stream2;
            cudaEvent_t ev_narrow = ctx->la_ev[0], ev_diag = ctx->la_ev[1];
            TcDiagSplit dsp;
            if ((rc = tc_diag_split_slots(ctx, &dsp))) return rc;
            if ((rc = tc_lu_scale(ctx, A, lda, n))) return rc;   // operand scale of the 3xFP16 block columns
            if ((rc = launch_diag_lu(ctx, st, A, lda, 0, std::min(kNP, n), Uinv_of(0), Linv_of(0), nullptr,
                                     stage_of(0), dst, &dsp)))
                return rc;
            if (n > kNP && (rc = tc_lu_panel_split(ctx, A, lda, 0, kNP, n - kNP))) return rc;
            bool diag_on_s2 = false;
            for (int k0 = 0; k0 < n; k0 += kNP) {
                const int jb = std::min(kNP, n - k0);
                const int rest = n - k0 - jb;
                if (diag_on_s2 && (rc = cuda_check(ctx, cudaStreamWaitEvent(st, ev_diag, 0), "wait diag"))) return rc;
                if (rest == 0) break;
                // L21 = A21 U11^{-1}, U12 = L11^{-1} A12 on the tensor cores, one launch (A21 and
                // A12 were split before the wait above, U11^{-1} and L11^{-1} by the diagonal-block
                // kernel) that also writes both as the operands of the updates below
                TcPanel pn;
                if ((rc = tc_lu_panel(ctx, A, lda, k0, jb, rest, &pn))) return rc;
                // trailing update, next block column first; that block's LU then runs on the
                // second stream while the rest of the update (on all but two SMs) proceeds
                const int jb1 = std::min(kNP, rest);
                C* Cm = A + int64_t(k0 + jb) * lda + k0 + jb;
                cudaEvent_t* ev = prof_event_pair(ctx);
                if (ev) {
                    ctx->stats.gemm_flops += 8.0 * double(rest) * double(jb1) * double(jb);
                    ctx->stats.gemm_bytes += sizeof(C) * (2.0 * double(rest) * double(jb1) + double(rest) * jb + double(jb) * jb1);
                }
                if ((rc = tc_lu_update(ctx, pn, Cm, lda, 0, jb1, 0, ev))) return rc;
                if ((rc = cuda_check(ctx, cudaEventRecord(ev_narrow, st), "record"))) return rc;
                if ((rc = cuda_check(ctx, cudaStreamWaitEvent(s2, ev_narrow, 0), "wait narrow"))) return rc;
                if ((rc = launch_diag_lu(ctx, s2, A, lda, k0 + jb, jb1, Uinv_of(k0 + jb), Linv_of(k0 + jb), nullptr,
                                         stage_of(k0 + jb), dst, &dsp)))
                    return rc;
                if ((rc = cuda_check(ctx, cudaEventRecord(ev_diag, s2), "record"))) return rc;
                diag_on_s2 = true;
                if (rest > jb1) {
                    const int nr = rest - jb1;
                    ev = prof_event_pair(ctx);
                    if (ev) {
                        ctx->stats.gemm_flops += 8.0 * double(rest) * double(nr) * double(jb);
                        ctx->stats.gemm_bytes += sizeof(C) * (2.0 * double(rest) * double(nr) + double(jb) * nr);
                    }
                    if ((rc = tc_lu_update(ctx, pn, Cm + int64_t(jb1) * lda, lda, jb1, nr, std::max(1, sms - 2), ev)))
                        return rc;
                    // the next block column's A21 and A12 are final now: split them while its
                    // diagonal block is still being factored on the second stream
                    if ((rc = tc_lu_panel_split(ctx, A, lda, k0 + jb, jb1, nr))) return rc;
                }
                if ((rc = cuda_check(ctx, cudaGetLastError(), "nopiv lu step"))) return rc;
            }
            if ((rc = launch_uinv_blocks(ctx, st, A, lda, n, Blk, Uinv_of(0)))) return rc;
            return trsv128_prepare(ctx, st);
        };
        if ((rc = run_lu_graph(ctx, enqueue))) return rc;
    } else {
        if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(DeviceStatus), st), "status")))
            return rc;
        k_ipiv_identity<C><<<(n + 255) / 256, 256, 0, st>>>(n, (int32_t*)ctx->ipiv.p, (int32_t*)ctx->perm.p);
        count_launch(ctx);
        for (int k0 = 0; k0 < n; k0 += kNP) {
            const int jb = std::min(kNP, n - k0);
            if ((rc = launch_diag_lu(ctx, st, A, lda, k0, jb, Uinv_of(k0), Linv_of(k0), Blk, nullptr, dst))) return rc;
            const int rest = n - k0 - jb;
            if (rest > 0) {
                // SIMT engine: L21 = A21 U11^{-1} with the inverse, U12 by the unit-lower TRSM
                k_trsm_right<C><<<(rest + 63) / 64, 256, sizeof(C) * (jb * jb + 64 * jb), st>>>(
                    A, lda, k0 + jb, n, k0, jb, Uinv_of(k0));
                count_launch(ctx);
                if ((rc = trsm_lower_unit_f32(ctx, A, lda, k0, jb, k0 + jb, n))) return rc;
                C* Cm = A + int64_t(k0 + jb) * lda + k0 + jb;
                const C* Lm = A + int64_t(k0) * lda + k0 + jb;
                const C* Um = A + int64_t(k0 + jb) * lda + k0;
                cudaEvent_t* ev = prof_event_pair(ctx);
                if (ev) {
                    ctx->stats.gemm_flops += 8.0 * double(rest) * double(rest) * double(jb);
                    ctx->stats.gemm_bytes += sizeof(C) * (2.0 * double(rest) * double(rest) + 2.0 * double(rest) * jb);
                }
                if (ev) cudaEventRecord(ev[0], st);
                if ((rc = gemm_update_simt32(ctx, Cm, lda, Lm, lda, Um, lda, rest, rest, jb))) return rc;
                if (ev) cudaEventRecord(ev[1], st);
            }
            if ((rc = cuda_check(ctx, cudaGetLastError(), "nopiv lu step"))) return rc;
        }
        if ((rc = launch_uinv_blocks(ctx, st, A, lda, n, nullptr, Uinv_of(0)))) return rc;
        if ((rc = trsv128_prepare(ctx, st))) return rc;
    }
    prof_event_collect(ctx);
    DeviceStatus hs;
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, st), "status")))
        return rc;
    if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "nopiv lu sync"))) return rc;
    if (hs.err == FRICO_DEV_ERR_TIMEOUT) return set_err(ctx, FRICO_GPU_ETIMEOUT, "tensor-core GEMM wait timed out");
    ctx->info = hs.info;
    if (hs.info != 0) return FRICO_GPU_OK;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(DeviceStatus), st), "status reset")))
        return rc;
    if ((rc = trsv_prepare_nopiv(ctx))) return rc;
    return FRICO_GPU_OK;
}

}  // namespace frico
