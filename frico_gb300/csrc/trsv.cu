// Triangular solves with the LU factors (the zgetrs part of FRICO's
// solve_general, src/lapack_wrappers.cpp:81-89), one launch per triangle.
//
// After factorisation the 64x64 diagonal blocks of L (unit lower) and U are
// inverted once (k_invert_diag). A solve then runs as a single kernel whose
// CTAs take block rows in ticket order (atomic counter, so a CTA only ever
// waits for blocks owned by CTAs that are already running). Block row b
// accumulates  y_b = w_b - sum_{c before b} T_bc y_c  as the y_c are published
// (per-block flag = launch epoch), applies the inverted diagonal block and
// publishes y_b. The only sequential part is the chain of 64-row blocks; the
// off-diagonal work of every block overlaps with the wait. Every wait is
// bounded: on timeout the CTA records FRICO_DEV_ERR_TIMEOUT and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "common.cuh"

namespace frico {

static const int kB = 64;        // block rows
static const int kRc = 8;        // right-hand sides per pass

// One CTA per diagonal block: Linv = L_bb^{-1} (unit lower), Uinv = U_bb^{-1}.
// Thread j owns column j of the inverse (forward / backward substitution
// against e_j); columns are held in shared memory, lanes on consecutive words.
template <typename C>
__global__ void __launch_bounds__(128) k_invert_diag(const C* __restrict__ LU, int64_t lda, int n, C* Linv, C* Uinv) {
    __shared__ C T[kB][kB + 1];   // T[r][c] = block entry (row r, col c)
    __shared__ C X[kB][kB + 1];   // X[r][j] = inverse entry (row r, col j)
    const int b = blockIdx.x, r0 = b * kB, bs = min(kB, n - r0);
    for (int idx = threadIdx.x; idx < kB * kB; idx += blockDim.x) {
        int r = idx % kB, c = idx / kB;
        T[r][c] = (r < bs && c < bs) ? LU[int64_t(r0 + c) * lda + r0 + r] : cmake(decltype(T[0][0].x)(0), decltype(T[0][0].x)(0));
    }
    __syncthreads();
    using R = decltype(T[0][0].x);
    const int j = threadIdx.x;
    if (j < kB) {
        // lower: X[:, j] = L^{-1} e_j
        for (int r = 0; r < kB; r++) {
            C s = cmake(R(r == j ? 1 : 0), R(0));
            for (int q = j; q < r; q++) s = cfms(s, T[r][q], X[q][j]);
            X[r][j] = (r < j) ? cmake(R(0), R(0)) : s;
        }
    }
    __syncthreads();
    C* Lo = Linv + int64_t(b) * kB * kB;
    for (int idx = threadIdx.x; idx < kB * kB; idx += blockDim.x) {
        int r = idx % kB, c = idx / kB;
        Lo[idx] = X[r][c];
    }
    __syncthreads();
    if (j < kB) {
        // upper: X[:, j] = U^{-1} e_j (rows beyond bs act as identity)
        for (int r = kB - 1; r >= 0; r--) {
            C s = cmake(R(r == j ? 1 : 0), R(0));
            if (r > j || r >= bs) {
                X[r][j] = (r < bs) ? cmake(R(0), R(0)) : s;
                continue;
            }
            for (int q = r + 1; q <= j && q < bs; q++) s = cfms(s, T[r][q], X[q][j]);
            X[r][j] = cdiv(s, T[r][r]);
        }
    }
    __syncthreads();
    C* Uo = Uinv + int64_t(b) * kB * kB;
    for (int idx = threadIdx.x; idx < kB * kB; idx += blockDim.x) {
        int r = idx % kB, c = idx / kB;
        Uo[idx] = X[r][c];
    }
}

// W <- T^{-1} W for T = unit-lower L (LOWER) or upper U, nrhs <= kRc.
// Critical path per chain link: flag seen by warp 0 -> warp 0 loads the
// published block (double-buffered, one barrier) -> 16 FMAs per thread from
// prefetched registers -> reduction -> Dinv (prefetched) -> store, fence, flag.
template <typename C, bool LOWER, int NC>
__global__ void __launch_bounds__(256) k_trsv_chain(const C* __restrict__ LU, int64_t lda, int n, const C* __restrict__ Dinv,
                                                   C* W, int64_t ldw, int nrhs, int* flags, unsigned* ticket, int epoch,
                                                   DeviceStatus* st, long long lim) {
    using R = decltype(W[0].x);
    __shared__ C xs[2][kB][kRc];         // published blocks y_c (double buffer)
    __shared__ C part[4][kB][kRc];       // partial sums of the 4 column groups
    __shared__ C yb[kB][kRc];
    __shared__ int s_t, s_abort;
    const int nb = (n + kB - 1) / kB;
    if (threadIdx.x == 0) {
        s_t = int(atomicAdd(ticket, 1u));
        s_abort = 0;
    }
    __syncthreads();
    const int t = s_t;
    if (t >= nb) return;
    const int b = LOWER ? t : nb - 1 - t;
    const int r0 = b * kB, bs = min(kB, n - r0);
    const int r = threadIdx.x & 63, q = threadIdx.x >> 6;   // row in block, column group (16 cols)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // independent of the chain: own right-hand side (into yb), Dinv block, first T block
    if (q == 0)
#pragma unroll
        for (int c = 0; c < NC; c++)
            yb[r][c] = (r < bs && c < nrhs) ? W[int64_t(c) * ldw + r0 + r] : cmake(R(0), R(0));
    const C* D = Dinv + int64_t(b) * kB * kB;
    C dv[16];
#pragma unroll
    for (int cc = 0; cc < 16; cc++) dv[cc] = (r < bs && q * 16 + cc < bs) ? D[(q * 16 + cc) * kB + r] : cmake(R(0), R(0));
    C acc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = cmake(R(0), R(0));
    const int ndep = LOWER ? b : nb - 1 - b;
    C lv[16];
    auto load_block = [&](int k) {
        const int cb = LOWER ? k : nb - 1 - k;
        const int c0 = cb * kB, cs = min(kB, n - c0);
        const C* col = LU + int64_t(c0 + q * 16) * lda + r0 + r;
#pragma unroll
        for (int cc = 0; cc < 16; cc++)
            lv[cc] = (r < bs && q * 16 + cc < cs) ? col[int64_t(cc) * lda] : cmake(R(0), R(0));
    };
    if (ndep > 0) load_block(0);

    for (int k = 0; k < ndep; k++) {
        const int cb = LOWER ? k : nb - 1 - k;
        const int c0 = cb * kB, cs = min(kB, n - c0);
        const int buf = k & 1;
        if (warp == 0) {
            if (lane == 0) {
                volatile int* f = flags + cb;
                volatile int* e = &st->err;
                long long t0 = clock64();
                while (*f != epoch) {
                    if (*e) { s_abort = 1; break; }
                    if (clock64() - t0 > lim) {
                        if (atomicCAS(&st->err, 0, FRICO_DEV_ERR_TIMEOUT) == 0) st->where = cb;
                        s_abort = 1;
                        break;
                    }
                }
            }
            __syncwarp();
            // rows past a short last block are zero: they meet zero T entries, and
            // stale shared memory there could hold NaN (0 * NaN = NaN)
            for (int idx = lane; idx < kB * nrhs; idx += 32) {
                const int rr = idx & (kB - 1), c = idx >> 6;
                xs[buf][rr][c] = rr < cs ? __ldcg(&W[int64_t(c) * ldw + c0 + rr]) : cmake(R(0), R(0));
            }
        }
        __syncthreads();
        if (s_abort) return;
        C cur[16];
#pragma unroll
        for (int cc = 0; cc < 16; cc++) cur[cc] = lv[cc];
        if (k + 1 < ndep) load_block(k + 1);   // prefetch the next block's T values
#pragma unroll
        for (int cc = 0; cc < 16; cc++) {
#pragma unroll
            for (int c = 0; c < NC; c++)
                if (NC == 1 || c < nrhs) acc[c] = cfms(acc[c], cur[cc], xs[buf][q * 16 + cc][c]);
        }
    }
    // y_pre = w_b + sum of the four partial sums
#pragma unroll
    for (int c = 0; c < NC; c++) part[q][r][c] = acc[c];
    __syncthreads();
    if (q == 0)
#pragma unroll
        for (int c = 0; c < NC; c++)
            yb[r][c] = cadd(yb[r][c], cadd(cadd(part[0][r][c], part[1][r][c]), cadd(part[2][r][c], part[3][r][c])));
    __syncthreads();
    // y = Dinv_b * y_pre
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = cmake(R(0), R(0));
#pragma unroll
    for (int cc = 0; cc < 16; cc++) {
#pragma unroll
        for (int c = 0; c < NC; c++)
            if (NC == 1 || c < nrhs) acc[c] = cadd(acc[c], cmul(dv[cc], yb[q * 16 + cc][c]));
    }
#pragma unroll
    for (int c = 0; c < NC; c++) part[q][r][c] = acc[c];
    __syncthreads();
    if (q == 0 && r < bs)
        for (int c = 0; c < nrhs; c++)
            W[int64_t(c) * ldw + r0 + r] = cadd(cadd(part[0][r][c], part[1][r][c]), cadd(part[2][r][c], part[3][r][c]));
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicExch(flags + b, epoch);
}

// The same chain with 128-row blocks for the complex64 no-pivot factors, whose
// 128 x 128 inverted diagonal blocks come out of the factorisation (column-major,
// identity-padded past the last row). Two changes shorten each link of the chain:
//  * the last dependency is folded into a precomputed block: with
//    M_b = Dinv_b T_{b,p} (p the block solved just before b),
//      x_b = Dinv_b (w_b - sum_{c != p} T_bc x_c) - M_b x_p,
//    so the first term is formed while x_p is still awaited and only one
//    128 x 128 block product remains once it arrives;
//  * results go to a buffer pre-filled with 0xFF bytes (a NaN pattern that
//    arithmetic does not produce): a block waits for x_c by loading x_c itself
//    until no half of it still holds the pattern, with no flag, fence or second
//    round trip. Each 32-bit half is written once, so a half read is either the
//    pattern or final.
// 512 threads (row r, group q of 32 columns); Dinv_b in shared memory.
constexpr int kB2 = 128;
constexpr size_t kChain128Smem = sizeof(float2) * (size_t(kB2) * kB2 + (2 + 4 + 1) * size_t(kB2) * kRc);
constexpr unsigned kUnset = 0xFFFFFFFFu;

__device__ __forceinline__ float2 ld_relaxed_f2(const float2* p) {
    float2 v;
    asm volatile("ld.relaxed.gpu.global.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_f2(float2* p, float2 v) {
    asm volatile("st.relaxed.gpu.global.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(v.x), "f"(v.y) : "memory");
}

// M_b for the chained solves: blockIdx.y = 0: Linv_b L_{b,b-1} (b >= 1), 1: Uinv_b U_{b,b+1}
// (b <= nb - 2); 128 x 128 column-major into M + (y nb + b) 128^2. blockIdx.z picks
// the 64 x 64 quadrant of the product; operands go through shared memory in 16-wide
// slabs; thread (tx, ty) owns rows ty + 16 i, columns tx + 16 j (i, j < 4).
__global__ void __launch_bounds__(256) k_chain_mats(const float2* __restrict__ LU, int64_t lda, int n,
                                                    const float2* __restrict__ Dinv, float2* __restrict__ M) {
    __shared__ float2 As[64][17];       // As[r][k]
    __shared__ float2 Bs[16][64 + 1];   // Bs[k][j]
    const int nb = (n + kB2 - 1) / kB2, b = blockIdx.x, upper = blockIdx.y;
    if (upper ? b >= nb - 1 : b == 0) return;
    const int qr = (blockIdx.z & 1) * 64, qc = (blockIdx.z >> 1) * 64;
    const float2* D = Dinv + (size_t(upper) * nb + b) * kB2 * kB2;
    const int r0 = b * kB2, bs = min(kB2, n - r0);
    const int cb = upper ? b + 1 : b - 1, c0 = cb * kB2, cs = min(kB2, n - c0);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = make_float2(0.f, 0.f);
    for (int k0 = 0; k0 < kB2; k0 += 16) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < 64 * 16; idx += 256) {
            const int r = idx & 63, k = idx >> 6;
            As[r][k] = D[int64_t(k0 + k) * kB2 + qr + r];
            const int kk = idx & 15, j = idx >> 4;   // T block row k0 + kk (of block b), column qc + j (of block cb)
            Bs[kk][j] = (k0 + kk < bs && qc + j < cs) ? LU[int64_t(c0 + qc + j) * lda + r0 + k0 + kk]
                                                      : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < 16; k++) {
            float2 a[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[ty + 16 * i][k];
#pragma unroll
            for (int j = 0; j < 4; j++) bv[j] = Bs[k][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    acc[i][j].x = fmaf(a[i].x, bv[j].x, fmaf(-a[i].y, bv[j].y, acc[i][j].x));
                    acc[i][j].y = fmaf(a[i].x, bv[j].y, fmaf(a[i].y, bv[j].x, acc[i][j].y));
                }
        }
    }
    float2* out = M + (size_t(upper) * nb + b) * kB2 * kB2;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) out[(qc + tx + 16 * j) * kB2 + qr + ty + 16 * i] = acc[i][j];
}

// NC: right-hand sides per launch (1, 2, 4 or 8), a compile-time bound on the column loops
template <bool LOWER, int NC>
__global__ void __launch_bounds__(512) k_trsv_chain128(const float2* __restrict__ LU, int64_t lda, int n,
                                                      const float2* __restrict__ Dinv, const float2* __restrict__ M,
                                                      const float2* __restrict__ Win, int64_t ldin, float2* Xout,
                                                      int64_t ldout, int nrhs, unsigned* ticket, DeviceStatus* st,
                                                      long long lim) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float2* Ds = (float2*)smraw;                                                  // [c * 128 + r]
    float2 (*xs)[kB2][kRc] = reinterpret_cast<float2 (*)[kB2][kRc]>(Ds + kB2 * kB2);   // [2]
    float2 (*part)[kB2][kRc] = xs + 2;                                            // [4]
    float2 (*yb)[kRc] = reinterpret_cast<float2 (*)[kRc]>(part + 4);             // [128]
    __shared__ int s_t, s_abort;
    const int nb = (n + kB2 - 1) / kB2;
    if (threadIdx.x == 0) {
        s_t = int(atomicAdd(ticket, 1u));
        s_abort = 0;
    }
    __syncthreads();
    const int t = s_t;
    if (t >= nb) return;
    const int b = LOWER ? t : nb - 1 - t;
    const int r0 = b * kB2, bs = min(kB2, n - r0);
    const int r = threadIdx.x & 127, q = threadIdx.x >> 7;   // row in block, column group (32 cols)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float2 z = make_float2(0.f, 0.f);

    // independent of the chain: Dinv of this block, own right-hand side, first T block;
    // M_b (the last dependency's block, loaded once the one before it is in) into L2 now,
    // so that its load on the chain waits on L2 rather than DRAM
    if (t > 0) {
        const char* mb = reinterpret_cast<const char*>(M + int64_t(b) * kB2 * kB2);
        for (int line = threadIdx.x; line < kB2 * kB2 * int(sizeof(float2)) / 128; line += 512)
            asm volatile("prefetch.global.L2::evict_last [%0];" ::"l"(mb + int64_t(line) * 128));
    }
    const float2* D = Dinv + int64_t(b) * kB2 * kB2;
    for (int idx = threadIdx.x; idx < kB2 * kB2; idx += 512) Ds[idx] = D[idx];
    if (q == 0)
#pragma unroll
        for (int c = 0; c < NC; c++) yb[r][c] = (r < bs && c < nrhs) ? Win[int64_t(c) * ldin + r0 + r] : z;
    float2 acc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = z;
    const int ndep = LOWER ? b : nb - 1 - b;
    float2 lv[32];
    // T block of dependency k, or M_b for the last one (rows of this block, 32 columns of group q)
    auto load_block = [&](int k) {
        if (k == ndep - 1) {
            const float2* m = M + int64_t(b) * kB2 * kB2 + int64_t(q * 32) * kB2 + r;
#pragma unroll
            for (int cc = 0; cc < 32; cc++) lv[cc] = m[cc * kB2];
        } else {
            const int cb = LOWER ? k : nb - 1 - k;
            const int c0 = cb * kB2, cs = min(kB2, n - c0);
            const float2* col = LU + int64_t(c0 + q * 32) * lda + r0 + r;
#pragma unroll
            for (int cc = 0; cc < 32; cc++) lv[cc] = (r < bs && q * 32 + cc < cs) ? col[int64_t(cc) * lda] : z;
        }
    };
    // x of block column cb into xs[buf] once every value of it is final (warp 0; bounded wait).
    // Per right-hand side a lane issues its 4 loads before it checks any, so that they cost
    // one L2 round trip rather than four.
    auto await_x = [&](int cb, int buf) {
        if (warp == 0) {
            const int c0 = cb * kB2, cs = min(kB2, n - c0);
            long long t0 = clock64();
            volatile int* e = &st->err;
            while (true) {
                bool pending = false;
#pragma unroll
                for (int c = 0; c < NC; c++) {
                    if (NC > 1 && c >= nrhs) break;
                    float2 v[4];
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const int rr = lane + 32 * i;
                        v[i] = rr < cs ? ld_relaxed_f2(&Xout[int64_t(c) * ldout + c0 + rr]) : z;
                    }
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        pending |= __float_as_uint(v[i].x) == kUnset || __float_as_uint(v[i].y) == kUnset;
                        xs[buf][lane + 32 * i][c] = v[i];
                    }
                }
                if (!__any_sync(0xffffffffu, pending)) break;
                if (lane == 0 && (*e || clock64() - t0 > lim)) {
                    if (!*e && atomicCAS(&st->err, 0, FRICO_DEV_ERR_TIMEOUT) == 0) st->where = cb;
                    s_abort = 1;
                }
                if (__shfl_sync(0xffffffffu, s_abort, 0)) break;
            }
        }
        __syncthreads();
    };
    if (ndep > 0) load_block(0);

    for (int k = 0; k < ndep - 1; k++) {
        const int cb = LOWER ? k : nb - 1 - k;
        const int buf = k & 1;
        await_x(cb, buf);
        if (s_abort) return;
#pragma unroll
        for (int cc = 0; cc < 32; cc++) {
#pragma unroll
            for (int c = 0; c < NC; c++)
                if (NC == 1 || c < nrhs) acc[c] = cfms(acc[c], lv[cc], xs[buf][q * 32 + cc][c]);
        }
        load_block(k + 1);   // next block's T values (or M_b), while the next x is awaited
    }
    // y' = Dinv_b (w_b - sum over all but the last dependency), before the last x is in
#pragma unroll
    for (int c = 0; c < NC; c++) part[q][r][c] = acc[c];
    __syncthreads();
    if (q == 0)
#pragma unroll
        for (int c = 0; c < NC; c++)
            yb[r][c] = cadd(yb[r][c], cadd(cadd(part[0][r][c], part[1][r][c]), cadd(part[2][r][c], part[3][r][c])));
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = z;
#pragma unroll 8
    for (int cc = 0; cc < 32; cc++) {
        const float2 d = Ds[(q * 32 + cc) * kB2 + r];
#pragma unroll
        for (int c = 0; c < NC; c++)
            if (NC == 1 || c < nrhs) acc[c] = cadd(acc[c], cmul(d, yb[q * 32 + cc][c]));
    }
#pragma unroll
    for (int c = 0; c < NC; c++) part[q][r][c] = acc[c];
    __syncthreads();
    if (q == 0)
#pragma unroll
        for (int c = 0; c < NC; c++)
            yb[r][c] = cadd(cadd(part[0][r][c], part[1][r][c]), cadd(part[2][r][c], part[3][r][c]));
    // the last dependency: x_b = y' - M_b x_p
    if (ndep > 0) {
        const int kl = ndep - 1, cb = LOWER ? kl : nb - 1 - kl;
        await_x(cb, kl & 1);   // (its barrier also publishes yb)
        if (s_abort) return;
#pragma unroll
        for (int c = 0; c < NC; c++) acc[c] = z;
#pragma unroll
        for (int cc = 0; cc < 32; cc++) {
#pragma unroll
            for (int c = 0; c < NC; c++)
                if (NC == 1 || c < nrhs) acc[c] = cfms(acc[c], lv[cc], xs[kl & 1][q * 32 + cc][c]);
        }
#pragma unroll
        for (int c = 0; c < NC; c++) part[q][r][c] = acc[c];
        __syncthreads();
        if (q == 0 && r < bs)
            for (int c = 0; c < nrhs; c++)
                st_relaxed_f2(&Xout[int64_t(c) * ldout + r0 + r],
                              cadd(yb[r][c], cadd(cadd(part[0][r][c], part[1][r][c]), cadd(part[2][r][c], part[3][r][c]))));
    } else {
        __syncthreads();
        if (q == 0 && r < bs)
            for (int c = 0; c < nrhs; c++) st_relaxed_f2(&Xout[int64_t(c) * ldout + r0 + r], yb[r][c]);
    }
}

// ------------------------------------------------------------------ host side
template <typename C, bool LOWER>
static void launch_chain_nc(int nc, int nb, cudaStream_t st, const C* LU, int n, const C* D, C* W, int64_t ldw,
                            int* flags, unsigned* ticket, int epoch, DeviceStatus* dst, long long lim) {
    if (nc == 1)
        k_trsv_chain<C, LOWER, 1><<<nb, 256, 0, st>>>(LU, n, n, D, W, ldw, nc, flags, ticket, epoch, dst, lim);
    else if (nc == 2)
        k_trsv_chain<C, LOWER, 2><<<nb, 256, 0, st>>>(LU, n, n, D, W, ldw, nc, flags, ticket, epoch, dst, lim);
    else if (nc <= 4)
        k_trsv_chain<C, LOWER, 4><<<nb, 256, 0, st>>>(LU, n, n, D, W, ldw, nc, flags, ticket, epoch, dst, lim);
    else
        k_trsv_chain<C, LOWER, kRc><<<nb, 256, 0, st>>>(LU, n, n, D, W, ldw, nc, flags, ticket, epoch, dst, lim);
}

template <typename C>
static void launch_chain(bool lower, int nc, int nb, cudaStream_t st, const C* LU, int n, const C* D, C* W,
                         int64_t ldw, int* flags, unsigned* ticket, int epoch, DeviceStatus* dst, long long lim) {
    if (lower)
        launch_chain_nc<C, true>(nc, nb, st, LU, n, D, W, ldw, flags, ticket, epoch, dst, lim);
    else
        launch_chain_nc<C, false>(nc, nb, st, LU, n, D, W, ldw, flags, ticket, epoch, dst, lim);
}

struct TrsvWs {
    void* dinv = nullptr;      // Linv blocks then Uinv blocks
    int* flags = nullptr;
    unsigned* ticket = nullptr;
    int epoch = 0;
};

template <typename C>
int trsv_prepare(frico_gpu_ctx* ctx, const C* LU, DevBuf& ws_buf, DevBuf& flag_buf) {
    const int n = int(ctx->n), nb = (n + kB - 1) / kB;
    int rc;
    ctx->dinv128_valid = false;   // set again by the no-pivot factorisation, which fills dinv128
    ctx->dinv64_stale = false;
    if ((rc = ensure(ctx, ws_buf, sizeof(C) * size_t(2) * nb * kB * kB))) return rc;
    if ((rc = ensure(ctx, flag_buf, sizeof(int) * (nb + 64)))) return rc;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(flag_buf.p, 0, sizeof(int) * (nb + 64), ctx->stream), "flags")))
        return rc;
    C* Linv = (C*)ws_buf.p;
    C* Uinv = Linv + size_t(nb) * kB * kB;
    k_invert_diag<C><<<nb, 128, 0, ctx->stream>>>(LU, n, n, Linv, Uinv);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_invert_diag");
}

template <typename C>
int trsv_solve(frico_gpu_ctx* ctx, const C* LU, DevBuf& ws_buf, DevBuf& flag_buf, C* W, int nrhs, int64_t ldw) {
    const int n = int(ctx->n), nb = (n + kB - 1) / kB;
    C* Linv = (C*)ws_buf.p;
    C* Uinv = Linv + size_t(nb) * kB * kB;
    int* flags = (int*)flag_buf.p;
    unsigned* ticket = (unsigned*)(flags + nb + 32);
    DeviceStatus* dst = (DeviceStatus*)ctx->status.p;
    int rc;
    // a wait that gave up in an earlier solve must not end this one's kernels
    if ((rc = cuda_check(ctx, cudaMemsetAsync(&dst->err, 0, sizeof(int), ctx->stream), "status"))) return rc;
    for (int c0 = 0; c0 < nrhs; c0 += kRc) {
        int nc = std::min(kRc, nrhs - c0);
        for (int pass = 0; pass < 2; pass++) {
            int epoch = ++ctx->trsv_epoch;
            if ((rc = cuda_check(ctx, cudaMemsetAsync(ticket, 0, sizeof(unsigned), ctx->stream), "ticket"))) return rc;
            launch_chain<C>(pass == 0, nc, nb, ctx->stream, LU, n, pass == 0 ? Linv : Uinv, W + c0 * ldw, ldw, flags,
                            ticket, epoch, dst, wait_limit(ctx));
            count_launch(ctx);
        }
    }
    return cuda_check(ctx, cudaGetLastError(), "k_trsv_chain");
}

int trsv_prepare_fp64(frico_gpu_ctx* ctx) {
    return trsv_prepare<double2>(ctx, (const double2*)ctx->z64.p, ctx->dinv, ctx->trsv_flags);
}
// After the no-pivot factorisation: the chain flags and ticket (the 128-row solves
// use the ticket); the 64-row inverted blocks are left for first use
// (trsv_dinv64_fp32), they only serve the transposed solves of the adjoint.
int trsv_prepare_nopiv(frico_gpu_ctx* ctx) {
    const int nb = int((ctx->n + kB - 1) / kB);
    int rc;
    if ((rc = ensure(ctx, ctx->trsv_flags, sizeof(int) * (nb + 64)))) return rc;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->trsv_flags.p, 0, sizeof(int) * (nb + 64), ctx->stream), "flags")))
        return rc;
    ctx->dinv64_stale = true;
    ctx->dinv128_valid = true;
    return FRICO_GPU_OK;
}

int trsv_dinv64_fp32(frico_gpu_ctx* ctx) {
    if (!ctx->dinv64_stale) return FRICO_GPU_OK;
    const int n = int(ctx->n), nb = (n + kB - 1) / kB;
    int rc;
    if ((rc = ensure(ctx, ctx->dinv, sizeof(float2) * size_t(2) * nb * kB * kB))) return rc;
    float2* Linv = (float2*)ctx->dinv.p;
    k_invert_diag<float2><<<nb, 128, 0, ctx->stream>>>((const float2*)ctx->z32.p, n, n, Linv, Linv + size_t(nb) * kB * kB);
    count_launch(ctx);
    ctx->dinv64_stale = false;
    return cuda_check(ctx, cudaGetLastError(), "k_invert_diag");
}

int trsv_prepare_fp32(frico_gpu_ctx* ctx) {
    return trsv_prepare<float2>(ctx, (const float2*)ctx->z32.p, ctx->dinv, ctx->trsv_flags);
}
int trsv_solve_fp64(frico_gpu_ctx* ctx, double2* W, int nrhs, int64_t ldw) {
    return trsv_solve<double2>(ctx, (const double2*)ctx->z64.p, ctx->dinv, ctx->trsv_flags, W, nrhs, ldw);
}
// M blocks of the 128-row chains (after dinv128's L^{-1}, U^{-1} blocks), once per factorisation.
int trsv128_prepare(frico_gpu_ctx* ctx, cudaStream_t st) {
    const int n = int(ctx->n), nb = (n + kB2 - 1) / kB2;
    const float2* Dinv = (const float2*)ctx->dinv128.p;
    k_chain_mats<<<dim3(nb, 2, 4), 256, 0, st>>>((const float2*)ctx->z32.p, n, n, Dinv,
                                              (float2*)ctx->dinv128.p + size_t(2) * nb * kB2 * kB2);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_chain_mats");
}

template <bool LOWER>
static void launch_chain128(int nc, int nb, cudaStream_t st, const float2* LU, int n, const float2* D,
                            const float2* M, const float2* Win, int64_t ldin, float2* Xout, int64_t ldout,
                            unsigned* ticket, DeviceStatus* dst, long long lim) {
    if (nc == 1)
        k_trsv_chain128<LOWER, 1><<<nb, 512, kChain128Smem, st>>>(LU, n, n, D, M, Win, ldin, Xout, ldout, nc, ticket, dst, lim);
    else if (nc == 2)
        k_trsv_chain128<LOWER, 2><<<nb, 512, kChain128Smem, st>>>(LU, n, n, D, M, Win, ldin, Xout, ldout, nc, ticket, dst, lim);
    else if (nc <= 4)
        k_trsv_chain128<LOWER, 4><<<nb, 512, kChain128Smem, st>>>(LU, n, n, D, M, Win, ldin, Xout, ldout, nc, ticket, dst, lim);
    else
        k_trsv_chain128<LOWER, kRc><<<nb, 512, kChain128Smem, st>>>(LU, n, n, D, M, Win, ldin, Xout, ldout, nc, ticket,
                                                                     dst, lim);
}

// Lower pass W -> X (scratch), upper pass X -> W; each output pre-filled with the pattern.
static int trsv128_solve(frico_gpu_ctx* ctx, float2* W, int nrhs, int64_t ldw) {
    const int n = int(ctx->n), nb = (n + kB2 - 1) / kB2, nb64 = (n + kB - 1) / kB;
    int* flags = (int*)ctx->trsv_flags.p;
    unsigned* ticket = (unsigned*)(flags + nb64 + 32);
    DeviceStatus* dst = (DeviceStatus*)ctx->status.p;
    const float2* LU = (const float2*)ctx->z32.p;
    const float2* Linv = (const float2*)ctx->dinv128.p;
    const float2* Uinv = Linv + size_t(nb) * kB2 * kB2;
    const float2* Mlow = Linv + size_t(2) * nb * kB2 * kB2;
    const float2* Mup = Linv + size_t(3) * nb * kB2 * kB2;
    const long long lim = wait_limit(ctx);
    cudaStream_t st = ctx->stream;
    int rc = device_once(ctx, kOnceTrsv128, [](frico_gpu_ctx* c) {
        const void* fns[8] = {(const void*)k_trsv_chain128<true, 1>,   (const void*)k_trsv_chain128<true, 2>,
                              (const void*)k_trsv_chain128<true, 4>,   (const void*)k_trsv_chain128<true, kRc>,
                              (const void*)k_trsv_chain128<false, 1>,  (const void*)k_trsv_chain128<false, 2>,
                              (const void*)k_trsv_chain128<false, 4>,  (const void*)k_trsv_chain128<false, kRc>};
        for (const void* f : fns) {
            int r = cuda_check(c, cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kChain128Smem)),
                               "chain128 smem");
            if (r) return r;
        }
        return 0;
    });
    if (rc) return rc;
    if ((rc = ensure(ctx, ctx->trsv_x, sizeof(float2) * size_t(n) * kRc))) return rc;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(&dst->err, 0, sizeof(int), st), "status"))) return rc;
    float2* X = (float2*)ctx->trsv_x.p;
    for (int c0 = 0; c0 < nrhs; c0 += kRc) {
        const int nc = std::min(kRc, nrhs - c0);
        float2* Wc = W + c0 * ldw;
        if ((rc = cuda_check(ctx, cudaMemsetAsync(X, 0xFF, sizeof(float2) * size_t(n) * nc, st), "unset x"))) return rc;
        if ((rc = cuda_check(ctx, cudaMemsetAsync(ticket, 0, sizeof(unsigned), st), "ticket"))) return rc;
        launch_chain128<true>(nc, nb, st, LU, n, Linv, Mlow, Wc, ldw, X, n, ticket, dst, lim);
        if ((rc = cuda_check(ctx, cudaMemset2DAsync(Wc, sizeof(float2) * ldw, 0xFF, sizeof(float2) * n, nc, st),
                             "unset w")))
            return rc;
        if ((rc = cuda_check(ctx, cudaMemsetAsync(ticket, 0, sizeof(unsigned), st), "ticket"))) return rc;
        launch_chain128<false>(nc, nb, st, LU, n, Uinv, Mup, X, n, Wc, ldw, ticket, dst, lim);
        count_launch(ctx, 2);
    }
    return cuda_check(ctx, cudaGetLastError(), "k_trsv_chain128");
}

int trsv_solve_fp32(frico_gpu_ctx* ctx, float2* W, int nrhs, int64_t ldw) {
    if (ctx->dinv128_valid) return trsv128_solve(ctx, W, nrhs, ldw);
    return trsv_solve<float2>(ctx, (const float2*)ctx->z32.p, ctx->dinv, ctx->trsv_flags, W, nrhs, ldw);
}

// The same chained solves with caller-supplied factors and inverted diagonal
// blocks (first nb blocks for the lower pass, next nb for the upper pass); the
// transposed solves of the adjoint use them on transposed factors.
int trsv_solve_with_fp64(frico_gpu_ctx* ctx, const double2* LU, DevBuf& dinv, double2* W, int nrhs, int64_t ldw) {
    return trsv_solve<double2>(ctx, LU, dinv, ctx->trsv_flags, W, nrhs, ldw);
}
int trsv_solve_with_fp32(frico_gpu_ctx* ctx, const float2* LU, DevBuf& dinv, float2* W, int nrhs, int64_t ldw) {
    return trsv_solve<float2>(ctx, LU, dinv, ctx->trsv_flags, W, nrhs, ldw);
}

// Checks the device status word after a solve (host-synchronous).
int trsv_check(frico_gpu_ctx* ctx, DeviceStatus* out) {
    DeviceStatus hs;
    int rc = cuda_check(ctx, cudaMemcpyAsync(&hs, ctx->status.p, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream),
                        "status");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    if (rc) return rc;
    if (out) *out = hs;
    if (hs.err == FRICO_DEV_ERR_TIMEOUT) {
        char buf[96];
        snprintf(buf, sizeof buf, "triangular solve wait timed out at block %d", hs.where);
        return set_err(ctx, FRICO_GPU_ETIMEOUT, buf);
    }
    return FRICO_GPU_OK;
}

}  // namespace frico
