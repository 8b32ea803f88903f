// Tensor-core (tcgen05) trailing update of the complex64 LU: C -= A B.
//
// Complex interleaved storage maps onto one real GEMM. With A (m x k) and
// B (k x n) complex, column-major:
//   A* (2m x 2k, K-major):  row 2r   = (Ar[r,0], -Ai[r,0], Ar[r,1], -Ai[r,1], ...)
//                           row 2r+1 = (Ai[r,0],  Ar[r,0], Ai[r,1],  Ar[r,1], ...)
//   B^ (n x 2k, K-major):   row j    = (Br[0,j], Bi[0,j], Br[1,j], Bi[1,j], ...)
//                                      = column j of B as it lies in memory
//   (A* B^T)[2r + s, j] = Re/Im (A B)[r, j]  for s = 0/1,
// i.e. the real product lands exactly in the interleaved column-major layout
// of C, which the epilogue updates in place.
//
// Precision: three products of split operands, accumulated in FP32.
//  3xTF32 (k_gemm_tf32x3): every operand x is split into hi = x with the low 13
//    mantissa bits cleared (exactly what the TF32 datapath reads) and
//    lo = x - hi; the MMA chain accumulates hi*hi + hi*lo + lo*hi, which keeps
//    the update at FP32-level accuracy.
//  3xFP16 (k_gemm_f16x3, the no-pivot LU's block columns with engine
//    FRICO_GEMM_TC_F16): hi = fp16(x),
//    lo = fp16(x - hi). FP16 keeps the same 10 explicit mantissa bits as TF32,
//    so the three products are as accurate, at twice the MMA rate and half the
//    operand bytes. Its 5-bit exponent needs scaling: every operand is stored
//    multiplied by an exact power of two (from the largest |Z| on the diagonal,
//    so that operands sit near 2^8 and keep 2^-25 of that as absolute floor),
//    and the epilogue multiplies the accumulator by the inverse power. An
//    operand beyond the FP16 range becomes infinite; the factorisation then
//    reports a non-finite pivot and the caller falls back to partial pivoting.
//
// Kernel: persistent, warp-specialised, one CTA per SM.
//   warp 0      TMA producer: per 128-byte K slab (32 TF32 or 64 FP16 values),
//               the four 128-row operand tiles (A hi/lo, B hi/lo) into a
//               3-stage shared-memory ring, 128-byte swizzle.
//   warp 1      allocates all 512 TMEM columns (four 128 x 128 FP32 accumulators
//               in rotation, so the MMAs can run up to three tiles ahead of the epilogue)
//               and issues tcgen05.mma (M = 128, N = 128, K = 8 per
//               instruction); tcgen05.commit frees ring stages and publishes
//               finished accumulators.
//   warps 2..9  epilogue: two warps per 32-lane TMEM quadrant, 64 columns
//               each. A warp loads its C values (64 coalesced 128-byte column
//               segments) BEFORE it waits for the accumulator, so the C read
//               overlaps the tile's MMAs; then tcgen05.ld, C -= D, stores.
// All mbarrier waits are bounded; on timeout the CTA records
// FRICO_DEV_ERR_TIMEOUT in the status word and leaves its loops.
// Trailing updates without operand emission and wider than 128 columns run on
// SM pairs instead (k_gemm_pair_*: 256 x 256 tiles per cluster of two CTAs,
// tcgen05.mma.cta_group::2), which halves the operand bytes per multiply-add.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace frico {

namespace tc {

static const int BM = 128, BK = 32;              // tile rows, floats per K slab (128 B)
static const int kEpiWarps = 8;                  // epilogue warps (2 per TMEM lane quadrant)
static const int kThreads = 64 + 32 * kEpiWarps; // producer + MMA + epilogue warps
static const long long kWait = 4000000000LL;
static const bool kPrefetchC = true;             // L2 prefetch of the next tile's C in the epilogue

// Tile configuration by tile width BN. A stage holds A hi, A lo (128 x 32 floats
// each) and B hi, B lo (BN x 32 floats each); the two TMEM accumulators take
// 2 BN columns.
template <int BN> struct Cfg {
    static constexpr int A_TILE = BM * BK * 4;
    static constexpr int B_TILE = BN * BK * 4;
    static constexpr int STAGES = BN == 128 ? 3 : 2;
    static constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
    static constexpr int STAGING = 8 * 32 * 32 * 4;   // per epilogue warp a 32 x 32 float block (A* emission)
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + STAGING + 1024 + 256;
    static constexpr int ACCS = 512 / BN;   // TMEM accumulators in rotation (all 512 columns)
    static constexpr int TMEM_COLS = ACCS * BN;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for the phase with the given parity; false on timeout / abort.
// The status word (global memory, hundreds of cycles away) is polled only every
// 256 failed tries, so that a wait that is about to end is not held up by it.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, DeviceStatus* st) {
    const uint32_t a = smem_u32(bar);
    if (mbar_try(a, parity)) return true;
    const long long t0 = clock64();
    for (uint32_t it = 1;; it++) {
        if (mbar_try(a, parity)) return true;
        if ((it & 15) == 0) {
            if (clock64() - t0 > kWait) {
                atomicCAS(&st->err, 0, FRICO_DEV_ERR_TIMEOUT);
                return false;
            }
            if ((it & 255) == 0 && *(volatile int*)&st->err) return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// tcgen05 shared-memory matrix descriptor: K-major operand, 128-byte swizzle,
// 8-row core-matrix groups 1024 B apart (SBO), start address in 16-byte units.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFF) >> 4);          // bits  0-13 start address
    d |= uint64_t(1) << 16;                          // bits 16-29 leading byte offset (unused with swizzle)
    d |= uint64_t(1024 >> 4) << 32;                  // bits 32-45 stride byte offset
    d |= uint64_t(1) << 46;                          // bits 46-48 fixed 0b001
    d |= uint64_t(2) << 61;                          // bits 61-63 swizzle mode: 128B
    return d;
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major,
// N = 128, M = 128.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// Instruction descriptor, kind::f16: D = F32, A = B = F16, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
    return (1u << 4) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float* v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// One problem of a launch. emit: the finished values of C also go, split into
// hi/lo TF32, to the operand layout of a later update: 1 = as its A* (rows of
// this C, K = this C's columns), 2 = as its B^ (row j = column j of this C).
struct GemmProb {
    float* C;          // real view of the complex C: M x N column-major, ld = ldc floats
    int64_t ldc;
    int M, N;          // real rows (2 x complex rows), columns
    int tiles_m, tiles;
    int nfast;         // 1: consecutive tiles walk N first (A tile reused from L2), else M first
    int accumulate;    // 1: C -= A B; 0: C = A B
    int emit;          // 0, 1 (A*) or 2 (B^), into eh / el with rows of KP operand values
    void* eh;          // float (3xTF32) or __half (3xFP16) operands
    void* el;
    // 3xFP16 only: result = accumulator x oc x (*osp)^op, emitted operand =
    // result x ec x (*esp)^ep, with *osp, *esp device powers of two and op, ep in {-1, 0, 1}
    const float* osp;
    const float* esp;
    float oc, ec;
    int op, ep;
};

// Up to two independent problems in one launch (tiles of problem 0, then 1),
// with the same padded K. KP = padded K in operand values (a multiple of one
// 128-byte slab: 32 TF32 or 64 FP16).
struct GemmArgs {
    GemmProb p[2];
    int nprob, KP;
    DeviceStatus* st;
};

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

// hi = fp16(x), lo = fp16(x - hi) (x - hi is exact in FP32)
__device__ __forceinline__ void split_f16(float x, __half& hi, __half& lo) {
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}

__device__ __forceinline__ float pow_scale(const float* sc, float c, int p) {
    if (p == 0) return c;
    const float s = *sc;
    return c * (p > 0 ? s : 1.f / s);   // powers of two: exact
}

// The kernel body for both operand types (H: 3xFP16, else 3xTF32).
template <int BN, bool H>
__device__ __forceinline__ void gemm_body(const CUtensorMap& tmAh0, const CUtensorMap& tmAl0,
                                          const CUtensorMap& tmBh0, const CUtensorMap& tmBl0,
                                          const CUtensorMap& tmAh1, const CUtensorMap& tmAl1,
                                          const CUtensorMap& tmBh1, const CUtensorMap& tmBl1, const GemmArgs& g) {
    constexpr int STAGES = Cfg<BN>::STAGES, STAGE_BYTES = Cfg<BN>::STAGE_BYTES;
    constexpr int BKE = H ? 2 * BK : BK;   // operand values per 128-byte slab
    constexpr int A_TILE = Cfg<BN>::A_TILE, B_TILE = Cfg<BN>::B_TILE, TMEM_COLS = Cfg<BN>::TMEM_COLS;
    static_assert(BN == 2 * 64, "the epilogue gives each of two warps per quadrant 64 columns");
    extern __shared__ __align__(1024) unsigned char smraw[];
    // 1024-byte aligned ring (128-byte swizzle atoms repeat every 1024 B)
    unsigned char* ring = (unsigned char*)((uintptr_t(smraw) + 1023) & ~uintptr_t(1023));
    uint64_t* bars = (uint64_t*)(ring + STAGES * STAGE_BYTES);
    uint64_t* full = bars;                 // [STAGES]
    uint64_t* empty = bars + STAGES;       // [STAGES]
    constexpr int ACCS = Cfg<BN>::ACCS;
    uint64_t* tfull = bars + 2 * STAGES;          // [ACCS]
    uint64_t* tempty = bars + 2 * STAGES + ACCS;  // [ACCS]
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 2 * ACCS);
    float* staging = (float*)(ring + STAGES * STAGE_BYTES + 256);   // 8 x 32 x 32 floats

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = g.p[0].tiles + (g.nprob > 1 ? g.p[1].tiles : 0);
    const int kslabs = g.KP / BKE;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < ACCS; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], kEpiWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int pi = t >= g.p[0].tiles ? 1 : 0;
                const GemmProb& PP = pi ? g.p[1] : g.p[0];
                const int tt = t - (pi ? g.p[0].tiles : 0), tm = PP.tiles_m, tn = PP.tiles / PP.tiles_m;
                const int mt = PP.nfast ? tt / tn : tt % tm, nt_ = PP.nfast ? tt % tn : tt / tm;
                const CUtensorMap* mAh = pi ? &tmAh1 : &tmAh0;
                const CUtensorMap* mAl = pi ? &tmAl1 : &tmAl0;
                const CUtensorMap* mBh = pi ? &tmBh1 : &tmBh0;
                const CUtensorMap* mBl = pi ? &tmBl1 : &tmBl0;
                for (int ks = 0; ks < kslabs; ks++, it++) {
                    const int s = it % STAGES, round = it / STAGES;
                    if (!(ok = mbar_wait(&empty[s], (round & 1) ^ 1, g.st))) break;
                    unsigned char* base = ring + s * STAGE_BYTES;
                    mbar_expect_tx(&full[s], STAGE_BYTES);
                    tma_load_2d(base, mAh, &full[s], ks * BKE, mt * BM);
                    tma_load_2d(base + A_TILE, mAl, &full[s], ks * BKE, mt * BM);
                    tma_load_2d(base + 2 * A_TILE, mBh, &full[s], ks * BKE, nt_ * BN);
                    tma_load_2d(base + 2 * A_TILE + B_TILE, mBl, &full[s], ks * BKE, nt_ * BN);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = H ? idesc_f16(BM, BN) : idesc_tf32(BM, BN);
            int it = 0, tcount = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, tcount++) {
                const int acc = tcount % ACCS, around = tcount / ACCS;
                if (!(ok = mbar_wait(&tempty[acc], (around & 1) ^ 1, g.st))) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t tmem_d = tmem_base + uint32_t(acc * BN);
                for (int ks = 0; ks < kslabs; ks++, it++) {
                    const int s = it % STAGES, round = it / STAGES;
                    if (!(ok = mbar_wait(&full[s], round & 1, g.st))) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t base = smem_u32(ring + s * STAGE_BYTES);
#pragma unroll
                    for (int kk = 0; kk < 4; kk++) {
                        const uint32_t off = uint32_t(kk * 32);   // 8 TF32 or 16 FP16 = 32 bytes along K
                        const uint64_t ah = smem_desc_sw128(base + off);
                        const uint64_t al = smem_desc_sw128(base + A_TILE + off);
                        const uint64_t bh = smem_desc_sw128(base + 2 * A_TILE + off);
                        const uint64_t bl = smem_desc_sw128(base + 2 * A_TILE + B_TILE + off);
                        const uint32_t first = (ks == 0 && kk == 0) ? 0u : 1u;
                        if constexpr (H) {
                            mma_f16(tmem_d, ah, bh, idesc, first);
                            mma_f16(tmem_d, ah, bl, idesc, 1u);
                            mma_f16(tmem_d, al, bh, idesc, 1u);
                        } else {
                            mma_tf32(tmem_d, ah, bh, idesc, first);
                            mma_tf32(tmem_d, ah, bl, idesc, 1u);
                            mma_tf32(tmem_d, al, bh, idesc, 1u);
                        }
                    }
                    mma_commit(&empty[s]);
                }
                if (!ok) break;
                mma_commit(&tfull[acc]);
            }
        }
    } else {
        // epilogue warps 2..9: TMEM lane quadrant q = warp % 4, columns [64 h, 64 h + 64)
        const int q = warp & 3, h = ((warp - 2) >> 2) * 64;
        const int row = q * 32 + lane;
        int tcount = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, tcount++) {
            const int acc = tcount % ACCS, around = tcount / ACCS;
            const int pi = t >= g.p[0].tiles ? 1 : 0;
            const GemmProb P = pi ? g.p[1] : g.p[0];
            const int tt = t - (pi ? g.p[0].tiles : 0), tn = P.tiles / P.tiles_m;
            const int mt = P.nfast ? tt / tn : tt % P.tiles_m, nt_ = P.nfast ? tt % tn : tt / P.tiles_m;
            const int gr = mt * BM + row;
            const int ncol = min(64, P.N - nt_ * BN - h);   // columns of this warp's half (may be <= 0)
            const bool rowok = gr < P.M;
            const int64_t ldc = P.ldc;
            const int accumulate = P.accumulate, emit = P.emit;
            float osc = 1.f, esc = 1.f;
            if constexpr (H) {
                osc = pow_scale(P.osp, P.oc, P.op);
                esc = pow_scale(P.esp, P.ec, P.ep);
            }
            float* cp = P.C + int64_t(nt_ * BN + h) * ldc + gr;
            // the C lines of this warp's part of the CTA's next tile into L2 (each lane two of the
            // 64 128-byte column segments), so that its loads there wait on L2 instead of DRAM
            if (kPrefetchC) {
                const int tq = t + int(gridDim.x);
                if (tq < ntiles) {
                    const int pq = tq >= g.p[0].tiles ? 1 : 0;
                    const GemmProb& Q = pq ? g.p[1] : g.p[0];
                    const int uq = tq - (pq ? g.p[0].tiles : 0), tnq = Q.tiles / Q.tiles_m;
                    const int mq = Q.nfast ? uq / tnq : uq % Q.tiles_m, nq = Q.nfast ? uq % tnq : uq / Q.tiles_m;
                    const int r0 = mq * BM + q * 32;
                    if (Q.accumulate && r0 < Q.M) {
#pragma unroll
                        for (int k = 0; k < 2; k++) {
                            const int j = lane + 32 * k;
                            if (nq * BN + h + j < Q.N)
                                asm volatile("prefetch.global.L2 [%0];" ::"l"(Q.C + int64_t(nq * BN + h + j) * Q.ldc + r0));
                        }
                    }
                }
            }
            // C values first: these reads do not depend on the accumulator
            float cv[64];
            if (accumulate && rowok && ncol == 64) {
#pragma unroll
                for (int j = 0; j < 64; j++) cv[j] = cp[int64_t(j) * ldc];
            } else {
#pragma unroll
                for (int j = 0; j < 64; j++) cv[j] = (accumulate && rowok && j < ncol) ? cp[int64_t(j) * ldc] : 0.f;
            }
            if (!mbar_wait(&tfull[acc], around & 1, g.st)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t taddr = tmem_base + (uint32_t(q * 32) << 16) + uint32_t(acc * BN + h);
            // an opaque copy of the base: the store addresses are recomputed here
            // instead of 64 load addresses being held across the wait
            float* sp;
            asm volatile("mov.b64 %0, %1;" : "=l"(sp) : "l"(cp));
#pragma unroll
            for (int c0 = 0; c0 < 64; c0 += 32) {
                float v[32];
                tmem_ld32(taddr + uint32_t(c0), v);
                float* wp = sp + int64_t(c0) * ldc;
                float* stg = staging + (warp - 2) * 1024;   // [row (lane)][column ^ row], 32 x 32
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const float d = H ? v[j] * osc : v[j];
                    const float o = accumulate ? cv[c0 + j] - d : d;
                    const bool ok = rowok && c0 + j < ncol;
                    if (ok) wp[int64_t(j) * ldc] = o;
                    if (emit == 1) {
                        stg[lane * 32 + (j ^ lane)] = o;
                    } else if (emit == 2 && ok) {
                        const int64_t off = int64_t(nt_ * BN + h + c0 + j) * g.KP + gr;
                        if constexpr (H) {
                            split_f16(o * esc, ((__half*)P.eh)[off], ((__half*)P.el)[off]);
                        } else {
                            const float hi = tf32_hi(o);
                            ((float*)P.eh)[off] = hi;
                            ((float*)P.el)[off] = o - hi;
                        }
                    }
                }
                if (emit == 1) {
                    // A* row R: (re, -im) (R = 2 r) or (im, re) (R = 2 r + 1) at K = 2 col, 2 col + 1.
                    // Read back transposed, lane = column: each store covers 256 contiguous bytes of a row.
                    __syncwarp();
                    const int col = nt_ * BN + h + c0 + lane;
                    const bool colok = c0 + lane < ncol;
                    for (int i = 0; i < 32; i++) {
                        const int R = mt * BM + q * 32 + i;
                        const float a = stg[i * 32 + (lane ^ i)], b = stg[(i ^ 1) * 32 + (lane ^ (i ^ 1))];
                        if (colok && R < P.M) {
                            const float2 w = (i & 1) ? make_float2(a, b) : make_float2(a, -b);
                            const int64_t off = int64_t(R) * g.KP + 2 * col;
                            if constexpr (H) {
                                __half2 wh, wl;
                                split_f16(w.x * esc, wh.x, wl.x);
                                split_f16(w.y * esc, wh.y, wl.y);
                                ((__half2*)P.eh)[off >> 1] = wh;
                                ((__half2*)P.el)[off >> 1] = wl;
                            } else {
                                const float2 wh = make_float2(tf32_hi(w.x), tf32_hi(w.y));
                                *reinterpret_cast<float2*>((float*)P.eh + off) = wh;
                                *reinterpret_cast<float2*>((float*)P.el + off) = make_float2(w.x - wh.x, w.y - wh.y);
                            }
                        }
                    }
                    __syncwarp();
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[acc]);
        }
    }
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS));
    }
}

template <int BN>
__global__ void __launch_bounds__(kThreads, 1) k_gemm_tf32x3(
    const __grid_constant__ CUtensorMap tmAh0, const __grid_constant__ CUtensorMap tmAl0,
    const __grid_constant__ CUtensorMap tmBh0, const __grid_constant__ CUtensorMap tmBl0,
    const __grid_constant__ CUtensorMap tmAh1, const __grid_constant__ CUtensorMap tmAl1,
    const __grid_constant__ CUtensorMap tmBh1, const __grid_constant__ CUtensorMap tmBl1,
    const __grid_constant__ GemmArgs g) {
    gemm_body<BN, false>(tmAh0, tmAl0, tmBh0, tmBl0, tmAh1, tmAl1, tmBh1, tmBl1, g);
}

template <int BN>
__global__ void __launch_bounds__(kThreads, 1) k_gemm_f16x3(
    const __grid_constant__ CUtensorMap tmAh0, const __grid_constant__ CUtensorMap tmAl0,
    const __grid_constant__ CUtensorMap tmBh0, const __grid_constant__ CUtensorMap tmBl0,
    const __grid_constant__ CUtensorMap tmAh1, const __grid_constant__ CUtensorMap tmAl1,
    const __grid_constant__ CUtensorMap tmBh1, const __grid_constant__ CUtensorMap tmBl1,
    const __grid_constant__ GemmArgs g) {
    gemm_body<BN, true>(tmAh0, tmAl0, tmBh0, tmBl0, tmAh1, tmAl1, tmBh1, tmBl1, g);
}

// ---- the trailing update on SM pairs (cta_group::2).
// The one-CTA kernel above is bound by the TMA operand feed from L2: per 128 x 128
// tile and 32-float K slab it loads 64 KB of operands for 128 x 128 x 32 x 3 MMA
// multiply-adds. Here the two CTAs of a cluster share one 256 x 256 tile: each loads
// its own 128 rows of A* and 128 rows of B^ (the same 64 KB per slab), and the even
// CTA's MMA warp issues M = 256, N = 256 tcgen05.mma (cta_group::2) over both CTAs'
// shared memory, so every CTA's slab feeds twice the multiply-adds. Each CTA's TMEM
// holds its own 128 rows x 256 columns (two accumulators in rotation); its eight
// epilogue warps update its half of the tile as above (no operand emission here).
// Hand-offs: both CTAs' TMA loads complete on the even CTA's full barrier (which
// expects both CTAs' bytes); its commits arrive on both CTAs' empty and tfull
// barriers (multicast); every epilogue warp of both CTAs arrives on the even CTA's
// tempty barrier. All waits are bounded as above.
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// The shared::cluster address of the same shared-memory object in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t mapa_rank(const void* p, uint32_t rank) {
    uint32_t a;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_u32(p)), "r"(rank));
    return a;
}

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void tma_load_2d_pair(void* dst, const CUtensorMap* map, uint32_t bar_cluster, int x,
                                                 int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
        "%4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(bar_cluster), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void mma_pair_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_pair_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

// arrive on the barrier at the same offset in both CTAs of the pair when the MMAs issued so far are done
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
            smem_u32(bar)),
        "h"((unsigned short)3)
        : "memory");
}

__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster) : "memory");
}

static const int kPairAccs = 2;   // 256-column accumulators in rotation (all 512 TMEM columns)
static const bool kPairPrefetchC = true;
static const int kPairGroup = 8;   // > 0: tiles walk M within groups of this many tile columns (measured best of 0, 4, 8, 16)

// Tile t of the pair grid (tm2 x tn2 tiles of 256 x 256): M first, or M first within
// groups of kPairGroup tile columns.
__device__ __forceinline__ void pair_tile(int t, int tm2, int tn2, int& mt, int& nt) {
    if (kPairGroup > 0) {
        const int per = tm2 * kPairGroup, gi = t / per, r = t - gi * per;
        const int gw = min(kPairGroup, tn2 - gi * kPairGroup);
        mt = r / gw;
        nt = gi * kPairGroup + r % gw;
    } else {
        mt = t % tm2;
        nt = t / tm2;
    }
}

template <bool H>
__device__ __forceinline__ void gemm_pair_body(const CUtensorMap& tmAh, const CUtensorMap& tmAl,
                                               const CUtensorMap& tmBh, const CUtensorMap& tmBl, const GemmArgs& g) {
    constexpr int STAGES = Cfg<128>::STAGES, STAGE_BYTES = Cfg<128>::STAGE_BYTES;
    constexpr int A_TILE = Cfg<128>::A_TILE, B_TILE = Cfg<128>::B_TILE;
    constexpr int BKE = H ? 2 * BK : BK;
    constexpr int PM = 2 * BM, PN = 256;   // the pair's tile
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char* ring = (unsigned char*)((uintptr_t(smraw) + 1023) & ~uintptr_t(1023));
    uint64_t* bars = (uint64_t*)(ring + STAGES * STAGE_BYTES);
    uint64_t* full = bars;                        // [STAGES], used in the even CTA
    uint64_t* empty = bars + STAGES;              // [STAGES]
    uint64_t* tfull = bars + 2 * STAGES;          // [kPairAccs]
    uint64_t* tempty = tfull + kPairAccs;         // [kPairAccs], used in the even CTA
    uint32_t* tmem_slot = (uint32_t*)(tempty + kPairAccs);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_rank();
    const GemmProb& P = g.p[0];
    const int tm2 = (P.M + PM - 1) / PM, tn2 = (P.N + PN - 1) / PN, ntp = tm2 * tn2;
    const int cid = int(blockIdx.x >> 1), ncl = int(gridDim.x >> 1);
    const int kslabs = g.KP / BKE;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < kPairAccs; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], 2 * kEpiWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {   // one warp of each CTA of the pair, collectively
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    cluster_sync_all();   // both CTAs' barriers initialised before any remote arrival
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            for (int t = cid; t < ntp && ok; t += ncl) {
                int mt, nt_;
                pair_tile(t, tm2, tn2, mt, nt_);
                for (int ks = 0; ks < kslabs; ks++, it++) {
                    const int s = it % STAGES, round = it / STAGES;
                    if (!(ok = mbar_wait(&empty[s], (round & 1) ^ 1, g.st))) break;
                    unsigned char* base = ring + s * STAGE_BYTES;
                    if (rank == 0) mbar_expect_tx(&full[s], 2 * STAGE_BYTES);
                    const uint32_t fb = mapa_rank(&full[s], 0);
                    const int ya = mt * PM + int(rank) * BM, yb = nt_ * PN + int(rank) * 128;
                    tma_load_2d_pair(base, &tmAh, fb, ks * BKE, ya);
                    tma_load_2d_pair(base + A_TILE, &tmAl, fb, ks * BKE, ya);
                    tma_load_2d_pair(base + 2 * A_TILE, &tmBh, fb, ks * BKE, yb);
                    tma_load_2d_pair(base + 2 * A_TILE + B_TILE, &tmBl, fb, ks * BKE, yb);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {
            const uint32_t idesc = H ? idesc_f16(PM, PN) : idesc_tf32(PM, PN);
            int it = 0, tcount = 0;
            bool ok = true;
            for (int t = cid; t < ntp && ok; t += ncl, tcount++) {
                const int acc = tcount % kPairAccs, around = tcount / kPairAccs;
                if (!(ok = mbar_wait(&tempty[acc], (around & 1) ^ 1, g.st))) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t tmem_d = tmem_base + uint32_t(acc * PN);
                for (int ks = 0; ks < kslabs; ks++, it++) {
                    const int s = it % STAGES, round = it / STAGES;
                    if (!(ok = mbar_wait(&full[s], round & 1, g.st))) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t base = smem_u32(ring + s * STAGE_BYTES);
#pragma unroll
                    for (int kk = 0; kk < 4; kk++) {
                        const uint32_t off = uint32_t(kk * 32);
                        const uint64_t ah = smem_desc_sw128(base + off);
                        const uint64_t al = smem_desc_sw128(base + A_TILE + off);
                        const uint64_t bh = smem_desc_sw128(base + 2 * A_TILE + off);
                        const uint64_t bl = smem_desc_sw128(base + 2 * A_TILE + B_TILE + off);
                        const uint32_t first = (ks == 0 && kk == 0) ? 0u : 1u;
                        if constexpr (H) {
                            mma_pair_f16(tmem_d, ah, bh, idesc, first);
                            mma_pair_f16(tmem_d, ah, bl, idesc, 1u);
                            mma_pair_f16(tmem_d, al, bh, idesc, 1u);
                        } else {
                            mma_pair_tf32(tmem_d, ah, bh, idesc, first);
                            mma_pair_tf32(tmem_d, ah, bl, idesc, 1u);
                            mma_pair_tf32(tmem_d, al, bh, idesc, 1u);
                        }
                    }
                    mma_commit_pair(&empty[s]);
                }
                if (!ok) break;
                mma_commit_pair(&tfull[acc]);
            }
        }
    } else {
        // epilogue warps 2..9: TMEM lane quadrant q, columns [128 h2, 128 h2 + 128) in two halves
        const int q = warp & 3, h2 = ((warp - 2) >> 2) * 128;
        const int row = q * 32 + lane;
        const int64_t ldc = P.ldc;
        const int accumulate = P.accumulate;
        float osc = 1.f;
        if constexpr (H) osc = pow_scale(P.osp, P.oc, P.op);
        int tcount = 0;
        for (int t = cid; t < ntp; t += ncl, tcount++) {
            const int acc = tcount % kPairAccs, around = tcount / kPairAccs;
            int mt, nt_;
            pair_tile(t, tm2, tn2, mt, nt_);
            const int gr = mt * PM + int(rank) * BM + row;
            const bool rowok = gr < P.M;
            if (kPairPrefetchC && accumulate) {   // the next tile's C lines of this warp into L2
                const int tq = t + ncl;
                if (tq < ntp) {
                    int mq, nq;
                    pair_tile(tq, tm2, tn2, mq, nq);
                    const int r0 = mq * PM + int(rank) * BM + q * 32;
                    if (r0 < P.M) {
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const int col = nq * PN + h2 + lane + 32 * k;
                            if (col < P.N) asm volatile("prefetch.global.L2 [%0];" ::"l"(P.C + int64_t(col) * ldc + r0));
                        }
                    }
                }
            }
            bool ready = true;
#pragma unroll 1
            for (int hh = 0; hh < 128; hh += 64) {
                const int c0 = nt_ * PN + h2 + hh;
                const int ncol = min(64, P.N - c0);
                float* cp = P.C + int64_t(c0) * ldc + gr;
                float cv[64];
                if (accumulate && rowok && ncol == 64) {
#pragma unroll
                    for (int j = 0; j < 64; j++) cv[j] = cp[int64_t(j) * ldc];
                } else {
#pragma unroll
                    for (int j = 0; j < 64; j++) cv[j] = (accumulate && rowok && j < ncol) ? cp[int64_t(j) * ldc] : 0.f;
                }
                if (hh == 0) {
                    if (!(ready = mbar_wait(&tfull[acc], around & 1, g.st))) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                }
                const uint32_t taddr = tmem_base + (uint32_t(q * 32) << 16) + uint32_t(acc * PN + h2 + hh);
                float* sp;
                asm volatile("mov.b64 %0, %1;" : "=l"(sp) : "l"(cp));
#pragma unroll
                for (int c1 = 0; c1 < 64; c1 += 32) {
                    float v[32];
                    tmem_ld32(taddr + uint32_t(c1), v);
                    float* wp = sp + int64_t(c1) * ldc;
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        const float d = H ? v[j] * osc : v[j];
                        if (rowok && c1 + j < ncol) wp[int64_t(j) * ldc] = accumulate ? cv[c1 + j] - d : d;
                    }
                }
            }
            if (!ready) break;
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive_cluster(mapa_rank(&tempty[acc], 0));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    cluster_sync_all();   // no CTA leaves while its peer may still signal its barriers or read its TMEM
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(512));
    }
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kThreads, 1)
    k_gemm_pair_tf32x3(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                       const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
                       const __grid_constant__ GemmArgs g) {
    gemm_pair_body<false>(tmAh, tmAl, tmBh, tmBl, g);
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kThreads, 1)
    k_gemm_pair_f16x3(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                      const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
                      const __grid_constant__ GemmArgs g) {
    gemm_pair_body<true>(tmAh, tmAl, tmBh, tmBl, g);
}

// ---- products whose sums must stay beyond FP32 accuracy (the far field, fields_gemm.cu).
// The tensor cores accumulate in FP32 with a rounding of the running sum at every MMA,
// which over the hundreds of MMAs of a long K loses several digits (about 1e-6 relative
// measured over K = 256 reals). Here the MMA warp starts a fresh TMEM accumulator every
// `group` k-steps (K = 8 per step; two accumulators of 128 columns in rotation), and the
// epilogue warps add each finished group into double-float sums (hi + lo, two-sum on the
// FP32 pipe) that live in the other half of TMEM (columns 256-383: hi, 384-511: lo), so
// registers hold only the 8 columns in flight. A tile's sums go to an FP64 array C
// (overwritten, or added to with accumulate = 1, for K split over launches). Two problems
// per launch as above.
struct DfProb {
    float2* C;        // M x N real double-float values (hi, lo), column-major, ld = ldc
    int64_t ldc;
    int M, N, tiles_m, tiles;
};
struct DfArgs {
    DfProb p[2];
    int nprob, KP, group, accumulate;
    DeviceStatus* st;
};
static const int kDfAccs = 2;   // group accumulators in rotation (TMEM columns 0-255)

__global__ void __launch_bounds__(kThreads, 1) k_gemm_dfacc(
    const __grid_constant__ CUtensorMap tmAh0, const __grid_constant__ CUtensorMap tmAl0,
    const __grid_constant__ CUtensorMap tmBh0, const __grid_constant__ CUtensorMap tmBl0,
    const __grid_constant__ CUtensorMap tmAh1, const __grid_constant__ CUtensorMap tmAl1,
    const __grid_constant__ CUtensorMap tmBh1, const __grid_constant__ CUtensorMap tmBl1,
    const __grid_constant__ DfArgs g) {
    constexpr int BN = 128, STAGES = Cfg<128>::STAGES, STAGE_BYTES = Cfg<128>::STAGE_BYTES;
    constexpr int A_TILE = Cfg<128>::A_TILE, B_TILE = Cfg<128>::B_TILE, TMEM_COLS = 512;
    constexpr uint32_t kHi = 2 * BN, kLo = 3 * BN;   // TMEM columns of the double-float sums
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char* ring = (unsigned char*)((uintptr_t(smraw) + 1023) & ~uintptr_t(1023));
    uint64_t* bars = (uint64_t*)(ring + STAGES * STAGE_BYTES);
    uint64_t* full = bars;                      // [STAGES]
    uint64_t* empty = bars + STAGES;            // [STAGES]
    uint64_t* tfull = bars + 2 * STAGES;        // [kDfAccs]
    uint64_t* tempty = tfull + kDfAccs;         // [kDfAccs]
    uint32_t* tmem_slot = (uint32_t*)(tempty + kDfAccs);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = g.p[0].tiles + (g.nprob > 1 ? g.p[1].tiles : 0);
    const int kslabs = g.KP / BK;
    const int grp = g.group, ngrp = 4 / grp;   // k-steps per accumulator, accumulators per slab
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < kDfAccs; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], kEpiWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem_base = *tmem_slot;
    // tile t -> problem, M tile, N tile (N first: the CTAs on one A tile run together)
    auto tile_of = [&](int t, int& pi, int& mt, int& nt_) {
        pi = t >= g.p[0].tiles ? 1 : 0;
        const DfProb& P = pi ? g.p[1] : g.p[0];
        const int tt = t - (pi ? g.p[0].tiles : 0), tn = P.tiles / P.tiles_m;
        mt = tt / tn;
        nt_ = tt % tn;
    };
    if (warp == 0) {
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                int pi, mt, nt_;
                tile_of(t, pi, mt, nt_);
                const CUtensorMap* mAh = pi ? &tmAh1 : &tmAh0;
                const CUtensorMap* mAl = pi ? &tmAl1 : &tmAl0;
                const CUtensorMap* mBh = pi ? &tmBh1 : &tmBh0;
                const CUtensorMap* mBl = pi ? &tmBl1 : &tmBl0;
                for (int ks = 0; ks < kslabs; ks++, it++) {
                    const int s = it % STAGES, round = it / STAGES;
                    if (!(ok = mbar_wait(&empty[s], (round & 1) ^ 1, g.st))) break;
                    unsigned char* base = ring + s * STAGE_BYTES;
                    mbar_expect_tx(&full[s], STAGE_BYTES);
                    tma_load_2d(base, mAh, &full[s], ks * BK, mt * BM);
                    tma_load_2d(base + A_TILE, mAl, &full[s], ks * BK, mt * BM);
                    tma_load_2d(base + 2 * A_TILE, mBh, &full[s], ks * BK, nt_ * BN);
                    tma_load_2d(base + 2 * A_TILE + B_TILE, mBl, &full[s], ks * BK, nt_ * BN);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_tf32(BM, BN);
            int it = 0, v = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                for (int ks = 0; ks < kslabs && ok; ks++, it++) {
                    const int s = it % STAGES, round = it / STAGES;
                    if (!(ok = mbar_wait(&full[s], round & 1, g.st))) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t base = smem_u32(ring + s * STAGE_BYTES);
                    for (int gi = 0; gi < ngrp; gi++, v++) {
                        const int acc = v % kDfAccs, around = v / kDfAccs;
                        if (!(ok = mbar_wait(&tempty[acc], (around & 1) ^ 1, g.st))) break;
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t tmem_d = tmem_base + uint32_t(acc * BN);
                        for (int kk = gi * grp; kk < (gi + 1) * grp; kk++) {
                            const uint32_t off = uint32_t(kk * 32);   // 8 TF32 values along K
                            const uint64_t ah = smem_desc_sw128(base + off);
                            const uint64_t al = smem_desc_sw128(base + A_TILE + off);
                            const uint64_t bh = smem_desc_sw128(base + 2 * A_TILE + off);
                            const uint64_t bl = smem_desc_sw128(base + 2 * A_TILE + B_TILE + off);
                            mma_tf32(tmem_d, ah, bh, idesc, kk == gi * grp ? 0u : 1u);
                            mma_tf32(tmem_d, ah, bl, idesc, 1u);
                            mma_tf32(tmem_d, al, bh, idesc, 1u);
                        }
                        mma_commit(&tfull[acc]);
                    }
                    if (!ok) break;
                    mma_commit(&empty[s]);
                }
            }
        }
    } else {
        // epilogue warps 2..9: TMEM lane quadrant q = warp % 4, columns [h, h + 64), 8 at a time
        const int q = warp & 3, h = ((warp - 2) >> 2) * 64;
        const int row = q * 32 + lane;
        const uint32_t lanes = uint32_t(q * 32) << 16;
        int v = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            int pi, mt, nt_;
            tile_of(t, pi, mt, nt_);
            const DfProb P = pi ? g.p[1] : g.p[0];
            for (int ks = 0; ks < kslabs && ok; ks++) {
                for (int gi = 0; gi < ngrp; gi++, v++) {
                    const int acc = v % kDfAccs, around = v / kDfAccs;
                    if (!(ok = mbar_wait(&tfull[acc], around & 1, g.st))) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const bool first = ks == 0 && gi == 0;
#pragma unroll 1
                    for (int c0 = 0; c0 < 64; c0 += 8) {
                        const uint32_t col = uint32_t(h + c0);
                        float x[8], hi[8], lo[8];
                        tmem_ld8(tmem_base + lanes + uint32_t(acc * BN) + col, x);
                        if (first) {
#pragma unroll
                            for (int j = 0; j < 8; j++) {
                                hi[j] = x[j];
                                lo[j] = 0.f;
                            }
                        } else {
                            tmem_ld8(tmem_base + lanes + kHi + col, hi);
                            tmem_ld8(tmem_base + lanes + kLo + col, lo);
#pragma unroll
                            for (int j = 0; j < 8; j++) {   // (hi, lo) += x, two-sum
                                const float a = hi[j], b = x[j];
                                const float sm = __fadd_rn(a, b);
                                const float bv = __fsub_rn(sm, a);
                                const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(sm, bv)), __fsub_rn(b, bv));
                                hi[j] = sm;
                                lo[j] = __fadd_rn(lo[j], e);
                            }
                        }
                        tmem_st8(tmem_base + lanes + kHi + col, hi);
                        tmem_st8(tmem_base + lanes + kLo + col, lo);
                    }
                    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[acc]);
                }
            }
            if (!ok) break;
            const int gr = mt * BM + row;
            const int ncol = min(64, P.N - nt_ * BN - h);
            float2* cp = P.C + int64_t(nt_ * BN + h) * P.ldc + gr;
#pragma unroll 1
            for (int c0 = 0; c0 < 64; c0 += 8) {
                float hi[8], lo[8];
                tmem_ld8(tmem_base + lanes + kHi + uint32_t(h + c0), hi);
                tmem_ld8(tmem_base + lanes + kLo + uint32_t(h + c0), lo);
                if (gr < P.M)
#pragma unroll
                    for (int j = 0; j < 8; j++)
                        if (c0 + j < ncol) {
                            // double-float on the FP32 pipe (the FP64 pipe is narrow on this part)
                            float2* o = cp + int64_t(c0 + j) * P.ldc;
                            float h2 = hi[j], l2 = lo[j];
                            if (g.accumulate) {
                                const float2 c = *o;
                                const float sm = __fadd_rn(c.x, h2);
                                const float bv = __fsub_rn(sm, c.x);
                                const float e = __fadd_rn(__fsub_rn(c.x, __fsub_rn(sm, bv)), __fsub_rn(h2, bv));
                                h2 = sm;
                                l2 = __fadd_rn(__fadd_rn(c.y, l2), e);
                            }
                            const float r = __fadd_rn(h2, l2);   // renormalise: |lo| <= ulp(hi) / 2
                            *o = make_float2(r, __fsub_rn(l2, __fsub_rn(r, h2)));
                        }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS));
    }
}

static constexpr int kDfSmemBytes = Cfg<128>::STAGES * Cfg<128>::STAGE_BYTES + 1024 + 256;

// Store x as a hi/lo operand pair at element o: TF32 (float arrays) or, with a
// scale, FP16 (__half arrays).
__device__ __forceinline__ void put_split(void* hp, void* lp, int64_t o, float x, bool h, float scale) {
    if (h) {
        split_f16(x * scale, ((__half*)hp)[o], ((__half*)lp)[o]);
    } else {
        const float hi = tf32_hi(x);
        ((float*)hp)[o] = hi;
        ((float*)lp)[o] = x - hi;
    }
}

// A* hi/lo from the complex panel L (m x k, column-major, lda): rows 2r, 2r+1,
// KP values each (zero beyond 2k). A CTA handles 32 complex rows.
__device__ __forceinline__ void split_a_tile(int bx, int by, const float2* __restrict__ L, int64_t lda, int m, int k,
                                             int KP, void* Ah, void* Al, bool h, float scale, float2 (*t)[65]) {
    const int r0 = bx * 32;
    // by takes one 64-column chunk of K (more CTAs in flight for this store-bound copy)
    for (int q0 = by * 64; q0 < min(KP / 2, (by + 1) * 64); q0 += 64) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < 32 * 64; idx += blockDim.x) {
            int rr = idx & 31, qq = idx >> 5;
            int r = r0 + rr, q = q0 + qq;
            t[rr][qq] = (r < m && q < k) ? L[int64_t(q) * lda + r] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        // 64 real rows x 128 floats of this chunk
        for (int idx = threadIdx.x; idx < 64 * 128; idx += blockDim.x) {
            int col = idx & 127, rrow = idx >> 7;   // rrow = 2*rr + s
            int rr = rrow >> 1, s = rrow & 1, qq = col >> 1, part = col & 1;
            int r = r0 + rr;
            if (r >= m || q0 + qq >= KP / 2) continue;
            float2 a = t[rr][qq];
            float x = s == 0 ? (part == 0 ? a.x : -a.y) : (part == 0 ? a.y : a.x);
            put_split(Ah, Al, int64_t(2 * r + s) * KP + 2 * q0 + col, x, h, scale);
        }
    }
}

// B^ hi/lo from the complex block U (k x n, column-major, lda): row j = the
// 2k floats of column j, zero-padded to KP.
__device__ __forceinline__ void split_b_elem(int64_t idx, const float2* __restrict__ U, int64_t lda, int k, int n,
                                             int KP, void* Bh, void* Bl, bool h, float scale) {
    if (idx >= int64_t(n) * KP) return;
    int j = int(idx / KP), c = int(idx % KP);
    float x = 0.f;
    if (c < 2 * k) {
        const float* col = (const float*)(U + int64_t(j) * lda);
        x = col[c];
    }
    put_split(Bh, Bl, idx, x, h, scale);
}

// Operand splits of one or two updates in a single launch: up to four parts,
// each an A* (32-row bands x 64-column chunks of K, a_cols chunks per band) or
// a B^ (256 floats per block) split; blocks are numbered part after part.
struct SplitPart {
    const float2* src;
    int64_t ld;
    int rows, k;       // A*: complex rows m; B^: columns n. k: complex K
    void* hi;
    void* lo;
    int isB, a_cols, blocks;
    int h;             // 1: FP16 operands, value x c x s^p (s = *sc); 0: TF32
    const float* sc;
    float c;
    int p;
};
struct SplitArgs {
    SplitPart p[4];
    int np, KP;
};

__global__ void __launch_bounds__(256) k_split_parts(SplitArgs a) {
    __shared__ float2 t[32][65];
    int b = blockIdx.x, i = 0;
    while (i + 1 < a.np && b >= (i == 0 ? a.p[0].blocks : i == 1 ? a.p[1].blocks : a.p[2].blocks)) {
        b -= i == 0 ? a.p[0].blocks : i == 1 ? a.p[1].blocks : a.p[2].blocks;
        i++;
    }
    const SplitPart P = i == 0 ? a.p[0] : i == 1 ? a.p[1] : i == 2 ? a.p[2] : a.p[3];
    const float scale = P.h ? pow_scale(P.sc, P.c, P.p) : 1.f;
    if (P.isB)
        split_b_elem(int64_t(b) * blockDim.x + threadIdx.x, P.src, P.ld, P.k, P.rows, a.KP, P.hi, P.lo, P.h != 0,
                     scale);
    else
        split_a_tile(b / P.a_cols, b % P.a_cols, P.src, P.ld, P.rows, P.k, a.KP, P.hi, P.lo, P.h != 0, scale, t);
}

}  // namespace tc

// ------------------------------------------------------------------ host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static const EncodeTiledFn fn = [] {   // thread-safe one-time lookup
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (EncodeTiledFn)p;
        cudaGetLastError();
        return (EncodeTiledFn) nullptr;
    }();
    return fn;
}

// rows x KP operand values (FP32, or FP16 with h), row-major (K-major), box
// box_rows x 128 bytes, 128B swizzle.
static bool make_map(CUtensorMap* m, const void* base, int rows, int KP, int box_rows, bool h = false) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const uint32_t esz = h ? 2 : 4;
    cuuint64_t dims[2] = {cuuint64_t(KP), cuuint64_t(rows)};
    cuuint64_t strides[1] = {cuuint64_t(KP) * esz};
    cuuint32_t box[2] = {128 / esz, uint32_t(box_rows)};
    cuuint32_t es[2] = {1, 1};
    return fn(m, h ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base),
              dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool gemm_tc_available(frico_gpu_ctx* ctx) {
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, ctx->device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, ctx->device);
    return major == 10 && minor == 3 && encode_fn() != nullptr;
}

// Operand scaling of a 3xFP16 operand or result: c x s^p, s the power of two at sc.
struct Pow2Scale {
    const float* sc;
    float c;
    int p;
};

static tc::SplitPart split_part(bool isB, const float2* src, int64_t ld, int rows, int k, void* hi, void* lo,
                                int KP, const Pow2Scale* h = nullptr) {
    tc::SplitPart p;
    p.h = h ? 1 : 0;
    p.sc = h ? h->sc : nullptr;
    p.c = h ? h->c : 1.f;
    p.p = h ? h->p : 0;
    p.src = src;
    p.ld = ld;
    p.rows = rows;
    p.k = k;
    p.hi = hi;
    p.lo = lo;
    p.isB = isB ? 1 : 0;
    p.a_cols = (KP / 2 + 63) / 64;
    p.blocks = isB ? int((int64_t(rows) * KP + 255) / 256) : ((rows + 31) / 32) * p.a_cols;
    return p;
}

static int launch_split(frico_gpu_ctx* ctx, cudaStream_t st, const tc::SplitPart* parts, int np, int KP) {
    tc::SplitArgs a;
    int blocks = 0;
    for (int i = 0; i < 4; i++) {
        a.p[i] = parts[i < np ? i : np - 1];
        if (i < np) blocks += parts[i].blocks;
    }
    a.np = np;
    a.KP = KP;
    if (blocks == 0) return FRICO_GPU_OK;
    tc::k_split_parts<<<unsigned(blocks), 256, 0, st>>>(a);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_split_parts");
}

// One problem of a launch: its four tensor maps (A* hi/lo with a_rows rows, B^
// hi/lo with b_rows rows, KP floats each) and its C.
struct TcProblem {
    CUtensorMap mah, mal, mbh, mbl;
    tc::GemmProb p;
    bool h;   // 3xFP16 operands
};

// res / emi (3xFP16 only, both or neither): the result's and the emitted operand's scales.
static int make_problem(frico_gpu_ctx* ctx, TcProblem& q, float2* C, int64_t ldc, int M, int N, const void* Ah,
                        const void* Al, const void* Bh, const void* Bl, int KP, int accumulate, int emit,
                        void* eh, void* el, const Pow2Scale* res = nullptr, const Pow2Scale* emi = nullptr) {
    const bool h = res != nullptr;
    if (!make_map(&q.mah, Ah, M, KP, tc::BM, h) || !make_map(&q.mal, Al, M, KP, tc::BM, h) ||
        !make_map(&q.mbh, Bh, N, KP, 128, h) || !make_map(&q.mbl, Bl, N, KP, 128, h))
        return set_err(ctx, FRICO_GPU_ECUDA, "cuTensorMapEncodeTiled failed");
    q.h = h;
    q.p.osp = h ? res->sc : nullptr;
    q.p.oc = h ? res->c : 1.f;
    q.p.op = h ? res->p : 0;
    q.p.esp = emi ? emi->sc : nullptr;
    q.p.ec = emi ? emi->c : 1.f;
    q.p.ep = emi ? emi->p : 0;
    q.p.C = (float*)C;
    q.p.ldc = 2 * ldc;
    q.p.M = M;
    q.p.N = N;
    q.p.tiles_m = (M + tc::BM - 1) / tc::BM;
    q.p.tiles = q.p.tiles_m * ((N + 127) / 128);
    q.p.nfast = 0;
    q.p.accumulate = accumulate;
    q.p.emit = emit;
    q.p.eh = eh;
    q.p.el = el;
    return FRICO_GPU_OK;
}

// Trailing updates without operand emission and more than 128 columns run on SM pairs
// (k_gemm_pair_*); the most clusters of two that the device keeps resident at once.
static const bool kPairGemm = true;
static std::atomic<int> g_pair_clusters[64];

static int launch_gemm_pair(frico_gpu_ctx* ctx, cudaStream_t st, const TcProblem& q, int KP, int cap,
                            cudaEvent_t* ev) {
    int rc;
    if ((rc = device_once(ctx, kOnceGemmPair, [](frico_gpu_ctx* c) {
             const void* fns[2] = {(const void*)tc::k_gemm_pair_tf32x3, (const void*)tc::k_gemm_pair_f16x3};
             int most = 1 << 30;
             for (const void* f : fns) {
                 int r = cuda_check(c, cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                            tc::Cfg<128>::SMEM_BYTES), "pair smem attribute");
                 if (r) return r;
                 cudaLaunchConfig_t cfg = {};
                 cfg.gridDim = dim3(2, 1, 1);
                 cfg.blockDim = dim3(tc::kThreads, 1, 1);
                 cfg.dynamicSmemBytes = tc::Cfg<128>::SMEM_BYTES;
                 int nc = 0;
                 if ((r = cuda_check(c, cudaOccupancyMaxActiveClusters(&nc, f, &cfg), "pair occupancy"))) return r;
                 most = std::min(most, nc);
             }
             if (most < 1) return set_err(c, FRICO_GPU_ECUDA, "no SM pair can hold the pair GEMM");
             g_pair_clusters[c->device & 63] = most;
             return FRICO_GPU_OK;
         })))
        return rc;
    const tc::GemmProb& P = q.p;
    const int ntp = ((P.M + 2 * tc::BM - 1) / (2 * tc::BM)) * ((P.N + 255) / 256);
    const int ncl = std::max(1, std::min({ntp, cap / 2, g_pair_clusters[ctx->device & 63].load()}));
    tc::GemmArgs ga;
    ga.p[0] = P;
    ga.p[1] = P;
    ga.nprob = 1;
    ga.KP = KP;
    ga.st = (DeviceStatus*)ctx->status.p;
    if (ev) cudaEventRecord(ev[0], st);
    if (q.h)
        tc::k_gemm_pair_f16x3<<<2 * ncl, tc::kThreads, tc::Cfg<128>::SMEM_BYTES, st>>>(q.mah, q.mal, q.mbh, q.mbl, ga);
    else
        tc::k_gemm_pair_tf32x3<<<2 * ncl, tc::kThreads, tc::Cfg<128>::SMEM_BYTES, st>>>(q.mah, q.mal, q.mbh, q.mbl, ga);
    if (ev) cudaEventRecord(ev[1], st);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), q.h ? "k_gemm_pair_f16x3" : "k_gemm_pair_tf32x3");
}

static int launch_gemm(frico_gpu_ctx* ctx, cudaStream_t st, const TcProblem* q, int np, int KP, int max_ctas,
                       cudaEvent_t* ev) {
    int rc;
    if ((rc = device_once(ctx, kOnceGemmTc, [](frico_gpu_ctx* c) {
             int r = cuda_check(c, cudaFuncSetAttribute(tc::k_gemm_tf32x3<128>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        tc::Cfg<128>::SMEM_BYTES), "tc smem attribute");
             if (r) return r;
             return cuda_check(c, cudaFuncSetAttribute(tc::k_gemm_f16x3<128>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       tc::Cfg<128>::SMEM_BYTES), "tc smem attribute");
         })))
        return rc;
    if (np > 1 && q[0].h != q[1].h) return set_err(ctx, FRICO_GPU_EINVAL, "launch_gemm: mixed operand types");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int cap = max_ctas > 0 ? std::min(max_ctas, sms) : sms;
    if (kPairGemm && np == 1 && q[0].p.emit == 0 && q[0].p.N > 128 && q[0].p.M > tc::BM && cap >= 2)
        return launch_gemm_pair(ctx, st, q[0], KP, cap, ev);
    tc::GemmArgs ga;
    ga.p[0] = q[0].p;
    ga.p[1] = q[np > 1 ? 1 : 0].p;
    ga.nprob = np;
    ga.KP = KP;
    ga.st = (DeviceStatus*)ctx->status.p;
    const int ntiles = q[0].p.tiles + (np > 1 ? q[1].p.tiles : 0);
    if (ntiles == 0) return FRICO_GPU_OK;
    const TcProblem& q1 = q[np > 1 ? 1 : 0];
    if (ev) cudaEventRecord(ev[0], st);
    if (q[0].h)
        tc::k_gemm_f16x3<128><<<std::min(ntiles, cap), tc::kThreads, tc::Cfg<128>::SMEM_BYTES, st>>>(
            q[0].mah, q[0].mal, q[0].mbh, q[0].mbl, q1.mah, q1.mal, q1.mbh, q1.mbl, ga);
    else
        tc::k_gemm_tf32x3<128><<<std::min(ntiles, cap), tc::kThreads, tc::Cfg<128>::SMEM_BYTES, st>>>(
            q[0].mah, q[0].mal, q[0].mbh, q[0].mbl, q1.mah, q1.mal, q1.mbh, q1.mbl, ga);
    if (ev) cudaEventRecord(ev[1], st);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), q[0].h ? "k_gemm_f16x3" : "k_gemm_tf32x3");
}

// C[m x n] -= L[m x k] * U[k x n] (accumulate = 1) or C = L U (accumulate = 0),
// complex64 column-major, leading dims ldc, ldl, ldu. C may alias L or U: both
// operands are copied (split) before the MMA kernel writes C. f16 = 1: 3xFP16
// operands (L x 2^6, U x 2^8, for entries of order one), else 3xTF32.
int gemm_update_tc(frico_gpu_ctx* ctx, float2* C, int64_t ldc, const float2* L, int64_t ldl, const float2* U,
                   int64_t ldu, int m, int n, int k, cudaEvent_t* ev, int accumulate, int max_ctas, int reuse_a,
                   int f16) {
    if (m <= 0 || n <= 0 || k <= 0) return FRICO_GPU_OK;
    const int slab = f16 ? 2 * tc::BK : tc::BK;
    const int KP = ((2 * k + slab - 1) / slab) * slab;
    const int M = 2 * m;
    const size_t a_elems = size_t(M) * KP, b_elems = size_t(n) * KP;
    int rc;
    const size_t before = ctx->tc_ws.bytes;
    if ((rc = ensure(ctx, ctx->tc_ws, sizeof(float) * 2 * (a_elems + b_elems) + 4096))) return rc;
    if (ctx->tc_ws.bytes != before) reuse_a = 0;   // regrown workspace (even at the same address): split again
    const size_t esz = f16 ? 2 : 4;
    char* Ah = (char*)(((uintptr_t)ctx->tc_ws.p + 1023) & ~uintptr_t(1023));
    char* Al = Ah + a_elems * esz;
    char* Bh = Al + a_elems * esz;
    char* Bl = Bh + b_elems * esz;
    cudaStream_t st = ctx->stream;
    const Pow2Scale as{nullptr, 64.f, 0}, bs{nullptr, 256.f, 0}, rs{nullptr, 1.f / (64.f * 256.f), 0};
    tc::SplitPart parts[2];
    int np = 0;
    if (!reuse_a) parts[np++] = split_part(false, L, ldl, m, k, Ah, Al, KP, f16 ? &as : nullptr);
    parts[np++] = split_part(true, U, ldu, n, k, Bh, Bl, KP, f16 ? &bs : nullptr);
    if ((rc = launch_split(ctx, st, parts, np, KP))) return rc;
    TcProblem q;
    if ((rc = make_problem(ctx, q, C, ldc, M, n, Ah, Al, Bh, Bl, KP, accumulate, 0, nullptr, nullptr,
                           f16 ? &rs : nullptr)))
        return rc;
    return launch_gemm(ctx, st, &q, 1, KP, max_ctas, ev);
}

// Two independent real products C_i = A_i B_i^T (overwrite, no accumulation) in one
// launch, from operands already split into TF32 hi / lo, K-major: A_i with M rows, B_i with
// N_i rows, KP values per row (a multiple of 32). C_i is real, M x N_i, column-major with
// leading dimension ldc_i floats. Consecutive tiles walk N first, so the CTAs working on
// the N tiles of one A tile run together and read it once from DRAM.
int gemm_tc_split_pair(frico_gpu_ctx* ctx, cudaStream_t st, int M, int KP, float* C1, int64_t ldc1, int N1,
                       const float* A1h, const float* A1l, const float* B1h, const float* B1l, float* C2,
                       int64_t ldc2, int N2, const float* A2h, const float* A2l, const float* B2h,
                       const float* B2l) {
    if (KP % tc::BK != 0 || M <= 0 || N1 <= 0 || N2 <= 0 || ldc1 < M || ldc2 < M)
        return set_err(ctx, FRICO_GPU_EINVAL, "gemm_tc_split_pair: bad shape");
    TcProblem q[2];
    int rc;
    if ((rc = make_problem(ctx, q[0], (float2*)C1, 0, M, N1, A1h, A1l, B1h, B1l, KP, 0, 0, nullptr, nullptr)))
        return rc;
    if ((rc = make_problem(ctx, q[1], (float2*)C2, 0, M, N2, A2h, A2l, B2h, B2l, KP, 0, 0, nullptr, nullptr)))
        return rc;
    q[0].p.ldc = ldc1;
    q[1].p.ldc = ldc2;
    q[0].p.nfast = q[1].p.nfast = 1;
    return launch_gemm(ctx, st, q, 2, KP, 0, nullptr);
}

// Two independent real products C_i (+)= A_i B_i^T with sums in double-float: as
// gemm_tc_split_pair, but C_i holds double-float (hi, lo) pairs (M x N_i, column-major,
// ld ldc_i pairs),
// overwritten (accumulate = 0) or added to (1); a fresh TMEM accumulator every `group`
// k-steps (1, 2 or 4).
int gemm_tc_dfacc_pair(frico_gpu_ctx* ctx, cudaStream_t st, int M, int KP, int group, int accumulate, float2* C1,
                       int64_t ldc1, int N1, const float* A1h, const float* A1l, const float* B1h, const float* B1l,
                       float2* C2, int64_t ldc2, int N2, const float* A2h, const float* A2l, const float* B2h,
                       const float* B2l) {
    if (KP % tc::BK != 0 || M <= 0 || N1 <= 0 || N2 <= 0 || ldc1 < M || ldc2 < M ||
        (group != 1 && group != 2 && group != 4))
        return set_err(ctx, FRICO_GPU_EINVAL, "gemm_tc_dfacc_pair: bad shape");
    int rc;
    if ((rc = device_once(ctx, kOnceGemmDf, [](frico_gpu_ctx* c) {
             return cuda_check(c, cudaFuncSetAttribute(tc::k_gemm_dfacc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       tc::kDfSmemBytes), "dfacc smem attribute");
         })))
        return rc;
    TcProblem q[2];
    if ((rc = make_problem(ctx, q[0], nullptr, 0, M, N1, A1h, A1l, B1h, B1l, KP, 0, 0, nullptr, nullptr))) return rc;
    if ((rc = make_problem(ctx, q[1], nullptr, 0, M, N2, A2h, A2l, B2h, B2l, KP, 0, 0, nullptr, nullptr))) return rc;
    tc::DfArgs a;
    a.p[0] = tc::DfProb{C1, ldc1, M, N1, q[0].p.tiles_m, q[0].p.tiles};
    a.p[1] = tc::DfProb{C2, ldc2, M, N2, q[1].p.tiles_m, q[1].p.tiles};
    a.nprob = 2;
    a.KP = KP;
    a.group = group;
    a.accumulate = accumulate;
    a.st = (DeviceStatus*)ctx->status.p;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int ntiles = a.p[0].tiles + a.p[1].tiles;
    tc::k_gemm_dfacc<<<std::min(ntiles, sms), tc::kThreads, tc::kDfSmemBytes, st>>>(
        q[0].mah, q[0].mal, q[0].mbh, q[0].mbl, q[1].mah, q[1].mal, q[1].mbh, q[1].mbl, a);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_gemm_dfacc");
}

// ---- the no-pivot LU's block column in three launches (see lu_nopiv.cu)
static const int kPanelKP = 256;   // K = 128 complex columns

static size_t al1k(size_t floats) { return (floats + 255) & ~size_t(255); }   // keep slots 1 KB aligned

// Fixed slots (sized for rest = n - 128, 4 bytes per value whichever the
// operand type): U11^-1 (B^), L11^-1 (A*) from the diagonal-block kernel; A21
// (A*), A12 (B^) from tc_lu_panel_split; L21 (A*), U12 (B^) from the panel
// GEMM's epilogue. Each hi then lo. Then the operand scale s of the 3xFP16 form.
struct PanelSlots {
    float *uh, *ul, *lh, *ll, *a21h, *a21l, *a12h, *a12l, *lah, *lal, *ubh, *ubl;
    float* scale;   // s, then the result scales of L21 and U12 (written by the diagonal-block kernel)
};

static PanelSlots panel_slots(void* ws, int64_t n) {
    const size_t r = size_t(std::max<int64_t>(n - 128, 0)), KP = kPanelKP;
    float* base = (float*)(((uintptr_t)ws + 1023) & ~uintptr_t(1023));
    auto take = [&](size_t floats) { float* p = base; base += al1k(floats); return p; };
    PanelSlots s;
    s.uh = take(128 * KP);
    s.ul = take(128 * KP);
    s.lh = take(256 * KP);
    s.ll = take(256 * KP);
    s.a21h = take(2 * r * KP);
    s.a21l = take(2 * r * KP);
    s.a12h = take(r * KP);
    s.a12l = take(r * KP);
    s.lah = take(2 * r * KP);
    s.lal = take(2 * r * KP);
    s.ubh = take(r * KP);
    s.ubl = take(r * KP);
    s.scale = take(3);
    return s;
}

size_t tc_panel_ws_bytes(int64_t n) {
    const size_t r = size_t(std::max<int64_t>(n - 128, 0)), KP = kPanelKP;
    return sizeof(float) * (2 * (2 * al1k(2 * r * KP) + 2 * al1k(r * KP) + al1k(128 * KP) + al1k(256 * KP)) +
                            al1k(3)) +
           4096;
}

// The block columns use 3xFP16 operands when that engine is asked for, else 3xTF32.
static bool panel_f16(const frico_gpu_ctx* ctx) { return ctx->opt.gemm_engine == FRICO_GEMM_TC_F16; }

// Scales of the 3xFP16 operands and results, all powers of two:
//   A21, A12, U12 (Z-sized)   x s, s = 2^(9 - e) with 2^(e-1) <= max |diag Z| < 2^e,
//                             so that Z-sized values sit in [2^8, 2^9)
//   L21 (multipliers)         x 2^6
//   U11^-1, L11^-1            x u, l: each diagonal block's own, its largest entry
//                             in [2^8, 2^9); the diagonal-block kernel writes them
//                             and the result scales 1 / (s u) (L21) and 1 / (l s) (U12)
// FP16 holds up to 65504, so a Z-sized operand may grow 2^7 past max |diag Z| and a
// multiplier may reach 2^10 before it overflows; the lo part keeps 2^-25 of the
// value or, below FP16's normal range, an absolute 2^-25.
static const float kOrderOne = 64.f;

namespace tc {
// One CTA: s from the diagonal of A (n x n, lda).
__global__ void __launch_bounds__(1024) k_lu_scale(const float2* __restrict__ A, int64_t lda, int n, float* sc) {
    __shared__ float red[32];
    float m = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float2 a = A[int64_t(i) * lda + i];
        m = fmaxf(m, fmaxf(fabsf(a.x), fabsf(a.y)));   // fmaxf drops NaN
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) {
            int ex = 0;   // s = 1 for a zero or non-finite diagonal
            if (m > 0.f && isfinite(m)) {
                const int eb = int((__float_as_uint(m) >> 23) & 0xFF);   // 0 for a subnormal maximum
                ex = min(60, max(-60, 135 - max(eb, 1)));                 // 2^(eb-127) <= m < 2^(eb-126)
            }
            *sc = __uint_as_float(uint32_t(127 + ex) << 23);
        }
    }
}
}  // namespace tc

int tc_diag_split_slots(frico_gpu_ctx* ctx, TcDiagSplit* out) {
    int rc;
    if ((rc = ensure(ctx, ctx->tc_ws, tc_panel_ws_bytes(ctx->n)))) return rc;
    const PanelSlots s = panel_slots(ctx->tc_ws.p, ctx->n);
    out->uh = s.uh;
    out->ul = s.ul;
    out->lh = s.lh;
    out->ll = s.ll;
    out->h = panel_f16(ctx) ? 1 : 0;
    out->sc = s.scale;
    out->res_l21 = s.scale + 1;
    out->res_u12 = s.scale + 2;
    return FRICO_GPU_OK;
}

// The operand scale s of the 3xFP16 block columns, from the diagonal of A (a
// no-op for 3xTF32 operands); before the first diagonal block.
int tc_lu_scale(frico_gpu_ctx* ctx, const float2* A, int64_t lda, int n) {
    if (!panel_f16(ctx)) return FRICO_GPU_OK;
    int rc;
    if ((rc = ensure(ctx, ctx->tc_ws, tc_panel_ws_bytes(ctx->n)))) return rc;
    const PanelSlots s = panel_slots(ctx->tc_ws.p, ctx->n);
    tc::k_lu_scale<<<1, 1024, 0, ctx->stream>>>(A, lda, n, s.scale);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_lu_scale");
}

// A21 (rest x 128, below the diagonal block) as A* and A12 (128 x rest, right of it)
// as B^ operands of the panel GEMM; independent of the diagonal block's factors.
int tc_lu_panel_split(frico_gpu_ctx* ctx, float2* A, int64_t lda, int k0, int jb, int rest) {
    const int KP = kPanelKP;
    if (jb != 128 || rest <= 0) return set_err(ctx, FRICO_GPU_EINVAL, "tc_lu_panel_split: block of 128 expected");
    int rc;
    if ((rc = ensure(ctx, ctx->tc_ws, tc_panel_ws_bytes(ctx->n)))) return rc;
    const PanelSlots s = panel_slots(ctx->tc_ws.p, ctx->n);
    const Pow2Scale zs{s.scale, 1.f, 1};
    const Pow2Scale* h = panel_f16(ctx) ? &zs : nullptr;
    float2* A21 = A + int64_t(k0) * lda + k0 + jb;
    float2* A12 = A + int64_t(k0 + jb) * lda + k0;
    const tc::SplitPart parts[2] = {split_part(false, A21, lda, rest, jb, s.a21h, s.a21l, KP, h),
                                    split_part(true, A12, lda, rest, jb, s.a12h, s.a12l, KP, h)};
    return launch_split(ctx, ctx->stream, parts, 2, KP);
}

// L21 = A21 U11^{-1} and U12 = L11^{-1} A12 (in place in A, jb = 128 columns /
// rows, rest = rows of A21 = columns of A12) as one launch from the split operands
// (tc_lu_panel_split, and the diagonal-block kernel for U11^{-1}, L11^{-1}); the
// epilogues also write L21 as the A* and U12 as the B^ operand of the block
// column's trailing updates (tc_lu_update).
int tc_lu_panel(frico_gpu_ctx* ctx, float2* A, int64_t lda, int k0, int jb, int rest, TcPanel* out) {
    const int KP = kPanelKP;
    if (jb != 128 || rest <= 0) return set_err(ctx, FRICO_GPU_EINVAL, "tc_lu_panel: block of 128 expected");
    int rc;
    if ((rc = ensure(ctx, ctx->tc_ws, tc_panel_ws_bytes(ctx->n)))) return rc;
    const PanelSlots s = panel_slots(ctx->tc_ws.p, ctx->n);
    const bool h = panel_f16(ctx);
    out->Lah = s.lah;
    out->Lal = s.lal;
    out->Ubh = s.ubh;
    out->Ubl = s.ubl;
    out->rest = rest;
    out->KP = KP;
    out->h = h ? 1 : 0;
    out->sc = s.scale;
    float2* A21 = A + int64_t(k0) * lda + k0 + jb;
    float2* A12 = A + int64_t(k0 + jb) * lda + k0;
    // L21: (A21 s)(U11^-1 u) = s u L21, emitted as 2^6 L21;
    // U12: (L11^-1 l)(A12 s) = l s U12, emitted as s U12
    const Pow2Scale r1{s.scale + 1, 1.f, 1}, e1{nullptr, kOrderOne, 0};
    const Pow2Scale r2{s.scale + 2, 1.f, 1}, e2{s.scale, 1.f, 1};
    TcProblem q[2];
    if ((rc = make_problem(ctx, q[0], A21, lda, 2 * rest, jb, s.a21h, s.a21l, s.uh, s.ul, KP, 0, 1, s.lah, s.lal,
                           h ? &r1 : nullptr, h ? &e1 : nullptr)))
        return rc;
    if ((rc = make_problem(ctx, q[1], A12, lda, 2 * jb, rest, s.lh, s.ll, s.a12h, s.a12l, KP, 0, 2, s.ubh, s.ubl,
                           h ? &r2 : nullptr, h ? &e2 : nullptr)))
        return rc;
    return launch_gemm(ctx, ctx->stream, q, 2, KP, 0, nullptr);
}

// C[rest x ncols] -= L21 U12[:, boff : boff + ncols] from the operands tc_lu_panel wrote.
int tc_lu_update(frico_gpu_ctx* ctx, const TcPanel& pn, float2* C, int64_t ldc, int boff, int ncols, int max_ctas,
                 cudaEvent_t* ev) {
    if (ncols <= 0) return FRICO_GPU_OK;
    const int KP = pn.KP;
    const size_t esz = pn.h ? 2 : 4, boff_bytes = size_t(boff) * KP * esz;
    // (L21 2^6)(U12 s) = 2^6 s L21 U12
    const Pow2Scale r3{pn.sc, 1.f / kOrderOne, -1};
    TcProblem q;
    int rc;
    if ((rc = make_problem(ctx, q, C, ldc, 2 * pn.rest, ncols, pn.Lah, pn.Lal, (const char*)pn.Ubh + boff_bytes,
                           (const char*)pn.Ubl + boff_bytes, KP, 1, 0, nullptr, nullptr, pn.h ? &r3 : nullptr)))
        return rc;
    return launch_gemm(ctx, ctx->stream, &q, 1, KP, max_ctas, ev);
}

}  // namespace frico
