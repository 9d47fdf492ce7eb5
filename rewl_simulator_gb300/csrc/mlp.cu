// Learned warm start: an MLP surrogate ln g(E)/N = f(E/N, 1/L, J, K, sigma_h,
// window lo/N, window hi/N), trained and evaluated on the GPU with hand-written
// BF16 tensor-core GEMMs (tcgen05.mma with the FP32 accumulator in tensor memory;
// an mma.sync m16n8k16 kernel is kept for comparison), a fused bias + GELU
// epilogue, split-K weight gradients, and Adam on FP32 master weights.
//
// Shapes: 7 inputs (padded to 64) -> 4 x 256 (GELU) -> 1 output (padded to 64).
// A batch of 4096 is 4096 x 256 x 256 per hidden GEMM, i.e. latency-bound work.
// The tiles are therefore small (128 x 64 on tcgen05, 64 x 64 on mma.sync) so
// that a layer spans many blocks, and every GEMM of a step runs on one stream.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rewl.h"
#include "rng.cuh"

namespace {

thread_local std::string g_mlp_error;

int mfail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_mlp_error = buf;
    return code;
}

#define MCUDA(expr)                                                                     \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess)                                                          \
            return mfail(REWL_EDEVICE, "%s: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                         __FILE__, __LINE__);                                           \
    } while (0)

typedef __nv_bfloat16 bf16;

constexpr int kBM = 64, kBN = 64, kBK = 32, kPad = 8;
constexpr int kIn = 64;        // padded input width (a multiple of the 64-wide tile)
constexpr int kOut = 64;       // padded output width

// ---------------------------------------------------------------------------
// GEMM: C[M x N] = op(A) * op(B) with bf16 operands, fp32 accumulation.
//   A_KM = false: A stored [M][K] (lda = K);  true: A stored [K][M] (lda = M)
//   B_NK = true:  B stored [N][K] (ldb = K);  false: B stored [K][N] (ldb = N)
// M, N multiples of 64, K (per split) a multiple of 32.
// Epilogues:
//   EPI_F32:       C fp32 (split over K: split z writes its partial at C + z * M * ldc)
//   EPI_BIAS_GELU: Z = acc + bias -> Zout (fp32), Y = gelu(Z) -> Yout (bf16)
//   EPI_BIAS_F32:  acc + bias -> fp32
//   EPI_BF16:      acc -> bf16
// ---------------------------------------------------------------------------
enum { EPI_F32 = 0, EPI_BIAS_GELU = 1, EPI_BIAS_F32 = 2, EPI_BF16 = 3 };

struct GemmArgs {
    const bf16* A;
    const bf16* B;
    int M, N, K, lda, ldb;
    int k_per_split;
    float* Cf;
    bf16* Cb;
    int ldc;
    const float* bias;
};

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <bool A_KM, bool B_NK, int EPI>
__global__ void __launch_bounds__(128) k_gemm(const GemmArgs g)
{
    // shared tiles, rows padded by 8 bf16 (16 B) so ldmatrix rows hit distinct banks
    constexpr int A_ROWS = A_KM ? kBK : kBM, A_COLS = A_KM ? kBM : kBK;
    constexpr int B_ROWS = B_NK ? kBN : kBK, B_COLS = B_NK ? kBK : kBN;
    __shared__ __align__(16) bf16 As[A_ROWS][A_COLS + kPad];
    __shared__ __align__(16) bf16 Bs[B_ROWS][B_COLS + kPad];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;   // warp's 32 x 32 sub-tile
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    const int kb = blockIdx.z * g.k_per_split, ke = kb + g.k_per_split;

    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    for (int k0 = kb; k0 < ke; k0 += kBK) {
        // global -> shared, 16-byte chunks: each tile is 64 x 32 bf16 = 256 chunks
        for (int c = tid; c < 256; c += 128) {
            if (!A_KM) {
                const int r = c >> 2, q = (c & 3) * 8;      // [64 m][32 k]
                *reinterpret_cast<uint4*>(&As[r][q]) = *reinterpret_cast<const uint4*>(g.A + (size_t)(m0 + r) * g.lda + k0 + q);
            } else {
                const int r = c >> 3, q = (c & 7) * 8;      // [32 k][64 m]
                *reinterpret_cast<uint4*>(&As[r][q]) = *reinterpret_cast<const uint4*>(g.A + (size_t)(k0 + r) * g.lda + m0 + q);
            }
            if (B_NK) {
                const int r = c >> 2, q = (c & 3) * 8;      // [64 n][32 k]
                *reinterpret_cast<uint4*>(&Bs[r][q]) = *reinterpret_cast<const uint4*>(g.B + (size_t)(n0 + r) * g.ldb + k0 + q);
            } else {
                const int r = c >> 3, q = (c & 7) * 8;      // [32 k][64 n]
                *reinterpret_cast<uint4*>(&Bs[r][q]) = *reinterpret_cast<const uint4*>(g.B + (size_t)(k0 + r) * g.ldb + n0 + q);
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; kk += 16) {
            uint32_t a[2][4], b[4][2];
            const int mat = lane >> 3, rin = lane & 7;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int mb = wm + i * 16;
                if (!A_KM) ldsm_x4(a[i][0], a[i][1], a[i][2], a[i][3], &As[mb + (mat & 1) * 8 + rin][kk + (mat >> 1) * 8]);
                else ldsm_x4_t(a[i][0], a[i][1], a[i][2], a[i][3], &As[kk + (mat >> 1) * 8 + rin][mb + (mat & 1) * 8]);
            }
#pragma unroll
            for (int jp = 0; jp < 2; ++jp) {
                const int nb = wn + jp * 16;
                if (B_NK) ldsm_x4(b[2 * jp][0], b[2 * jp][1], b[2 * jp + 1][0], b[2 * jp + 1][1],
                                  &Bs[nb + (mat >> 1) * 8 + rin][kk + (mat & 1) * 8]);
                else ldsm_x4_t(b[2 * jp][0], b[2 * jp][1], b[2 * jp + 1][0], b[2 * jp + 1][1],
                               &Bs[kk + (mat & 1) * 8 + rin][nb + (mat >> 1) * 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i][0], a[i][1], a[i][2], a[i][3], b[j][0], b[j][1]);
        }
        __syncthreads();
    }
    // epilogue: thread owns rows (lane>>2) and +8, columns 2*(lane&3) + {0,1} of each 16 x 8 tile
    const int gr = lane >> 2, tc = (lane & 3) * 2;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = m0 + wm + i * 16 + gr + h * 8;
                const int col = n0 + wn + j * 8 + tc;
                float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
                const size_t o = (size_t)row * g.ldc + col;
                if (EPI == EPI_F32) {
                    // a K split stores its partial product in its own slice (summed in order afterwards)
                    float* c = g.Cf + (size_t)blockIdx.z * g.M * g.ldc;
                    c[o] = v0; c[o + 1] = v1;
                } else if (EPI == EPI_BIAS_GELU) {
                    v0 += g.bias[col]; v1 += g.bias[col + 1];
                    g.Cf[o] = v0; g.Cf[o + 1] = v1;
                    *reinterpret_cast<__nv_bfloat162*>(g.Cb + o) = __floats2bfloat162_rn(gelu_f(v0), gelu_f(v1));
                } else if (EPI == EPI_BIAS_F32) {
                    g.Cf[o] = v0 + g.bias[col]; g.Cf[o + 1] = v1 + g.bias[col + 1];
                } else {
                    *reinterpret_cast<__nv_bfloat162*>(g.Cb + o) = __floats2bfloat162_rn(v0, v1);
                }
            }
}

// ---------------------------------------------------------------------------
// The same GEMM on the 5th-generation tensor cores (tcgen05), the default.
//
// One CTA computes a 128 x 64 tile of C.  Its K range is cut into blocks of 64
// that stream through a ring of four shared-memory stages, loaded by the tensor
// memory accelerator (cp.async.bulk.tensor, 2-D tensor maps over A and B, rows
// beyond the matrix zero-filled) three blocks ahead of the one being multiplied.
// Tiles are kept in tcgen05's canonical layouts without swizzle, built from
// "core matrices" of 8 rows x 16 B (128 contiguous bytes):
//  * an operand stored with K contiguous (K-major: a core row = 8 consecutive k
//    of one row) is loaded as 8 boxes of 8 k x R rows, one per 8-wide column of
//    k, each landing R x 16 B: core matrices along K are R x 16 B apart (LBO),
//    8-row groups 128 B apart (SBO);
//  * an operand stored with M or N contiguous (MN-major: a core row = 8
//    consecutive rows at one k) is loaded as R / 8 boxes of 8 rows x 64 k, each
//    landing 1024 B: core matrices along K 128 B apart (LBO), 8-row groups 1024 B
//    (SBO), with the transpose bit of the instruction descriptor.
// One thread issues the copies (arming the stage's "full" mbarrier with the
// stage's byte count) and, once a stage is full, four tcgen05.mma (M 128, N 64,
// K 16 each) from shared-memory descriptors into an FP32 accumulator in tensor
// memory (64 columns, allocated per CTA), committed to the stage's "empty"
// mbarrier, which releases the stage for the block four ahead.  The epilogue reads
// the accumulator back with tcgen05.ld (warp w owns rows 32w..32w+31, one row per
// thread) and applies the same epilogues as above.
//
// Every wait on an mbarrier is bounded: on a timeout the block records
// kTcTimeout in g_tc_error, waits once more (bounded) for the copies it issued
// and its MMAs, frees its tensor memory and skips the epilogue.  K splits are
// whole 64-wide blocks (gemm() checks it), so no box reaches another split's K.
// ---------------------------------------------------------------------------
namespace tc {
constexpr int BM = 128, BN = 64, BK = 64, STAGES = 4;
constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 128;  // + full / empty mbarriers and the tensor-memory address
constexpr uint32_t kTmemCols = 64;                     // FP32 accumulator: 128 lanes x 64 columns
// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// A / B MN-major (transposed) in bits 15 / 16, N >> 3 in bits 17-22, M >> 4 in bits 24-28
__host__ __device__ constexpr uint32_t idesc(bool a_mn, bool b_mn)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
           ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}
constexpr int kSpinLimit = 1 << 18;
constexpr int kTcTimeout = 1;
static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256 && BM == 128, "tcgen05.mma cta_group::1 kind::f16 shape");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert(STAGE_BYTES % 1024 == 0 && A_BYTES % 1024 == 0, "stages and tiles on 1024-byte boundaries");
}  // namespace tc

__device__ int g_tc_error;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29), SBO >> 4 (32-45),
// descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (int i = 0; i < tc::kSpinLimit; ++i) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// one 2-D box of the tensor map at (x, y) (x along the contiguous dimension, a multiple of 8
// elements: 16 bytes) into shared memory at dst, completing `bytes` on the mbarrier bar
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n"
                 :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar) : "memory");
}

// The boxes of one operand tile (R rows from r0, K block from k0) into shared memory at dst.
// KMAJ: the map's contiguous dimension is K (boxes of 8 k x R rows); otherwise it is the rows
// (boxes of 8 rows x BK k).
template <int R, bool KMAJ>
__device__ __forceinline__ void load_tile(uint32_t dst, const CUtensorMap* map, int r0, int k0, uint32_t bar)
{
    if (KMAJ) {
#pragma unroll
        for (int c = 0; c < tc::BK / 8; ++c) tma_load_2d(dst + c * (R * 16), map, k0 + 8 * c, r0, bar);
    } else {
#pragma unroll
        for (int g = 0; g < R / 8; ++g) tma_load_2d(dst + g * 1024, map, r0 + 8 * g, k0, bar);
    }
}

// descriptor of the K = 16 slice kk of an R-row operand tile at addr (layouts above)
template <int R, bool KMAJ>
__device__ __forceinline__ uint64_t tile_desc(uint32_t addr, int kk)
{
    return KMAJ ? smem_desc(addr + kk * 2 * (R * 16), R * 16, 128) : smem_desc(addr + kk * 256, 128, 1024);
}

template <bool A_KM, bool B_NK, int EPI>
__global__ void __launch_bounds__(128) k_gemm_tc(const GemmArgs g, const __grid_constant__ CUtensorMap tmA,
                                                 const __grid_constant__ CUtensorMap tmB)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + tc::STAGES * tc::STAGE_BYTES);
    uint64_t* empty = full + tc::STAGES;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(empty + tc::STAGES);
    int* status = reinterpret_cast<int*>(tslot + 1);        // thread 0's outcome: MMAs committed, or -1
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * tc::BM, n0 = blockIdx.x * tc::BN;
    const int kb = blockIdx.z * g.k_per_split, ke = min(kb + g.k_per_split, g.K);
    const int nk = (ke - kb + tc::BK - 1) / tc::BK;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" :: "r"(smem_u32(tslot)), "r"(tc::kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < 2 * tc::STAGES; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(full + s)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" :: "l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" :: "l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;

    constexpr int S = tc::STAGES;
    constexpr uint32_t kId = tc::idesc(A_KM, !B_NK);
    if (tid == 0) {
        const uint32_t sbase = smem_u32(sm);
        auto load = [&](int t) {                        // block t into stage t % S
            const uint32_t As = sbase + (t % S) * tc::STAGE_BYTES, fb = smem_u32(full + t % S);
            const int k0 = kb + t * tc::BK;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(fb), "r"(tc::STAGE_BYTES) : "memory");
            load_tile<tc::BM, !A_KM>(As, &tmA, m0, k0, fb);
            load_tile<tc::BN, B_NK>(As + tc::A_BYTES, &tmB, n0, k0, fb);
        };
        int loaded = 0, issued = 0;                     // blocks whose copies / MMAs were issued
        bool ok = true;
        for (; loaded < min(S - 1, nk); ++loaded) load(loaded);
        for (int t = 0; t < nk; ++t) {
            if (loaded < nk) {                          // block t+S-1 reuses the stage of block t-1
                if (t >= 1 && !mbar_wait(smem_u32(empty + (t - 1) % S), (uint32_t)(((t - 1) / S) & 1))) { ok = false; break; }
                load(loaded++);
            }
            if (!mbar_wait(smem_u32(full + t % S), (uint32_t)((t / S) & 1))) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t As = sbase + (t % S) * tc::STAGE_BYTES, Bs = As + tc::A_BYTES;
#pragma unroll
            for (int kk = 0; kk < tc::BK / 16; ++kk) {
                const uint64_t ad = tile_desc<tc::BM, !A_KM>(As, kk);
                const uint64_t bd = tile_desc<tc::BN, B_NK>(Bs, kk);
                const uint32_t accumulate = (t > 0 || kk > 0) ? 1u : 0u;
                asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                             :: "r"(tmem), "l"(ad), "l"(bd), "r"(kId), "r"(accumulate) : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" :: "r"(smem_u32(empty + t % S)) : "memory");
            issued = t + 1;
        }
        if (!ok) {
            // no copy outlives the block: wait (bounded) for the copies not yet consumed
            for (int u = issued; u < loaded; ++u) mbar_wait(smem_u32(full + u % S), (uint32_t)((u / S) & 1));
        }
        if (issued > 0) {                               // the last commit covers every earlier MMA
            const int t = issued - 1;
            ok = mbar_wait(smem_u32(empty + t % S), (uint32_t)((t / S) & 1)) && ok;
        }
        if (!ok) atomicOr(&g_tc_error, tc::kTcTimeout);
        *status = ok ? issued : -1;
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

    if (*status > 0) {
        const int row = m0 + warp * 32 + lane;
#pragma unroll
        for (int c0 = 0; c0 < tc::BN; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                           "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (row < g.M) {
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
                const int col = n0 + c0;
                const size_t o = (size_t)row * g.ldc + col;
                if (EPI == EPI_F32) {
                    // a K split stores its partial product in its own slice (summed in order afterwards)
                    float* c = g.Cf + (size_t)blockIdx.z * g.M * g.ldc;
#pragma unroll
                    for (int j = 0; j < 16; j += 4) *reinterpret_cast<float4*>(c + o + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                } else if (EPI == EPI_BIAS_GELU || EPI == EPI_BIAS_F32) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] += g.bias[col + j];
#pragma unroll
                    for (int j = 0; j < 16; j += 4) *reinterpret_cast<float4*>(g.Cf + o + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                    if (EPI == EPI_BIAS_GELU) {
                        uint32_t h[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const __nv_bfloat162 b2 = __floats2bfloat162_rn(gelu_f(v[2 * j]), gelu_f(v[2 * j + 1]));
                            h[j] = *reinterpret_cast<const uint32_t*>(&b2);
                        }
                        *reinterpret_cast<uint4*>(g.Cb + o) = make_uint4(h[0], h[1], h[2], h[3]);
                        *reinterpret_cast<uint4*>(g.Cb + o + 8) = make_uint4(h[4], h[5], h[6], h[7]);
                    }
                } else {
                    uint32_t h[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                        h[j] = *reinterpret_cast<const uint32_t*>(&b2);
                    }
                    *reinterpret_cast<uint4*>(g.Cb + o) = make_uint4(h[0], h[1], h[2], h[3]);
                    *reinterpret_cast<uint4*>(g.Cb + o + 8) = make_uint4(h[4], h[5], h[6], h[7]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(tmem), "r"(tc::kTmemCols) : "memory");
    }
}

// cuTensorMapEncodeTiled from the driver, found once through the runtime (no link-time
// dependence on libcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled()
{
    static const EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (EncodeTiledFn) nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// A 2-D BF16 map over a matrix of `outer` rows of `inner` contiguous elements (row pitch ld
// elements) with boxes of 8 x box_outer; reads outside the matrix return zeros.
bool encode_operand(CUtensorMap* map, const bf16* p, int inner, int outer, int ld, int box_outer)
{
    const EncodeTiledFn fn = encode_tiled();
    if (!fn || (reinterpret_cast<uintptr_t>(p) & 15) || (ld & 7) || (inner & 7)) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(bf16)};
    const cuuint32_t box[2] = {8, (cuuint32_t)box_outer};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(p), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// REWL_MLP_GEMM=mma_sync selects the mma.sync kernel (kept for comparison)
bool use_tcgen05()
{
    static const bool tc5 = [] {
        const char* v = std::getenv("REWL_MLP_GEMM");
        return !(v && std::strcmp(v, "mma_sync") == 0);
    }();
    return tc5;
}

template <bool A_KM, bool B_NK, int EPI>
cudaError_t launch_gemm(cudaStream_t st, const GemmArgs& g, int splits)
{
    if (use_tcgen05()) {
        static_assert(tc::BN == kBN, "tile widths agree");
        // A: [M][K] (K-major, boxes 8 k x 128 rows) or [K][M] (boxes 8 rows x 64 k); B likewise with N
        CUtensorMap ma, mb;
        if (splits > 1 && g.k_per_split % tc::BK) return cudaErrorInvalidValue;     // a box would reach the next split
        const bool ok = (A_KM ? encode_operand(&ma, g.A, g.M, g.K, g.lda, tc::BK) : encode_operand(&ma, g.A, g.K, g.M, g.lda, tc::BM)) &&
                        (B_NK ? encode_operand(&mb, g.B, g.K, g.N, g.ldb, tc::BN) : encode_operand(&mb, g.B, g.N, g.K, g.ldb, tc::BK));
        if (!ok) return cudaErrorInvalidValue;
        k_gemm_tc<A_KM, B_NK, EPI><<<dim3(g.N / tc::BN, (g.M + tc::BM - 1) / tc::BM, splits), 128, tc::SMEM_BYTES, st>>>(g, ma, mb);
    } else {
        k_gemm<A_KM, B_NK, EPI><<<dim3(g.N / kBN, g.M / kBM, splits), 128, 0, st>>>(g);
    }
    return cudaGetLastError();
}

// The tensor-core GEMMs need more than the default 48 KB of dynamic shared memory.  Set
// once per device when a network is created, so that rewl_mlp_predict_noalloc, which only
// enqueues work, makes no attribute call.
cudaError_t prepare_tc_kernels()
{
    if (use_tcgen05() && !encode_tiled()) return cudaErrorNotSupported;   // found here, not while a caller captures
    const void* kernels[] = {
        reinterpret_cast<const void*>(k_gemm_tc<false, true, EPI_BIAS_GELU>),
        reinterpret_cast<const void*>(k_gemm_tc<false, true, EPI_BIAS_F32>),
        reinterpret_cast<const void*>(k_gemm_tc<true, false, EPI_F32>),
        reinterpret_cast<const void*>(k_gemm_tc<false, false, EPI_BF16>),
    };
    for (const void* k : kernels) {
        const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// a bounded wait in a tensor-core GEMM ran out since the last call: report it once
int take_tc_error()
{
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof v) != cudaSuccess) return mfail(REWL_EDEVICE, "reading the GEMM status failed");
    if (!v) return REWL_OK;
    const int zero = 0;
    cudaMemcpyToSymbol(g_tc_error, &zero, sizeof zero);
    return mfail(REWL_EDEVICE, "a tensor-core GEMM timed out waiting for its MMAs (results discarded)");
}

// G = dY * gelu'(Z) (bf16), dY given in bf16
__global__ void k_gelu_back(const bf16* dY, const float* Z, bf16* G, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float z = Z[i];
    const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
    const float pdf = 0.3989422804014327f * __expf(-0.5f * z * z);
    G[i] = __float2bfloat16_rn(__bfloat162float(dY[i]) * (cdf + z * pdf));
}

constexpr int kColChunk = 256;                                 // rows per column-sum partial

// column sums over chunks of kColChunk rows: part[chunk][n] = sum_{b in chunk} G[b][n]
__global__ void k_colsum(const bf16* G, int B, int N, float* part)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int b0 = blockIdx.y * kColChunk;
    if (n >= N) return;
    float s = 0.f;
    for (int b = b0; b < b0 + kColChunk && b < B; ++b) s += __bfloat162float(G[(size_t)b * N + n]);
    part[(size_t)blockIdx.y * N + n] = s;
}

// dst[i] = sum_p parts[p * stride + i], p in order: gradients are reproducible run to run
__global__ void k_sum_parts(const float* parts, int nparts, size_t stride, size_t n, float* dst)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.f;
    for (int p = 0; p < nparts; ++p) s += parts[(size_t)p * stride + i];
    dst[i] = s;
}

// K splits of a weight gradient over a batch of B rows: whole 64-row blocks per split (the
// tensor-core GEMM's K block), 16 from 4096 rows, 4 from 1024
int weight_splits(int B)
{
    if (B >= 4096 && B % (64 * 16) == 0) return 16;
    if (B >= 1024 && B % (64 * 4) == 0) return 4;
    return 1;
}

// loss gradient of the mean squared error mean((out[:,0] - y)^2); each row's share of the loss
// goes to rows[b] (summed in a fixed order by k_loss_sum)
__global__ void k_loss_grad(const float* out, const float* y, int B, bf16* dOut, float* rows)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float e = out[(size_t)b * kOut] - y[b];
    for (int c = 0; c < kOut; ++c) dOut[(size_t)b * kOut + c] = __float2bfloat16_rn(c == 0 ? 2.0f * e / (float)B : 0.f);
    rows[b] = e * e / (float)B;
}

// loss = sum of rows[0..B): one block of 256 threads, strided partial sums, then a fixed tree
__global__ void __launch_bounds__(256) k_loss_sum(const float* rows, int B, float* loss)
{
    __shared__ float part[256];
    float s = 0.f;
    for (int b = threadIdx.x; b < B; b += 256) s += rows[b];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = part[0];
}

// Adam on fp32 masters; refresh the bf16 copy.  mask zeroes the padded entries.
// Device state of a training call: the network's step counter and the index of the step within
// the call.  The kernels of a step read it, so that one captured step replays as the next.
struct TrainCursor {
    unsigned long long step;
    int k;
    int pad;
};

// Adam with the bias corrections of the cursor's step (c1 = 1 - b1^t, c2 = 1 - b2^t, computed on
// the host for every step of the call, two floats per step).
__global__ void k_adam(float* p, float* m, float* v, const float* grad, const float* mask, bf16* pb, size_t n,
                       float lr, float b1, float b2, float eps, const float* ctab, const TrainCursor* cur)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = cur->k;
    const float c1 = ctab[2 * k], c2 = ctab[2 * k + 1];
    const float gi = grad[i] * mask[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi; v[i] = vi;
    const float pi = (p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps)) * mask[i];
    p[i] = pi;
    if (pb) pb[i] = __float2bfloat16_rn(pi);
}

// batch gather with Philox indices: Xb = X[idx], yb = y[idx]
__global__ void k_gather(const bf16* X, const float* y, int n, bf16* Xb, float* yb, int B, uint64_t seed,
                         const TrainCursor* cur)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const uint64_t step = cur->step;
    const uint32_t w = rewl::philox_word(seed, 0x4D4C5000u, step * (uint64_t)B + (uint64_t)b, 0x4D4C5001u);
    const int i = (int)rewl::mulhi32(w, (uint32_t)n);
    for (int c = 0; c < kIn; c += 8)
        *reinterpret_cast<uint4*>(Xb + (size_t)b * kIn + c) = *reinterpret_cast<const uint4*>(X + (size_t)i * kIn + c);
    yb[b] = y[i];
}

// End of a training step: keep its loss, advance the cursor.
__global__ void k_train_advance(TrainCursor* cur, const float* loss, float* losses)
{
    losses[cur->k] = *loss;
    cur->step += 1;
    cur->k += 1;
}

template <typename T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        n = count;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return mfail(REWL_ENOMEM, "cudaMalloc failed");
        return cudaMemset(p, 0, count * sizeof(T)) == cudaSuccess ? REWL_OK : mfail(REWL_EDEVICE, "cudaMemset failed");
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
    }
};

} // namespace

struct rewl_mlp {
    int device = 0;
    int hidden = 256, layers = 4;
    int batch_cap = 0;
    cudaStream_t stream = nullptr;
    // layer l: weight [out_l x in_l] row-major, bias [out_l]; in_0 = 32, out_last = 64
    std::vector<int> din, dout;
    std::vector<size_t> woff, boff;
    size_t nparams = 0;
    Buf<float> P, Mm, Vm, Gr, Mask;   // fp32 master params, Adam moments, grads, pad mask
    Buf<bf16> Pb;                     // bf16 params (weights used by the GEMMs)
    // activations for the current batch
    std::vector<Buf<bf16>> H;         // H[0] = input (B x 32), H[l+1] = gelu(Z_l)
    std::vector<Buf<float>> Z;        // pre-activations (hidden layers)
    Buf<float> out, yb, loss, lossrow;
    Buf<float> Part;                  // per-split weight-gradient and per-chunk bias-gradient partials
    Buf<bf16> dOut, dH, G;
    Buf<bf16> Xall;
    Buf<float> yall;
    Buf<TrainCursor> cursor;          // training: step counter on the device
    Buf<float> ctab, lossv;           // training: bias corrections and losses of the call's steps
    int nall = 0;
    int64_t step = 0;
    uint64_t seed = 1;
    std::atomic<int64_t> launches{0};   // calls on one network from several threads may overlap

    void release()
    {
        P.release(); Mm.release(); Vm.release(); Gr.release(); Mask.release(); Pb.release();
        for (auto& h : H) h.release();
        for (auto& z : Z) z.release();
        out.release(); yb.release(); loss.release(); lossrow.release(); dOut.release(); dH.release(); G.release();
        Part.release();
        Xall.release(); yall.release();
        cursor.release(); ctab.release(); lossv.release();
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

namespace {

int ensure_batch(rewl_mlp* m, int B)
{
    if (B <= m->batch_cap) return REWL_OK;
    for (auto& h : m->H) h.release();
    for (auto& z : m->Z) z.release();
    m->out.release(); m->yb.release(); m->dOut.release(); m->dH.release(); m->G.release(); m->Part.release();
    m->lossrow.release();
    m->H.assign(m->layers + 1, Buf<bf16>());
    m->Z.assign(m->layers, Buf<float>());
    int rc;
    if ((rc = m->H[0].alloc((size_t)B * kIn))) return rc;
    for (int l = 0; l < m->layers; ++l) {
        if ((rc = m->H[l + 1].alloc((size_t)B * m->hidden))) return rc;
        if ((rc = m->Z[l].alloc((size_t)B * m->hidden))) return rc;
    }
    if ((rc = m->out.alloc((size_t)B * kOut)) || (rc = m->yb.alloc(B)) || (rc = m->dOut.alloc((size_t)B * kOut)) ||
        (rc = m->dH.alloc((size_t)B * m->hidden)) || (rc = m->G.alloc((size_t)B * m->hidden)))
        return rc;
    const size_t wmax = (size_t)std::max(m->hidden, std::max(kIn, kOut)) * m->hidden;     // largest weight block
    const size_t part = std::max((size_t)weight_splits(B) * wmax,
                                 (size_t)((B + kColChunk - 1) / kColChunk) * std::max(m->hidden, kOut));
    if ((rc = m->Part.alloc(part)) || (rc = m->lossrow.alloc(B))) return rc;
    m->batch_cap = B;
    return REWL_OK;
}

template <bool A_KM, bool B_NK, int EPI>
int gemm(rewl_mlp* m, const bf16* A, const bf16* B, int M, int N, int K, int lda, int ldb, int splits, float* Cf,
         bf16* Cb, int ldc, const float* bias)
{
    if (M % kBM || N % kBN || K % (kBK * splits)) return mfail(REWL_EINVAL, "gemm shape %d x %d x %d (split %d)", M, N, K, splits);
    GemmArgs g{A, B, M, N, K, lda, ldb, K / splits, Cf, Cb, ldc, bias};
    m->launches++;
    MCUDA((launch_gemm<A_KM, B_NK, EPI>(m->stream, g, splits)));
    return REWL_OK;
}

// forward for B rows already in H[0]; leaves outputs in m->out
int forward(rewl_mlp* m, int B)
{
    int rc;
    for (int l = 0; l < m->layers; ++l) {
        const bf16* W = m->Pb.p + m->woff[l];
        const float* bias = m->P.p + m->boff[l];
        if ((rc = gemm<false, true, EPI_BIAS_GELU>(m, m->H[l].p, W, B, m->dout[l], m->din[l], m->din[l], m->din[l], 1,
                                                   m->Z[l].p, m->H[l + 1].p, m->dout[l], bias)))
            return rc;
    }
    const int L = m->layers;
    return gemm<false, true, EPI_BIAS_F32>(m, m->H[L].p, m->Pb.p + m->woff[L], B, kOut, m->hidden, m->hidden, m->hidden,
                                           1, m->out.p, nullptr, kOut, m->P.p + m->boff[L]);
}

// dW (M x N, rows of N) = A^T H over the batch (A stored B x M, H stored B x N), split over the
// batch when it is large; the splits' partial products are summed in a fixed order
int weight_grad(rewl_mlp* m, const bf16* A, const bf16* H, int M, int N, int B, float* dst)
{
    const int splits = weight_splits(B);
    int rc;
    if ((rc = gemm<true, false, EPI_F32>(m, A, H, M, N, B, M, N, splits, splits > 1 ? m->Part.p : dst, nullptr, N, nullptr)))
        return rc;
    if (splits > 1) {
        const size_t n = (size_t)M * N;
        k_sum_parts<<<(unsigned)((n + 255) / 256), 256, 0, m->stream>>>(m->Part.p, splits, n, n, dst);
        m->launches++;
        MCUDA(cudaGetLastError());
    }
    return REWL_OK;
}

// db (N) = column sums of G (B x N): per-chunk partials, then their ordered sum
int bias_grad(rewl_mlp* m, const bf16* G, int B, int N, float* dst)
{
    const int chunks = (B + kColChunk - 1) / kColChunk;
    k_colsum<<<dim3((N + 127) / 128, chunks), 128, 0, m->stream>>>(G, B, N, m->Part.p);
    k_sum_parts<<<(unsigned)((N + 255) / 256), 256, 0, m->stream>>>(m->Part.p, chunks, (size_t)N, (size_t)N, dst);
    m->launches += 2;
    MCUDA(cudaGetLastError());
    return REWL_OK;
}

// backward of the mean squared error on m->yb; every gradient entry is written once into Gr
// (zeroed here, so that padding entries stay zero)
int backward(rewl_mlp* m, int B)
{
    MCUDA(cudaMemsetAsync(m->Gr.p, 0, m->nparams * sizeof(float), m->stream));
    k_loss_grad<<<(B + 127) / 128, 128, 0, m->stream>>>(m->out.p, m->yb.p, B, m->dOut.p, m->lossrow.p);
    k_loss_sum<<<1, 256, 0, m->stream>>>(m->lossrow.p, B, m->loss.p);
    m->launches += 2;
    const int L = m->layers;
    int rc;
    // output layer: dW = dOut^T H_L, db = colsum(dOut), dH = dOut W
    if ((rc = weight_grad(m, m->dOut.p, m->H[L].p, kOut, m->hidden, B, m->Gr.p + m->woff[L])) ||
        (rc = bias_grad(m, m->dOut.p, B, kOut, m->Gr.p + m->boff[L])))
        return rc;
    if ((rc = gemm<false, false, EPI_BF16>(m, m->dOut.p, m->Pb.p + m->woff[L], B, m->hidden, kOut, kOut, m->hidden, 1,
                                           nullptr, m->dH.p, m->hidden, nullptr)))
        return rc;
    for (int l = L - 1; l >= 0; --l) {
        const size_t n = (size_t)B * m->hidden;
        k_gelu_back<<<(unsigned)((n + 255) / 256), 256, 0, m->stream>>>(m->dH.p, m->Z[l].p, m->G.p, n);
        m->launches++;
        if ((rc = weight_grad(m, m->G.p, m->H[l].p, m->dout[l], m->din[l], B, m->Gr.p + m->woff[l])) ||
            (rc = bias_grad(m, m->G.p, B, m->dout[l], m->Gr.p + m->boff[l])))
            return rc;
        if (l > 0)
            if ((rc = gemm<false, false, EPI_BF16>(m, m->G.p, m->Pb.p + m->woff[l], B, m->din[l], m->dout[l], m->dout[l],
                                                   m->din[l], 1, nullptr, m->dH.p, m->din[l], nullptr)))
                return rc;
    }
    return REWL_OK;
}

uint64_t splitmix(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int upload_features(rewl_mlp* m, const float* X, int n, int in_dim, bf16* dst)
{
    std::vector<bf16> h((size_t)n * kIn, __float2bfloat16(0.f));
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < in_dim; ++c) h[(size_t)i * kIn + c] = __float2bfloat16(X[(size_t)i * in_dim + c]);
    MCUDA(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(bf16), cudaMemcpyHostToDevice, m->stream));
    MCUDA(cudaStreamSynchronize(m->stream));
    return REWL_OK;
}

} // namespace

extern "C" {

const char* rewl_mlp_last_error_string(void) { return g_mlp_error.c_str(); }

int rewl_mlp_create(int32_t device, int32_t hidden, int32_t layers, uint64_t seed, rewl_mlp** out)
{
    if (!out || hidden <= 0 || hidden % 64 || layers < 1 || layers > 16) return mfail(REWL_EINVAL, "hidden must be a positive multiple of 64, layers in 1..16");
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return mfail(REWL_EDEVICE, "cannot open device %d", device);
    rewl_mlp* m = new rewl_mlp();
    m->device = device; m->hidden = hidden; m->layers = layers; m->seed = seed;
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) { delete m; return mfail(REWL_EDEVICE, "stream"); }
    if (prepare_tc_kernels() != cudaSuccess) { m->release(); delete m; return mfail(REWL_EDEVICE, "tensor-core GEMM setup failed"); }
    for (int l = 0; l <= layers; ++l) {
        m->din.push_back(l == 0 ? kIn : hidden);
        m->dout.push_back(l == layers ? kOut : hidden);
    }
    size_t off = 0;
    for (int l = 0; l <= layers; ++l) {
        m->woff.push_back(off); off += (size_t)m->dout[l] * m->din[l];
        m->boff.push_back(off); off += (size_t)m->dout[l];
        off = (off + 7) & ~size_t(7);               // keep every weight block 16-byte aligned in bf16
    }
    m->nparams = off;
    int rc;
    if ((rc = m->P.alloc(off)) || (rc = m->Mm.alloc(off)) || (rc = m->Vm.alloc(off)) || (rc = m->Gr.alloc(off)) ||
        (rc = m->Mask.alloc(off)) || (rc = m->Pb.alloc(off)) || (rc = m->loss.alloc(1))) {
        m->release(); delete m; return rc;
    }
    // PyTorch-style uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) init over the real (unpadded) entries
    std::vector<float> p(off, 0.f), mask(off, 0.f);
    uint64_t s = seed;
    for (int l = 0; l <= layers; ++l) {
        const int fan_in = l == 0 ? 7 : hidden;
        const int real_in = l == 0 ? 7 : hidden;
        const int real_out = l == layers ? 1 : hidden;
        const float bound = 1.0f / std::sqrt((float)fan_in);
        for (int o = 0; o < m->dout[l]; ++o)
            for (int i = 0; i < m->din[l]; ++i) {
                const bool real = o < real_out && i < real_in;
                const size_t k = m->woff[l] + (size_t)o * m->din[l] + i;
                mask[k] = real ? 1.f : 0.f;
                p[k] = real ? bound * (2.0f * (float)((splitmix(s) >> 11) * (1.0 / 9007199254740992.0)) - 1.0f) : 0.f;
            }
        for (int o = 0; o < m->dout[l]; ++o) {
            const size_t k = m->boff[l] + o;
            const bool real = o < real_out;
            mask[k] = real ? 1.f : 0.f;
            p[k] = real ? bound * (2.0f * (float)((splitmix(s) >> 11) * (1.0 / 9007199254740992.0)) - 1.0f) : 0.f;
        }
    }
    std::vector<bf16> pb(off);
    for (size_t k = 0; k < off; ++k) pb[k] = __float2bfloat16(p[k]);
    if (cudaMemcpy(m->P.p, p.data(), off * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->Mask.p, mask.data(), off * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->Pb.p, pb.data(), off * 2, cudaMemcpyHostToDevice) != cudaSuccess) {
        m->release(); delete m; return mfail(REWL_EDEVICE, "parameter upload failed");
    }
    *out = m;
    return REWL_OK;
}

int rewl_mlp_destroy(rewl_mlp* m)
{
    if (!m) return REWL_OK;
    cudaSetDevice(m->device);
    m->release();
    delete m;
    return REWL_OK;
}

int rewl_mlp_num_params(const rewl_mlp* m, int64_t* n)
{
    if (!m || !n) return mfail(REWL_EINVAL, "null argument");
    *n = (int64_t)m->nparams;
    return REWL_OK;
}

// parameter vector in the engine's padded layout (fp32 masters); `which` 0 = params, 1 = grads
int rewl_mlp_get_params(rewl_mlp* m, int32_t which, float* out, int64_t n)
{
    if (!m || !out || n < (int64_t)m->nparams) return mfail(REWL_EINVAL, "bad arguments");
    cudaSetDevice(m->device);
    MCUDA(cudaStreamSynchronize(m->stream));
    MCUDA(cudaMemcpy(out, which ? m->Gr.p : m->P.p, m->nparams * 4, cudaMemcpyDeviceToHost));
    return REWL_OK;
}

int rewl_mlp_set_params(rewl_mlp* m, const float* in, int64_t n)
{
    if (!m || !in || n < (int64_t)m->nparams) return mfail(REWL_EINVAL, "bad arguments");
    cudaSetDevice(m->device);
    std::vector<bf16> pb(m->nparams);
    for (size_t k = 0; k < m->nparams; ++k) pb[k] = __float2bfloat16(in[k]);
    MCUDA(cudaMemcpy(m->P.p, in, m->nparams * 4, cudaMemcpyHostToDevice));
    MCUDA(cudaMemcpy(m->Pb.p, pb.data(), m->nparams * 2, cudaMemcpyHostToDevice));
    return REWL_OK;
}

// layer geometry: din, dout, weight offset, bias offset per layer (layers + 1 rows of 4)
int rewl_mlp_layout(const rewl_mlp* m, int64_t* out, int32_t cap_rows)
{
    if (!m || !out || cap_rows < m->layers + 1) return mfail(REWL_EINVAL, "bad arguments");
    for (int l = 0; l <= m->layers; ++l) {
        out[4 * l] = m->din[l]; out[4 * l + 1] = m->dout[l];
        out[4 * l + 2] = (int64_t)m->woff[l]; out[4 * l + 3] = (int64_t)m->boff[l];
    }
    return REWL_OK;
}

int rewl_mlp_predict(rewl_mlp* m, const float* X, int32_t n, int32_t in_dim, float* y)
{
    if (!m || !X || !y || n < 1 || in_dim < 1 || in_dim > kIn) return mfail(REWL_EINVAL, "bad arguments");
    cudaSetDevice(m->device);
    const int Bp = (n + kBM - 1) / kBM * kBM;
    int rc = ensure_batch(m, Bp);
    if (rc) return rc;
    MCUDA(cudaMemsetAsync(m->H[0].p, 0, (size_t)Bp * kIn * sizeof(bf16), m->stream));
    if ((rc = upload_features(m, X, n, in_dim, m->H[0].p))) return rc;
    if ((rc = forward(m, Bp))) return rc;
    std::vector<float> o((size_t)Bp * kOut);
    MCUDA(cudaMemcpyAsync(o.data(), m->out.p, o.size() * 4, cudaMemcpyDeviceToHost, m->stream));
    MCUDA(cudaStreamSynchronize(m->stream));
    if ((rc = take_tc_error())) return rc;
    for (int i = 0; i < n; ++i) y[i] = o[(size_t)i * kOut];
    return REWL_OK;
}

// One forward + backward on the given rows (no update); gradients readable with
// rewl_mlp_get_params(which = 1); returns the loss.
int rewl_mlp_gradient(rewl_mlp* m, const float* X, const float* y, int32_t n, int32_t in_dim, float* loss)
{
    if (!m || !X || !y || n < 1 || n % kBM || in_dim < 1 || in_dim > kIn) return mfail(REWL_EINVAL, "n must be a multiple of 64");
    cudaSetDevice(m->device);
    int rc = ensure_batch(m, n);
    if (rc) return rc;
    if ((rc = upload_features(m, X, n, in_dim, m->H[0].p))) return rc;
    MCUDA(cudaMemcpyAsync(m->yb.p, y, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream));
    if ((rc = forward(m, n)) || (rc = backward(m, n))) return rc;
    MCUDA(cudaMemcpyAsync(loss, m->loss.p, 4, cudaMemcpyDeviceToHost, m->stream));
    MCUDA(cudaStreamSynchronize(m->stream));
    return take_tc_error();
}

// Load a training set (features n x in_dim, targets n) into device memory.
int rewl_mlp_set_data(rewl_mlp* m, const float* X, const float* y, int32_t n, int32_t in_dim)
{
    if (!m || !X || !y || n < 1 || in_dim < 1 || in_dim > kIn) return mfail(REWL_EINVAL, "bad arguments");
    cudaSetDevice(m->device);
    m->Xall.release(); m->yall.release();
    int rc;
    if ((rc = m->Xall.alloc((size_t)n * kIn)) || (rc = m->yall.alloc(n))) return rc;
    if ((rc = upload_features(m, X, n, in_dim, m->Xall.p))) return rc;
    MCUDA(cudaMemcpy(m->yall.p, y, (size_t)n * 4, cudaMemcpyHostToDevice));
    m->nall = n;
    return REWL_OK;
}

// `steps` Adam steps on batches of `batch` rows drawn (Philox) from the loaded set.
// losses (may be NULL) receives the loss of every step.
int rewl_mlp_train(rewl_mlp* m, int32_t steps, int32_t batch, float lr, float* losses)
{
    if (!m || steps < 0 || batch < 64 || batch % kBM || !(lr > 0)) return mfail(REWL_EINVAL, "bad arguments");
    if (m->nall < 1) return mfail(REWL_ESTATE, "no training data (rewl_mlp_set_data)");
    if (steps == 0) return REWL_OK;
    cudaSetDevice(m->device);
    int rc = ensure_batch(m, batch);
    if (rc) return rc;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    // the call's bias corrections and its losses live on the device; the cursor starts at the
    // network's step
    if (m->ctab.n < (size_t)2 * steps) {
        m->ctab.release(); m->lossv.release();
        if ((rc = m->ctab.alloc((size_t)2 * steps)) || (rc = m->lossv.alloc((size_t)steps))) return rc;
    }
    if (!m->cursor.p && (rc = m->cursor.alloc(1))) return rc;
    std::vector<float> ct((size_t)2 * steps);
    for (int s = 0; s < steps; ++s) {
        const float t = (float)(m->step + s + 1);
        ct[2 * s] = 1.f - std::pow(b1, t);
        ct[2 * s + 1] = 1.f - std::pow(b2, t);
    }
    const TrainCursor c0{(unsigned long long)m->step, 0, 0};
    MCUDA(cudaMemcpyAsync(m->ctab.p, ct.data(), ct.size() * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(cudaMemcpyAsync(m->cursor.p, &c0, sizeof c0, cudaMemcpyHostToDevice, m->stream));
    MCUDA(cudaStreamSynchronize(m->stream));       // the host copies above leave scope

    // one step: sample the batch, forward, backward, Adam, keep the loss and advance; captured as
    // a CUDA graph and replayed `steps` times (about 30 launches a step, launch-bound otherwise)
    const int64_t l0 = m->launches;
    auto enqueue_step = [&]() -> int {
        k_gather<<<(batch + 127) / 128, 128, 0, m->stream>>>(m->Xall.p, m->yall.p, m->nall, m->H[0].p, m->yb.p, batch,
                                                             m->seed, m->cursor.p);
        m->launches++;
        int r;
        if ((r = forward(m, batch)) || (r = backward(m, batch))) return r;
        k_adam<<<(unsigned)((m->nparams + 255) / 256), 256, 0, m->stream>>>(m->P.p, m->Mm.p, m->Vm.p, m->Gr.p, m->Mask.p,
                                                                            m->Pb.p, m->nparams, lr, b1, b2, eps,
                                                                            m->ctab.p, m->cursor.p);
        k_train_advance<<<1, 1, 0, m->stream>>>(m->cursor.p, m->loss.p, m->lossv.p);
        m->launches += 2;
        MCUDA(cudaGetLastError());
        return REWL_OK;
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    MCUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeRelaxed));
    rc = enqueue_step();
    const cudaError_t ce = cudaStreamEndCapture(m->stream, &graph);
    if (rc == REWL_OK && ce != cudaSuccess) rc = mfail(REWL_EDEVICE, "capturing a training step: %s", cudaGetErrorString(ce));
    if (rc == REWL_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
        rc = mfail(REWL_EDEVICE, "instantiating the training-step graph failed");
    if (graph) cudaGraphDestroy(graph);
    const int64_t per_step = m->launches - l0;
    for (int s = 0; s < steps && rc == REWL_OK; ++s)
        if (cudaGraphLaunch(exec, m->stream) != cudaSuccess) rc = mfail(REWL_EDEVICE, "training-step graph launch failed");
    const cudaError_t se = cudaStreamSynchronize(m->stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (rc) return rc;
    if (se != cudaSuccess) return mfail(REWL_EDEVICE, "training: %s", cudaGetErrorString(se));
    m->launches += per_step * (steps - 1);     // the capture counted one step
    m->step += steps;
    if ((rc = take_tc_error())) return rc;
    if (losses) MCUDA(cudaMemcpy(losses, m->lossv.p, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost));
    return REWL_OK;
}

int rewl_mlp_launches(const rewl_mlp* m, int64_t* n)
{
    if (!m || !n) return mfail(REWL_EINVAL, "null argument");
    *n = m->launches;
    return REWL_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free prediction (rewl_mlp_predict_noalloc).
//
// rewl_mlp_predict grows its activation buffers with cudaMalloc when a larger
// batch arrives and stages inputs through host memory.  Some callers cannot do
// that: a host program whose own allocator already holds the device's memory, a
// loop running at its device-memory limit, or a driver loop that must not stall,
// since cudaMalloc may synchronise the device.  They use this variant instead:
// inputs and outputs are device pointers owned by the caller, and the activations
// live in one file-scope static device array.  Its address is looked up once per
// device (cudaGetSymbolAddress with that device current) on the first call, so
// make that first call before any stream capture.
//
// Limits: at most kNoAllocMaxRows rows per call and hidden width at most
// kNoAllocMaxHidden (9.5 MiB of scratch); larger requests fail with REWL_EINVAL.
// Nothing in the scratch has to start at zero: every call writes each element
// it later reads (the staging kernel writes the zero padding too).  The scratch
// is shared by every network on a device, so calls that may overlap -- on
// different streams, or from different host threads -- race on it and must be
// ordered by the caller (for example, issue them on one stream).
//
// The call never waits for the GPU, so a GEMM whose bounded wait ran out cannot
// be reported by its return code: the last kernel then writes NaN to every y
// instead of the stale scratch, for as long as the timeout flag stands (it is
// reported and cleared by the next rewl_mlp_* call that synchronises).
// ---------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxRows = 4096;
constexpr int kNoAllocMaxHidden = 256;
constexpr int kNoAllocMaxDevices = 64;
constexpr size_t kNaIn = (size_t)kNoAllocMaxRows * kIn * sizeof(bf16);                   // padded inputs
constexpr size_t kNaH = (size_t)kNoAllocMaxRows * kNoAllocMaxHidden * sizeof(bf16);      // activations (x2)
constexpr size_t kNaZ = (size_t)kNoAllocMaxRows * kNoAllocMaxHidden * sizeof(float);     // pre-activations
constexpr size_t kNaOut = (size_t)kNoAllocMaxRows * kOut * sizeof(float);                // padded outputs
constexpr size_t kNoAllocBytes = kNaIn + 2 * kNaH + kNaZ + kNaOut;
static_assert(kNaIn % 256 == 0 && kNaH % 256 == 0 && kNaZ % 256 == 0, "sub-buffers stay 256-byte aligned");

} // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Address of the static scratch on `device` (which must be current).
int noalloc_scratch(int device, unsigned char** out)
{
    if (device < 0 || device >= kNoAllocMaxDevices) return mfail(REWL_EINVAL, "device %d out of range", device);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return mfail(REWL_EDEVICE, "cudaGetSymbolAddress(scratch) on device %d: %s", device, cudaGetErrorString(e));
        g_noalloc_ptr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_ptr[device];
    return REWL_OK;
}

// rows x kIn bf16 inputs, zero beyond n rows and in_dim columns
__global__ void k_noalloc_stage(const float* X, int n, int in_dim, int rows, bf16* H0)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)rows * kIn) return;
    const int r = (int)(i / kIn), c = (int)(i % kIn);
    H0[i] = __float2bfloat16(r < n && c < in_dim ? X[(size_t)r * in_dim + c] : 0.f);
}

__global__ void k_noalloc_take(const float* out, int n, float* y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool timed_out = *reinterpret_cast<const volatile int*>(&g_tc_error) != 0;
    if (i < n) y[i] = timed_out ? __int_as_float(0x7FC00000) : out[(size_t)i * kOut];
}

template <int EPI>
cudaError_t noalloc_layer(cudaStream_t st, const bf16* A, const bf16* W, int M, int N, int K, float* Cf, bf16* Cb,
                          const float* bias)
{
    const GemmArgs g{A, W, M, N, K, K, K, K, Cf, Cb, N, bias};
    return launch_gemm<false, true, EPI>(st, g, 1);
}

int predict_noalloc_on_device(rewl_mlp* m, const float* X, int32_t n, int32_t in_dim, float* y, void* stream);

} // namespace

extern "C" int rewl_mlp_predict_noalloc(rewl_mlp* m, const float* X, int32_t n, int32_t in_dim, float* y, void* stream)
{
    if (!m || !X || !y || n < 1 || in_dim < 1 || in_dim > kIn) return mfail(REWL_EINVAL, "bad arguments");
    if (n > kNoAllocMaxRows)
        return mfail(REWL_EINVAL, "rewl_mlp_predict_noalloc: %d rows exceed the static scratch limit of %d rows per call",
                     n, kNoAllocMaxRows);
    if (m->hidden > kNoAllocMaxHidden)
        return mfail(REWL_EINVAL, "rewl_mlp_predict_noalloc: hidden width %d exceeds the static scratch limit of %d",
                     m->hidden, kNoAllocMaxHidden);
    int caller_device = 0;
    MCUDA(cudaGetDevice(&caller_device));
    MCUDA(cudaSetDevice(m->device));
    const int rc = predict_noalloc_on_device(m, X, n, in_dim, y, stream);
    // leave the caller's current device as it was, whatever happened
    const cudaError_t back = cudaSetDevice(caller_device);
    if (rc) return rc;
    if (back != cudaSuccess) return mfail(REWL_EDEVICE, "restoring the current device: %s", cudaGetErrorString(back));
    return REWL_OK;
}

namespace {
int predict_noalloc_on_device(rewl_mlp* m, const float* X, int32_t n, int32_t in_dim, float* y, void* stream)
{
    unsigned char* s = nullptr;
    int rc = noalloc_scratch(m->device, &s);
    if (rc) return rc;
    bf16* H0 = reinterpret_cast<bf16*>(s);
    bf16* Ha = reinterpret_cast<bf16*>(s + kNaIn);
    bf16* Hb = reinterpret_cast<bf16*>(s + kNaIn + kNaH);
    float* Z = reinterpret_cast<float*>(s + kNaIn + 2 * kNaH);
    float* out = reinterpret_cast<float*>(s + kNaIn + 2 * kNaH + kNaZ);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int rows = (n + kBM - 1) / kBM * kBM;

    k_noalloc_stage<<<(unsigned)(((size_t)rows * kIn + 255) / 256), 256, 0, st>>>(X, n, in_dim, rows, H0);
    MCUDA(cudaGetLastError());
    const bf16* cur = H0;
    for (int l = 0; l < m->layers; ++l) {
        bf16* nxt = (l & 1) ? Hb : Ha;
        MCUDA(noalloc_layer<EPI_BIAS_GELU>(st, cur, m->Pb.p + m->woff[l], rows, m->dout[l], m->din[l], Z, nxt,
                                           m->P.p + m->boff[l]));
        cur = nxt;
    }
    const int L = m->layers;
    MCUDA(noalloc_layer<EPI_BIAS_F32>(st, cur, m->Pb.p + m->woff[L], rows, kOut, m->hidden, out, nullptr,
                                      m->P.p + m->boff[L]));
    k_noalloc_take<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, y);
    MCUDA(cudaGetLastError());
    m->launches += L + 3;
    return REWL_OK;
}
} // namespace
