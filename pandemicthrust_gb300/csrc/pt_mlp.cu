// pt_mlp.cu - the surrogate's multilayer perceptron: BF16 weights and activations,
// FP32 accumulation, FP32 master weights and Adam, all in hand-written kernels.
//
// Layers l = 0..L-1 map width[l] -> width[l+1]; hidden layers apply GELU, the last
// is linear.  Parameters live in one FP32 array, layer by layer: W_l (width[l+1] x
// width[l], row-major) then b_l (width[l+1]); a BF16 copy of every weight feeds the
// tensor cores.  The library owns all device memory; callers pass host arrays.
//
// Training GEMMs are small (a minibatch of a few hundred rows by 256) and need
// transposed operands, so they run on the warp-level tensor-core instruction mma.sync
// m16n8k16 (BF16 in, FP32 accumulate): one kernel with strided operands serves the
// forward product X W^T, the data gradient dZ W and the weight gradient dZ^T X.
// Inference over large batches runs every layer on tcgen05.mma (k_umma_layer below).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "pandemic_gb300.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kTile = 64;   // block tile (M and N)
constexpr int kTileK = 16;  // reduction step (one mma k-step)

enum { kStoreF32 = 0, kForward = 1, kBackward = 2 };

// C(i, j) = sum_r A(i, r) B(r, j) with A(i, r) = A[i*sa_i + r*sa_r] and
// B(r, j) = B[r*sb_r + j*sb_j]; M x N outputs, R terms; any sizes (tiles zero-fill).
struct GemmArgs {
    const bf16 *A;
    long long sa_i, sa_r;
    const bf16 *B;
    long long sb_r, sb_j;
    int M, N, R;
    int mode;
    // kStoreF32: C[i*ldc + j] = acc
    float *C;
    long long ldc;
    // kForward: z = acc + bias[j]; Z = z (FP32), H = act(z) (BF16); act = GELU if gelu
    const float *bias;
    float *Z;
    bf16 *H;
    int gelu;
    // kBackward: dz = acc * GELU'(Zprev); dZf = dz (FP32), dZb = dz (BF16)
    const float *Zprev;
    float *dZf;
    bf16 *dZb;
};

// The activation: GELU in its tanh form (Hendrycks and Gimpel, arXiv:1606.08415),
// 0.5 z (1 + tanh(u)), u = sqrt(2/pi) (z + 0.044715 z^3), with the hardware tanh
// (tanh.approx.f32).  Training and inference evaluate the same expression.
constexpr float kGeluC0 = 0.7978845608028654f;               // sqrt(2 / pi)
constexpr float kGeluC1 = 0.7978845608028654f * 0.044715f;   // sqrt(2 / pi) * 0.044715

__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// rounded step by step as the tcgen05 epilogue's paired form (gelu_bf16x2):
// w = c0 + c1 z^2, t = tanh(w z), h = z / 2, h + h t
__device__ __forceinline__ float gelu(float z)
{
    const float w = __fmaf_rn(__fmul_rn(z, z), kGeluC1, kGeluC0);
    const float t = tanh_approx(__fmul_rn(w, z));
    const float h = __fmul_rn(0.5f, z);
    return __fmaf_rn(h, t, h);
}

__device__ __forceinline__ float gelu_grad(float z)
{
    // d/dz [0.5 z (1 + t)] = 0.5 (1 + t) + 0.5 z (1 - t^2) du/dz, du/dz = c0 + 3 c1 z^2
    const float z2 = z * z;
    const float t = tanh_approx(z * (kGeluC0 + kGeluC1 * z2));
    return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * (kGeluC0 + 3.f * kGeluC1 * z2);
}

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// 128 threads: four warps, each a 32 x 32 part of the 64 x 64 block tile (2 x 4 mma
// tiles of 16 x 8).  Fragment layout of m16n8k16 (g = lane / 4, t = lane % 4):
// A rows g / g+8, columns 2t, 2t+1 / 2t+8, 2t+9; B rows 2t, 2t+1 / 2t+8, 2t+9, column g;
// C rows g / g+8, columns 2t, 2t+1.
__global__ void __launch_bounds__(128) k_gemm(GemmArgs g)
{
    __shared__ bf16 As[kTile][kTileK + 8];
    __shared__ bf16 Bs[kTileK][kTile + 8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gq = lane >> 2, tq = lane & 3;
    const int bm = blockIdx.y * kTile, bn = blockIdx.x * kTile;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[a][b][q] = 0.f;
    const bf16 zero = __float2bfloat16(0.f);
    for (int r0 = 0; r0 < g.R; r0 += kTileK) {
        // consecutive threads read consecutive addresses: the index with stride 1 varies fastest
        for (int e = threadIdx.x; e < kTile * kTileK; e += 128) {
            const bool r_fast = g.sa_r == 1;
            const int i = r_fast ? e / kTileK : e % kTile, r = r_fast ? e % kTileK : e / kTile;
            const int gi = bm + i, gr = r0 + r;
            As[i][r] = (gi < g.M && gr < g.R) ? g.A[gi * g.sa_i + gr * g.sa_r] : zero;
        }
        for (int e = threadIdx.x; e < kTileK * kTile; e += 128) {
            const bool j_fast = g.sb_j == 1;
            const int r = j_fast ? e / kTile : e % kTileK, j = j_fast ? e % kTile : e / kTileK;
            const int gr = r0 + r, gj = bn + j;
            Bs[r][j] = (gr < g.R && gj < g.N) ? g.B[gr * g.sb_r + gj * g.sb_j] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            const int row = wm + mt * 16;
            uint32_t a[4];
            a[0] = pack2(As[row + gq][2 * tq], As[row + gq][2 * tq + 1]);
            a[1] = pack2(As[row + gq + 8][2 * tq], As[row + gq + 8][2 * tq + 1]);
            a[2] = pack2(As[row + gq][2 * tq + 8], As[row + gq][2 * tq + 9]);
            a[3] = pack2(As[row + gq + 8][2 * tq + 8], As[row + gq + 8][2 * tq + 9]);
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const int col = wn + nt * 8;
                uint32_t b[2];
                b[0] = pack2(Bs[2 * tq][col + gq], Bs[2 * tq + 1][col + gq]);
                b[1] = pack2(Bs[2 * tq + 8][col + gq], Bs[2 * tq + 9][col + gq]);
                mma_bf16(acc[mt][nt], a, b);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int i = bm + wm + mt * 16 + gq + (q >= 2 ? 8 : 0);
                const int j = bn + wn + nt * 8 + 2 * tq + (q & 1);
                if (i >= g.M || j >= g.N) continue;
                const float v = acc[mt][nt][q];
                const long long o = (long long)i * g.N + j;
                if (g.mode == kStoreF32) {
                    g.C[(long long)i * g.ldc + j] = v;
                } else if (g.mode == kForward) {
                    const float z = v + g.bias[j];
                    g.Z[o] = z;
                    g.H[o] = __float2bfloat16(g.gelu ? gelu(z) : z);
                } else {
                    const float dz = v * gelu_grad(g.Zprev[o]);
                    g.dZf[o] = dz;
                    g.dZb[o] = __float2bfloat16(dz);
                }
            }
}

// ---------------------------------------------------------------- tcgen05 inference
// Forward layers for inference on the fifth-generation tensor cores.  One persistent
// CTA per SM, in three roles:
//   warp 0 (one lane), the producer: loads the layer's weights (Np x Kp BF16, at most
//     256 x 256 = 128 KB) once, then streams 128-row tiles of the input through a ring
//     of kUmmaStages shared-memory stages (up to 128 K columns each) with TMA
//     (cp.async.bulk.tensor), each stage completing on its `full` mbarrier;
//   warp 1 (one lane), the MMA issuer: per tile it waits for a free accumulator (two
//     128 x 256 FP32 accumulators in tensor memory, all 512 columns), then per stage
//     waits for `full`, issues tcgen05.mma (kind::f16, K = 16 each) and commits the
//     stage back to the producer (`empty`); the tile's last commit goes to the
//     epilogue (`acc_full`);
//   the epilogue warps: read the accumulator with tcgen05.ld.32x32b (warp w reads
//     lanes, i.e. tile rows, 32 (w % 4) .. + 31), add the bias, apply GELU, store,
//     and release the accumulator (`acc_empty`).
// So the fill of tile i + 1, its MMAs and the epilogue of tile i overlap.  Every wait
// is bounded: one that gives up sets the error word and a shared flag that ends every
// role's loop; the MMA issuer then waits (bounded) for its last MMAs and the producer
// for its last copies before the tensor memory is freed.
//
// Shared-memory operand layouts (K-major), each written by TMA boxes as they land:
//  * 128-byte swizzle, when K is a multiple of 64: a box is 64 columns (128 bytes) x R
//    rows, row r at byte 128 r of its block with its eight 16-byte pieces permuted by
//    r % 8 (the TMA's SWIZZLE_128B); blocks of 64 columns follow each other at 128 R
//    bytes.  Descriptor: stride byte offset 1024 (eight rows), swizzle mode 128-byte;
//    the MMA over K columns [16 s, 16 s + 16) starts at block s / 4, byte 32 (s % 4).
//  * no swizzle, otherwise: a box is 8 columns (16 bytes) x R rows, so the 8-row x
//    16-byte core matrix (row group g, K group c) sits at byte (c R / 8 + g) * 128.
//    The K-direction core stride (leading byte offset) is 16 R bytes, the row-group
//    stride (stride byte offset) 128 bytes; the MMA over K columns [16 s, 16 s + 16)
//    starts at byte 32 R s.
// Wide boxes matter: a 16-byte box row is one request that moves a 32-byte sector.
constexpr int kUmmaM = 128;                    // rows per tile (the MMA's M)
constexpr int kUmmaStages = 3;                 // input stages in the ring
constexpr int kUmmaKS = 128;                   // K columns per stage at most
constexpr int kUmmaMaxN = 256, kUmmaMaxK = 256;
constexpr int kUmmaStageBytes = kUmmaM * kUmmaKS * 2;
constexpr int kUmmaBarBytes = 1024, kUmmaBiasBytes = 4 * kUmmaMaxN;
constexpr int kUmmaSmem = kUmmaBarBytes + kUmmaBiasBytes + kUmmaMaxN * kUmmaMaxK * 2 + kUmmaStages * kUmmaStageBytes;
constexpr int kUmmaEpiWarps = 8;               // epilogue warps: two per lane quarter
constexpr long long kUmmaSpin = 1ll << 22;     // polls of an mbarrier before a wait gives up
static_assert(kUmmaSmem <= 227 * 1024, "the tcgen05 layer needs more shared memory than a CTA has");

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// two FP32 lanes in one 64-bit register, for the paired FP32 instructions (f32x2)
__device__ __forceinline__ uint64_t f2(float lo, float hi)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__device__ __forceinline__ void f2_split(uint64_t x, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(x));
}

__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b)
{
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b)
{
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// BF16 pair, lo in the low half (round to nearest even)
__device__ __forceinline__ uint32_t bf16x2(float lo, float hi)
{
    uint32_t d;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

// GELU (the tanh form above) of a pair of pre-activations, packed to BF16: four
// paired FP32 instructions and two tanh per pair
__device__ __forceinline__ uint32_t gelu_bf16x2(uint64_t z)
{
    const uint64_t w = f2_fma(f2_mul(z, z), f2(kGeluC1, kGeluC1), f2(kGeluC0, kGeluC0));   // c0 + c1 z^2
    float u0, u1;
    f2_split(f2_mul(w, z), u0, u1);
    const uint64_t h = f2_mul(z, f2(0.5f, 0.5f));
    float r0, r1;
    f2_split(f2_fma(h, f2(tanh_approx(u0), tanh_approx(u1)), h), r0, r1);   // h (1 + t)
    return bf16x2(r0, r1);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Waits for the phase of the given parity to complete; false when it gives up after
// kUmmaSpin polls or when another role has raised `fail` (if given).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, const volatile int *fail)
{
    for (long long i = 0; i < kUmmaSpin; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (fail && (i & 63) == 63 && *fail) return false;
    }
    return false;
}

__device__ __forceinline__ void umma_fail(volatile int *fail, int *error)
{
    *fail = 1;
    atomicExch(error, 1);
}

// TMA: the box at element coordinates (x, y) of the map into shared memory at dst,
// completing on the mbarrier
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t ad, uint64_t bd, uint32_t idesc, bool accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(ad), "l"(bd), "r"(idesc), "r"((uint32_t)accumulate));
}

// the mbarrier completes when every tcgen05.mma this thread issued before has completed
__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// tcgen05 shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte offset
// >> 4 (16-29), stride byte offset >> 4 (32-45), the fixed 0b001 (46-48), base offset 0
// (49-51, the operands are 1024-byte aligned), the swizzle mode (61-63: 0 none,
// 2 128-byte).
constexpr uint32_t kSwizzleNone = 0, kSwizzle128B = 2;
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo, uint32_t swizzle)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | ((uint64_t)swizzle << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 (17-22), M >> 4 (24-28).
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// tcgen05.ld of 32 consecutive accumulator columns of the warp's 32 lanes (one row a
// thread).  The registers are written asynchronously: read them only after
// tmem_ld_wait on the same array.
__device__ __forceinline__ void tmem_ld32_issue(uint32_t taddr, uint32_t v[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}

// Waits for the warp's tcgen05.ld; the array is an operand so that no use of it is
// moved above the wait.
__device__ __forceinline__ void tmem_ld_wait(uint32_t v[32])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                   "+r"(v[15]), "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]),
                   "+r"(v[22]), "+r"(v[23]), "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]),
                   "+r"(v[29]), "+r"(v[30]), "+r"(v[31])
                 :
                 : "memory");
}

// The epilogue of one 32-column chunk of a tile row (v: its accumulator values): bias,
// GELU and BF16 stores for hidden layers (H), the accumulating FP32 stores for the last.
__device__ __forceinline__ void epilogue_chunk(const uint32_t v[32], int c0, long long row, const float *s_bias,
                                               int N, int gelu, bf16 *H, long long ldh, float *Y, long long ldy,
                                               float scale, int first, int vec)
{
    if (H) {
        const float4 *bq = reinterpret_cast<const float4 *>(s_bias + c0);
        uint32_t packed[16];
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
            const float4 bb = bq[j / 4];
            const uint64_t z01 = f2_add(f2(__uint_as_float(v[j]), __uint_as_float(v[j + 1])), f2(bb.x, bb.y));
            const uint64_t z23 = f2_add(f2(__uint_as_float(v[j + 2]), __uint_as_float(v[j + 3])), f2(bb.z, bb.w));
            if (gelu) {
                packed[j / 2] = gelu_bf16x2(z01);
                packed[j / 2 + 1] = gelu_bf16x2(z23);
            } else {
                float a0, a1, a2, a3;
                f2_split(z01, a0, a1);
                f2_split(z23, a2, a3);
                packed[j / 2] = bf16x2(a0, a1);
                packed[j / 2 + 1] = bf16x2(a2, a3);
            }
        }
        // N is a multiple of 32 for hidden layers: two 32-byte stores, whole sectors
        bf16 *dst = H + row * ldh + c0;
#pragma unroll
        for (int k = 0; k < 2; k++)
            asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(dst + 16 * k),
                         "r"(packed[8 * k]), "r"(packed[8 * k + 1]), "r"(packed[8 * k + 2]), "r"(packed[8 * k + 3]),
                         "r"(packed[8 * k + 4]), "r"(packed[8 * k + 5]), "r"(packed[8 * k + 6]),
                         "r"(packed[8 * k + 7])
                         : "memory");
        return;
    }
    float *dst = Y + row * ldy + c0;
    if (vec) {
        // the four 32-byte runs of the accumulator are loaded together
        float o[32];
        if (!first)
#pragma unroll
            for (int k = 0; k < 4; k++)
                asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                             : "=f"(o[8 * k]), "=f"(o[8 * k + 1]), "=f"(o[8 * k + 2]), "=f"(o[8 * k + 3]),
                               "=f"(o[8 * k + 4]), "=f"(o[8 * k + 5]), "=f"(o[8 * k + 6]), "=f"(o[8 * k + 7])
                             : "l"(dst + 8 * k));
#pragma unroll
        for (int i = 0; i < 32; i++) {
            const float z = __uint_as_float(v[i]) + s_bias[c0 + i];
            o[i] = first ? scale * z : fmaf(scale, z, o[i]);
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(dst + 8 * k),
                         "f"(o[8 * k]), "f"(o[8 * k + 1]), "f"(o[8 * k + 2]), "f"(o[8 * k + 3]), "f"(o[8 * k + 4]),
                         "f"(o[8 * k + 5]), "f"(o[8 * k + 6]), "f"(o[8 * k + 7])
                         : "memory");
    } else {
#pragma unroll
        for (int j = 0; j < 32; j++) {
            const int c = c0 + j;
            if (c < N) {
                const float z = __uint_as_float(v[j]) + s_bias[c];
                dst[j] = first ? scale * z : fmaf(scale, z, dst[j]);
            }
        }
    }
}

// One layer: out = act(A W^T + bias) over M rows, EPI epilogue warps.  tmA: the input
// (M x Kp BF16), box bw x kUmmaM; tmW: the weights (Np x Kp BF16, zero rows past N),
// box bw x Np; bw = 64 with the 128-byte swizzle (sw, Kp a multiple of 64), else 8.
// Kp a multiple of 16, Np of 16, both <= 256.  Hidden layers (H set) store
// BF16 activations (row stride ldh, N a multiple of 32).  The last layer (Y set)
// accumulates its FP32 outputs z: Y = scale z (first) or Y + scale z, row stride ldy;
// with `vec` (ldy a multiple of 32, Y 32-byte aligned) in whole 32-byte sectors,
// columns from N to the next multiple of 32 included (padding).  error: set when a
// wait gives up.
template <int EPI>
__global__ void __launch_bounds__(32 * (2 + EPI), 1)
    k_umma_layer(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmW, int M, int Kp,
                 int Np, int N, int sw, const float *bias, int gelu, bf16 *H, long long ldh, float *Y, long long ldy,
                 float scale, int first, int vec, int *error)
{
    static_assert(EPI % 4 == 0, "each of the four lane quarters needs the same number of epilogue warps");
    extern __shared__ __align__(1024) uint8_t smem[];
    // barrier page: full[S], empty[S], acc_full[2], acc_empty[2], weights, drain;
    // then the tensor-memory address and the failure flag
    const uint32_t b_full = smem_u32(smem), b_empty = b_full + 8 * kUmmaStages, b_accf = b_empty + 8 * kUmmaStages,
                   b_acce = b_accf + 16, b_w = b_acce + 16, b_drain = b_w + 8;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 256);
    volatile int *fail = reinterpret_cast<volatile int *>(smem + 320);
    float *s_bias = reinterpret_cast<float *>(smem + kUmmaBarBytes);
    uint8_t *sW = smem + kUmmaBarBytes + kUmmaBiasBytes;
    const uint32_t sW_u = smem_u32(sW), sA_u = sW_u + kUmmaMaxN * kUmmaMaxK * 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        for (int i = 0; i < kUmmaStages; i++) {
            mbar_init(b_full + 8 * i, 1);
            mbar_init(b_empty + 8 * i, 1);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(b_accf + 8 * i, 1);
            mbar_init(b_acce + 8 * i, EPI);
        }
        mbar_init(b_w, 1);
        mbar_init(b_drain, 1);
        *fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    for (int c = threadIdx.x; c < kUmmaMaxN; c += blockDim.x) s_bias[c] = c < N ? bias[c] : 0.f;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    const int tiles = (M + kUmmaM - 1) / kUmmaM;
    const int bw = sw ? 64 : 8;   // K columns per TMA box
    // K columns per stage: all of K up to kUmmaKS, else about half, in whole boxes and MMA steps
    const int KS = Kp <= kUmmaKS ? Kp : (sw ? 64 * ((Kp / 64 + 1) / 2) : 16 * ((Kp / 16 + 1) / 2));
    const int nks = (Kp + KS - 1) / KS;                              // stages per tile: 1 or 2
    if (warp == 0) {
        if (lane == 0) {
            // producer
            mbar_expect_tx(b_w, (uint32_t)(Np * Kp * 2));
            for (int c = 0; c < Kp / bw; c++) tma_load_2d(sW_u + c * Np * bw * 2, &tmW, bw * c, 0, b_w);
            bool ok = true;
            int it = 0;   // stage fills issued
            for (int t = blockIdx.x; ok && t < tiles; t += gridDim.x)
                for (int ks = 0; ks < nks; ks++) {
                    const int s = it % kUmmaStages, use = it / kUmmaStages;
                    if (use > 0 && !mbar_wait(b_empty + 8 * s, (use - 1) & 1, fail)) {
                        ok = false;
                        break;
                    }
                    const int k0 = ks * KS, kc = min(KS, Kp - k0);
                    const uint32_t dst = sA_u + s * kUmmaStageBytes;
                    mbar_expect_tx(b_full + 8 * s, (uint32_t)(kUmmaM * kc * 2));
                    for (int c = 0; c < kc / bw; c++)
                        tma_load_2d(dst + c * kUmmaM * bw * 2, &tmA, k0 + bw * c, t * kUmmaM, b_full + 8 * s);
                    it++;
                }
            if (!ok) umma_fail(fail, error);
            // every copy lands before the CTA ends: the last fill of each stage, the weights
            for (int s = 0; s < kUmmaStages; s++) {
                const int uses = it / kUmmaStages + (s < it % kUmmaStages ? 1 : 0);
                if (uses > 0) mbar_wait(b_full + 8 * s, (uses - 1) & 1, nullptr);
            }
            mbar_wait(b_w, 0, nullptr);
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            bool ok = mbar_wait(b_w, 0, fail);
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t idesc = umma_idesc(kUmmaM, Np);
            int it = 0, tc = 0;
            for (int t = blockIdx.x; ok && t < tiles; t += gridDim.x, tc++) {
                const int b = tc & 1, use = tc >> 1;
                if (use > 0 && !mbar_wait(b_acce + 8 * b, (use - 1) & 1, fail)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t d = tmem + 256u * b;
                for (int ks = 0; ks < nks; ks++, it++) {
                    const int s = it % kUmmaStages, u = it / kUmmaStages;
                    if (!mbar_wait(b_full + 8 * s, u & 1, fail)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const int k0 = ks * KS, kc = min(KS, Kp - k0);
                    const uint32_t a0 = sA_u + s * kUmmaStageBytes;
                    for (int j = 0; j < kc / 16; j++) {
                        const int g = k0 / 16 + j;   // the MMA step within K
                        uint64_t ad, wd;
                        if (sw) {
                            ad = umma_desc(a0 + (j >> 2) * kUmmaM * 128 + 32 * (j & 3), 16, 1024, kSwizzle128B);
                            wd = umma_desc(sW_u + (g >> 2) * Np * 128 + 32 * (g & 3), 16, 1024, kSwizzle128B);
                        } else {
                            ad = umma_desc(a0 + j * 32 * kUmmaM, 16 * kUmmaM, 128, kSwizzleNone);
                            wd = umma_desc(sW_u + g * 32 * Np, 16 * Np, 128, kSwizzleNone);
                        }
                        umma_bf16(d, ad, wd, idesc, (ks | j) != 0);
                    }
                    umma_commit(b_empty + 8 * s);   // the stage is free once these MMAs complete
                }
                if (!ok) break;
                umma_commit(b_accf + 8 * b);
            }
            if (!ok) umma_fail(fail, error);
            // every MMA issued completes before the tensor memory is freed
            umma_commit(b_drain);
            mbar_wait(b_drain, 0, nullptr);
        }
        __syncwarp();
    } else {
        // epilogue: lanes (tile rows) 32 q .. 32 q + 31, 32-column chunks part, part + EPI / 4, ...
        const int q = warp & 3, part = (warp - 2) >> 2;
        constexpr int parts = EPI / 4;
        int tc = 0;
        for (int t = blockIdx.x; t < tiles; t += gridDim.x, tc++) {
            const int b = tc & 1, use = tc >> 1;
            if (!__all_sync(0xffffffffu, mbar_wait(b_accf + 8 * b, use & 1, fail))) {
                if (lane == 0) umma_fail(fail, error);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const int row = t * kUmmaM + 32 * q + lane;
            const uint32_t tb = tmem + ((uint32_t)(32 * q) << 16) + 256u * b;
            for (int c0 = 32 * part; c0 < Np; c0 += 32 * parts) {
                uint32_t v[32];
                __syncwarp();   // tcgen05.ld and its wait are warp-collective
                tmem_ld32_issue(tb + c0, v);
                tmem_ld_wait(v);
                if (row < M) epilogue_chunk(v, c0, row, s_bias, N, gelu, H, ldh, Y, ldy, scale, first, vec);
            }
            // the accumulator is free for the tile after next
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(b_acce + 8 * b);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

// ---------------------------------------------------------------- ensemble mean layer
// The members' last layers in one GEMM: y = inv * (sum_m W_m h_m + sum_m b_m), the
// mean of the members' outputs.  The members' last hidden activations h_m (M x Kh BF16
// each) are one operand concatenated along K, their weights W_m (Np x Kh) side by
// side in Wc (Np x members * Kh), so the tensor cores sum over members in the
// accumulator and the outputs are written once (instead of a read-modify-write of an
// FP32 accumulator per member).  Wc is too large for shared memory, so every stage of
// the ring carries a 64-column slice of both operands (128-byte swizzled boxes); the
// roles, accumulators, waits and epilogue are those of k_umma_layer.
constexpr int kMeanMaxMembers = 8;
constexpr int kMeanStages = 4;
constexpr int kMeanAStage = kUmmaM * 64 * 2;        // 16 KB
constexpr int kMeanWStage = kUmmaMaxN * 64 * 2;     // 32 KB
constexpr int kMeanSmem = kUmmaBarBytes + kUmmaBiasBytes + kMeanStages * (kMeanAStage + kMeanWStage);
static_assert(kMeanSmem <= 227 * 1024, "the ensemble layer needs more shared memory than a CTA has");

struct MeanMaps {
    CUtensorMap a[kMeanMaxMembers];   // member m's hidden activations, box 64 x kUmmaM, 128-byte swizzle
};

template <int EPI>
__global__ void __launch_bounds__(32 * (2 + EPI), 1)
    k_umma_mean_layer(const __grid_constant__ MeanMaps maps, const __grid_constant__ CUtensorMap tmW, int M, int Kh,
                      int members, int Np, int N, const float *bias_sum, float inv, float *Y, long long ldy, int vec,
                      int *error)
{
    static_assert(EPI % 4 == 0, "each of the four lane quarters needs the same number of epilogue warps");
    extern __shared__ __align__(1024) uint8_t smem[];
    const uint32_t b_full = smem_u32(smem), b_empty = b_full + 8 * kMeanStages, b_accf = b_empty + 8 * kMeanStages,
                   b_acce = b_accf + 16, b_drain = b_acce + 16;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 256);
    volatile int *fail = reinterpret_cast<volatile int *>(smem + 320);
    float *s_bias = reinterpret_cast<float *>(smem + kUmmaBarBytes);
    const uint32_t sA_u = smem_u32(smem + kUmmaBarBytes + kUmmaBiasBytes);   // stage s: A at +s*(A+W), W after it
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        for (int i = 0; i < kMeanStages; i++) {
            mbar_init(b_full + 8 * i, 1);
            mbar_init(b_empty + 8 * i, 1);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(b_accf + 8 * i, 1);
            mbar_init(b_acce + 8 * i, EPI);
        }
        mbar_init(b_drain, 1);
        *fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    for (int c = threadIdx.x; c < kUmmaMaxN; c += blockDim.x) s_bias[c] = c < N ? bias_sum[c] : 0.f;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    const int tiles = (M + kUmmaM - 1) / kUmmaM;
    const int per = Kh / 64, nks = per * members;   // 64-column slices per member, per tile
    const uint32_t stage_bytes = kMeanAStage + kMeanWStage;
    if (warp == 0) {
        if (lane == 0) {
            // producer: per stage, the slice of one member's activations and of the weights
            bool ok = true;
            int it = 0;
            for (int t = blockIdx.x; ok && t < tiles; t += gridDim.x)
                for (int j = 0; j < nks; j++) {
                    const int s = it % kMeanStages, use = it / kMeanStages;
                    if (use > 0 && !mbar_wait(b_empty + 8 * s, (use - 1) & 1, fail)) {
                        ok = false;
                        break;
                    }
                    const uint32_t a = sA_u + s * stage_bytes;
                    mbar_expect_tx(b_full + 8 * s, (uint32_t)(kUmmaM * 128 + Np * 128));
                    tma_load_2d(a, &maps.a[j / per], 64 * (j % per), t * kUmmaM, b_full + 8 * s);
                    tma_load_2d(a + kMeanAStage, &tmW, 64 * j, 0, b_full + 8 * s);
                    it++;
                }
            if (!ok) umma_fail(fail, error);
            for (int s = 0; s < kMeanStages; s++) {
                const int uses = it / kMeanStages + (s < it % kMeanStages ? 1 : 0);
                if (uses > 0) mbar_wait(b_full + 8 * s, (uses - 1) & 1, nullptr);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer: 4 MMAs (K = 16) per 64-column slice
            bool ok = true;
            const uint32_t idesc = umma_idesc(kUmmaM, Np);
            int it = 0, tc = 0;
            for (int t = blockIdx.x; ok && t < tiles; t += gridDim.x, tc++) {
                const int b = tc & 1, use = tc >> 1;
                if (use > 0 && !mbar_wait(b_acce + 8 * b, (use - 1) & 1, fail)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t d = tmem + 256u * b;
                for (int j = 0; j < nks; j++, it++) {
                    const int s = it % kMeanStages, u = it / kMeanStages;
                    if (!mbar_wait(b_full + 8 * s, u & 1, fail)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t a = sA_u + s * stage_bytes, w = a + kMeanAStage;
                    for (int q = 0; q < 4; q++)
                        umma_bf16(d, umma_desc(a + 32 * q, 16, 1024, kSwizzle128B),
                                  umma_desc(w + 32 * q, 16, 1024, kSwizzle128B), idesc, (j | q) != 0);
                    umma_commit(b_empty + 8 * s);
                }
                if (!ok) break;
                umma_commit(b_accf + 8 * b);
            }
            if (!ok) umma_fail(fail, error);
            umma_commit(b_drain);
            mbar_wait(b_drain, 0, nullptr);
        }
        __syncwarp();
    } else {
        // epilogue: y = inv * (acc + sum of the biases), written once
        const int q = warp & 3, part = (warp - 2) >> 2;
        constexpr int parts = EPI / 4;
        int tc = 0;
        for (int t = blockIdx.x; t < tiles; t += gridDim.x, tc++) {
            const int b = tc & 1, use = tc >> 1;
            if (!__all_sync(0xffffffffu, mbar_wait(b_accf + 8 * b, use & 1, fail))) {
                if (lane == 0) umma_fail(fail, error);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const int row = t * kUmmaM + 32 * q + lane;
            const uint32_t tb = tmem + ((uint32_t)(32 * q) << 16) + 256u * b;
            for (int c0 = 32 * part; c0 < Np; c0 += 32 * parts) {
                uint32_t v[32];
                __syncwarp();
                tmem_ld32_issue(tb + c0, v);
                tmem_ld_wait(v);
                if (row < M) epilogue_chunk(v, c0, row, s_bias, N, 0, nullptr, 0, Y, ldy, inv, 1, vec);
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(b_acce + 8 * b);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

// Wc (np x members * kh): member m's padded last-layer weights in columns [m kh, (m+1) kh)
__global__ void k_concat_weights(const bf16 *const *w, int members, int np, int kh, bf16 *wc)
{
    const long long n = (long long)np * kh * members;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long r = i / ((long long)kh * members);
        const int c = (int)(i % ((long long)kh * members));
        wc[i] = w[c / kh][r * kh + c % kh];
    }
}

// sum over members of the last layer's biases (n outputs)
__global__ void k_bias_sum(const float *const *b, int members, int n, float *out)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int m = 0; m < members; m++) s += b[m][c];
        out[c] = s;
    }
}

// Zero-padded BF16 copies for the tcgen05 path: src rows x cols (row stride cols) ->
// dst prow x pcol.
__global__ void k_pad_bf16(const bf16 *src, int rows, int cols, bf16 *dst, int prow, int pcol)
{
    const long long n = (long long)prow * pcol;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i / pcol), c = (int)(i % pcol);
        dst[i] = (r < rows && c < cols) ? src[(long long)r * cols + c] : __float2bfloat16(0.f);
    }
}

// The tcgen05 path's input: rows x din FP32 -> rows x kp BF16 (round to nearest even,
// zero columns past din), one 16-byte group of eight columns per thread.
__global__ void k_input_bf16(const float *x, int rows, int din, bf16 *dst, int kp)
{
    const int groups = kp / 8;
    const long long n = (long long)rows * groups;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long r = i / groups;
        const int c0 = (int)(i % groups) * 8;
        const float *xr = x + r * din;
        uint32_t w[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int c = c0 + 2 * k;
            w[k] = bf16x2(c < din ? xr[c] : 0.f, c + 1 < din ? xr[c + 1] : 0.f);
        }
        *reinterpret_cast<uint4 *>(dst + r * kp + c0) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// rows x cols FP32 from src (row stride lds) to dst (contiguous rows), a warp per row
__global__ void k_compact_rows(const float *src, long long lds, float *dst, int rows, int cols)
{
    const int lane = threadIdx.x & 31, wpb = blockDim.x / 32;
    const long long warps = (long long)gridDim.x * wpb;
    for (long long r = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); r < rows; r += warps) {
        const float *s = src + r * lds;
        float *d = dst + r * cols;
        for (int c = lane; c < cols; c += 32) d[c] = s[c];
    }
}

// rows of the data set -> a BF16 input batch and an FP32 target batch
__global__ void k_gather(const float *X, const float *Y, const int *idx, int B, int din, int dout, bf16 *Hb,
                         float *Yb)
{
    const int row = blockIdx.x;
    if (row >= B) return;
    const long long src = idx ? idx[row] : row;
    for (int c = threadIdx.x; c < din; c += blockDim.x) Hb[(long long)row * din + c] = __float2bfloat16(X[src * din + c]);
    if (Yb)
        for (int c = threadIdx.x; c < dout; c += blockDim.x) Yb[(long long)row * dout + c] = Y[src * dout + c];
}

// acc = scale z (first) or acc + scale z over rows x cols (row strides lda, cols), the
// arithmetic of the tcgen05 layer's accumulating epilogue
__global__ void k_accumulate(float *acc, long long lda, const float *z, int rows, int cols, float scale, int first)
{
    const long long n = (long long)rows * cols;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float *a = acc + (i / cols) * lda + i % cols;
        *a = first ? scale * z[i] : fmaf(scale, z[i], *a);
    }
}

// mean squared error over B x dout; gradient of the output layer
__global__ void k_mse(const float *Z, const float *Y, int B, int dout, float *dZf, bf16 *dZb, float *loss)
{
    const long long n = (long long)B * dout;
    const float scale = 2.f / (float)n;
    float part = 0.f;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float d = Z[e] - Y[e];
        part += d * d;
        dZf[e] = scale * d;
        dZb[e] = __float2bfloat16(scale * d);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, part / (float)n);
}

// db[j] = sum_i dZ[i][j]
__global__ void k_bias_grad(const float *dZf, int B, int N, float *db)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int i = 0; i < B; i++) s += dZf[(long long)i * N + j];
    db[j] = s;
}

// Adam (Kingma and Ba, 2015) on the FP32 master parameters; refreshes the BF16 copy.
__global__ void k_adam(float *w, float *m, float *v, const float *grad, bf16 *wb, long long n, float lr, float b1,
                       float b2, float eps, float c1, float c2)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gr = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * gr;
        const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        wb[i] = __float2bfloat16(wi);
    }
}

__global__ void k_to_bf16(const float *src, bf16 *dst, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = __float2bfloat16(src[i]);
}

thread_local std::string g_mlp_create_error;

}  // namespace

struct pt_mlp {
    int L = 0;
    std::vector<int> width;
    std::vector<long long> woff, boff;   // offsets of W_l and b_l in the parameter arrays
    long long nparam = 0;
    int max_batch = 0;
    cudaStream_t stream = nullptr;
    // device
    float *w = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    bf16 *wb = nullptr;
    std::vector<bf16 *> H;      // H[0] = input batch, H[l+1] = layer l output (BF16)
    std::vector<float *> Z;     // Z[l] = layer l pre-activation (FP32)
    std::vector<float *> dZf;   // dZ[l] (FP32)
    std::vector<bf16 *> dZb;    // dZ[l] (BF16)
    float *Ybatch = nullptr, *loss = nullptr;
    float *X = nullptr, *Y = nullptr;   // data set
    int *perm = nullptr;
    int n = 0;
    long long step = 0;
    std::string err;
    std::vector<void *> allocs;
    // tcgen05 inference: zero-padded BF16 copies of the weights (rows and columns to
    // multiples of 16), the padded input batch, and a wait error word
    int use_umma = 1;
    bool packed_stale = true;
    std::vector<bf16 *> wpk;
    std::vector<int> kpad, npad;
    bf16 *h0p = nullptr;
    int *umma_err = nullptr;
    // inference input (FP32 rows copied from the host) and output (the last layer's
    // outputs, rows padded to a multiple of 32), max_batch rows each
    float *xin = nullptr;
    float *zout = nullptr;
    int ldz = 0;
    // the ensemble mean layer (held by an ensemble's first network): the members' last
    // weights side by side, their summed biases, and device copies of the pointers
    bf16 *wcat = nullptr;
    float *bsum = nullptr;
    void **mean_ptrs = nullptr;   // kMeanMaxMembers weight pointers, then as many bias pointers
    size_t wcat_elems = 0;
};

static pt_status mfail(pt_mlp *m, pt_status st, const std::string &msg)
{
    if (m) m->err = msg;
    else g_mlp_create_error = msg;
    return st;
}

#define MCK(expr, where)                                                                                       \
    do {                                                                                                       \
        cudaError_t _e = (expr);                                                                               \
        if (_e != cudaSuccess)                                                                                 \
            return mfail(m, _e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA,                        \
                         std::string(where) + ": " + cudaGetErrorString(_e));                                  \
    } while (0)

template <typename T>
static cudaError_t dalloc(pt_mlp *m, T **p, size_t count)
{
    cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) m->allocs.push_back(*p);
    return e;
}

static cudaError_t gemm(pt_mlp *m, const GemmArgs &g)
{
    dim3 grid((g.N + kTile - 1) / kTile, (g.M + kTile - 1) / kTile);
    k_gemm<<<grid, 128, 0, m->stream>>>(g);
    return cudaGetLastError();
}

// forward pass over the B rows already in H[0]
static cudaError_t forward(pt_mlp *m, int B)
{
    for (int l = 0; l < m->L; l++) {
        const int din = m->width[l], dout = m->width[l + 1];
        GemmArgs g{};
        g.A = m->H[l];
        g.sa_i = din;
        g.sa_r = 1;
        g.B = m->wb + m->woff[l];   // B(r, j) = W_l[j][r]
        g.sb_r = 1;
        g.sb_j = din;
        g.M = B;
        g.N = dout;
        g.R = din;
        g.mode = kForward;
        g.bias = m->w + m->boff[l];
        g.Z = m->Z[l];
        g.H = m->H[l + 1];
        g.gelu = l + 1 < m->L;
        cudaError_t e = gemm(m, g);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// loss and gradients of every parameter for the B rows in H[0] / Ybatch
static cudaError_t backward(pt_mlp *m, int B)
{
    const int Lz = m->L - 1;
    cudaError_t e = cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
    if (e != cudaSuccess) return e;
    k_mse<<<std::min(1024, (B * m->width[m->L] + 255) / 256), 256, 0, m->stream>>>(
        m->Z[Lz], m->Ybatch, B, m->width[m->L], m->dZf[Lz], m->dZb[Lz], m->loss);
    for (int l = Lz; l >= 0; l--) {
        const int din = m->width[l], dout = m->width[l + 1];
        // dW_l[j][k] = sum_i dZ_l[i][j] H_l[i][k]
        GemmArgs gw{};
        gw.A = m->dZb[l];
        gw.sa_i = 1;
        gw.sa_r = dout;
        gw.B = m->H[l];
        gw.sb_r = din;
        gw.sb_j = 1;
        gw.M = dout;
        gw.N = din;
        gw.R = B;
        gw.mode = kStoreF32;
        gw.C = m->grad + m->woff[l];
        gw.ldc = din;
        e = gemm(m, gw);
        if (e != cudaSuccess) return e;
        k_bias_grad<<<(dout + 127) / 128, 128, 0, m->stream>>>(m->dZf[l], B, dout, m->grad + m->boff[l]);
        if (l > 0) {
            // dZ_{l-1}[i][k] = (sum_j dZ_l[i][j] W_l[j][k]) GELU'(Z_{l-1}[i][k])
            GemmArgs gd{};
            gd.A = m->dZb[l];
            gd.sa_i = dout;
            gd.sa_r = 1;
            gd.B = m->wb + m->woff[l];
            gd.sb_r = din;
            gd.sb_j = 1;
            gd.M = B;
            gd.N = din;
            gd.R = dout;
            gd.mode = kBackward;
            gd.Zprev = m->Z[l - 1];
            gd.dZf = m->dZf[l - 1];
            gd.dZb = m->dZb[l - 1];
            e = gemm(m, gd);
            if (e != cudaSuccess) return e;
        }
    }
    return cudaGetLastError();
}

static int grid_for(long long n) { return (int)std::min<long long>((n + 255) / 256, 4096); }

static int pad16(int x) { return (x + 15) / 16 * 16; }

// The tcgen05 path takes every layer whose padded sizes fit the kernel: inputs and
// outputs at most 256 wide, hidden widths a multiple of 32.
static bool umma_fits(const pt_mlp *m)
{
    for (int l = 0; l < m->L; l++) {
        const int din = m->width[l], dout = m->width[l + 1];
        if (pad16(din) > kUmmaMaxK || pad16(dout) > kUmmaMaxN) return false;
        if (l > 0 && din % 16 != 0) return false;           // read in place from H[l]
        if (l + 1 < m->L && dout % 32 != 0) return false;  // whole 64-byte output runs
    }
    return true;
}

static int sm_count_mlp()
{
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}

// The driver's tensor-map encoder, through the runtime's entry-point query (no link
// against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled()
{
    static const EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (EncodeTiledFn) nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// A map over a rows x cols BF16 matrix (row stride ld elements, a multiple of 8) whose
// box is box_rows rows by 64 columns with the 128-byte swizzle (sw; cols a multiple of
// 64) or by 8 columns without: the TMA boxes of a tcgen05 operand in the kernel's two
// shared-memory layouts.  Rows past `rows` read as zeros.
static bool operand_map(CUtensorMap *map, const bf16 *base, int rows, int cols, long long ld, int box_rows, bool sw)
{
    const EncodeTiledFn fn = encode_tiled();
    if (!fn || ld % 8 != 0 || cols % (sw ? 64 : 8) != 0) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {sw ? 64u : 8u, (cuuint32_t)box_rows};
    const cuuint32_t elem[2] = {1u, 1u};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, sw ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int pad32(int x) { return (x + 31) / 32 * 32; }

// rows x cols outputs from the padded accumulator (row stride lds) to dst (contiguous
// rows): on the device straight into dst, for the host through the contiguous device
// buffer `staging` and one copy.
static cudaError_t copy_out(const float *src, int lds, float *staging, int rows, int cols, float *dst,
                            cudaMemcpyKind kind, cudaStream_t s)
{
    if (rows == 0) return cudaSuccess;
    float *to = kind == cudaMemcpyDeviceToDevice ? dst : staging;
    k_compact_rows<<<std::min((rows + 7) / 8, 8192), 256, 0, s>>>(src, lds, to, rows, cols);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && kind != cudaMemcpyDeviceToDevice)
        e = cudaMemcpyAsync(dst, staging, (size_t)rows * cols * sizeof(float), kind, s);
    return e;
}

// The inference input and padded output buffers of a network, kept between calls.
static cudaError_t ensure_zout(pt_mlp *m)
{
    if (m->zout) return cudaSuccess;
    cudaError_t e = dalloc(m, &m->xin, (size_t)m->max_batch * m->width[0]);
    if (e != cudaSuccess) return e;
    m->ldz = pad32(m->width[m->L]);
    return dalloc(m, &m->zout, (size_t)m->max_batch * m->ldz);
}

// forward pass for inference over B rows of x (device, B x width[0] FP32), its outputs
// z accumulated into y (row stride ldy): y = scale z when `first`, else y + scale z.
// tcgen05 layers when the shapes fit (hidden H[l] receive the activations, the last
// layer accumulates in its epilogue), else forward() and k_accumulate.  *x0 caches the
// zero-padded BF16 copy of x that the tcgen05 layers read: the first network of an
// ensemble makes it (into its h0p), the others reuse it.
// The tcgen05 path's per-network state: padded BF16 weights (re-padded after a
// parameter change), the padded input buffer and the wait error word.
static cudaError_t umma_prepare(pt_mlp *m)
{
    cudaError_t e = cudaSuccess;
    if (m->wpk.empty()) {
        static const cudaError_t attr = [] {
            cudaError_t a = cudaFuncSetAttribute(k_umma_layer<kUmmaEpiWarps>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, kUmmaSmem);
            if (a == cudaSuccess)
                a = cudaFuncSetAttribute(k_umma_mean_layer<kUmmaEpiWarps>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kMeanSmem);
            return a;
        }();
        if (attr != cudaSuccess) return attr;
        for (int l = 0; l < m->L; l++) {
            m->kpad.push_back(pad16(m->width[l]));
            m->npad.push_back(pad16(m->width[l + 1]));
            bf16 *p = nullptr;
            e = dalloc(m, &p, (size_t)m->kpad[l] * m->npad[l]);
            if (e != cudaSuccess) return e;
            m->wpk.push_back(p);
        }
        e = dalloc(m, &m->h0p, (size_t)m->max_batch * m->kpad[0]);
        if (e == cudaSuccess) e = dalloc(m, &m->umma_err, 1);
        if (e == cudaSuccess) e = cudaMemsetAsync(m->umma_err, 0, sizeof(int), m->stream);
        if (e != cudaSuccess) return e;
        m->packed_stale = true;
    }
    if (m->packed_stale) {
        for (int l = 0; l < m->L; l++)
            k_pad_bf16<<<grid_for((long long)m->npad[l] * m->kpad[l]), 256, 0, m->stream>>>(
                m->wb + m->woff[l], m->width[l + 1], m->width[l], m->wpk[l], m->npad[l], m->kpad[l]);
        m->packed_stale = false;
        e = cudaGetLastError();
    }
    return e;
}

// With hidden_only, the tcgen05 path stops after the last hidden layer (H[L-1] holds
// its activations) and y is not written.
static cudaError_t forward_infer(pt_mlp *m, int B, const float *x, const bf16 **x0, float *y, long long ldy,
                                 float scale, bool first, bool hidden_only = false)
{
    if (!m->use_umma || !umma_fits(m)) {
        k_gather<<<B, 128, 0, m->stream>>>(x, nullptr, nullptr, B, m->width[0], m->width[m->L], m->H[0], nullptr);
        cudaError_t e = forward(m, B);
        if (e != cudaSuccess || B == 0) return e;
        const long long total = (long long)B * m->width[m->L];
        k_accumulate<<<(int)std::min<long long>((total + 255) / 256, 4096), 256, 0, m->stream>>>(
            y, ldy, m->Z[m->L - 1], B, m->width[m->L], scale, first ? 1 : 0);
        return cudaGetLastError();
    }
    cudaError_t e = umma_prepare(m);
    if (e != cudaSuccess) return e;
    if (!*x0) {
        k_input_bf16<<<grid_for((long long)B * m->kpad[0] / 8), 256, 0, m->stream>>>(x, B, m->width[0], m->h0p,
                                                                                    m->kpad[0]);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        *x0 = m->h0p;
    }
    const int tiles = (B + kUmmaM - 1) / kUmmaM;
    for (int l = 0; l < (hidden_only ? m->L - 1 : m->L); l++) {
        const int Kp = m->kpad[l], Np = m->npad[l];
        const bool last = l + 1 == m->L;
        // one CTA per SM: the full shared-memory request keeps a second one off the SM,
        // so the 512 tensor-memory columns a CTA allocates are always free
        const int grid = std::max(1, std::min(tiles, sm_count_mlp()));
        const bf16 *A = l == 0 ? *x0 : m->H[l];
        const long long lda = l == 0 ? m->kpad[0] : m->width[l];
        const bool sw = Kp % 64 == 0;   // the 128-byte swizzled layout: whole 128-byte box rows
        CUtensorMap ma, mw;
        if (!operand_map(&ma, A, B, Kp, lda, kUmmaM, sw) || !operand_map(&mw, m->wpk[l], Np, Kp, Kp, Np, sw))
            return cudaErrorNotSupported;
        const int N = m->width[l + 1];
        const float *bias = m->w + m->boff[l];
        bf16 *Hn = last ? nullptr : m->H[l + 1];
        float *Yn = last ? y : nullptr;
        // whole-sector accumulation: 32-column runs fit the row and start 32-byte aligned
        const int vec = last && ldy % 32 == 0 && ldy >= pad32(N) && reinterpret_cast<uintptr_t>(y) % 32 == 0;
        k_umma_layer<kUmmaEpiWarps><<<grid, 32 * (2 + kUmmaEpiWarps), kUmmaSmem, m->stream>>>(
            ma, mw, B, Kp, Np, N, sw ? 1 : 0, bias, last ? 0 : 1, Hn, N, Yn, ldy, scale, first ? 1 : 0, vec,
            m->umma_err);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Whether an ensemble runs its last layers as one GEMM (k_umma_mean_layer): 2 to
// kMeanMaxMembers members, all on the tcgen05 path, the last layer's input a
// multiple of 64 wide and its output at most kUmmaMaxN.
static bool mean_layer_fits(pt_mlp *const *members, int count)
{
    if (count < 2 || count > kMeanMaxMembers) return false;
    for (int j = 0; j < count; j++)
        if (!members[j]->use_umma || !umma_fits(members[j])) return false;
    const pt_mlp *m = members[0];
    return m->L >= 2 && m->width[m->L - 1] % 64 == 0 && pad16(m->width[m->L]) <= kUmmaMaxN;
}

// The mean of the members' last layers over B rows into y (row stride ldy), after
// every member's hidden layers have run (H[L-1] of each holds its activations).
static cudaError_t mean_layer(pt_mlp *const *members, int count, int B, float *y, int ldy, cudaStream_t s)
{
    pt_mlp *m = members[0];
    const int L = m->L, kh = m->width[L - 1], N = m->width[L], np = pad16(N);
    const size_t need = (size_t)np * kh * count;
    cudaError_t e = cudaSuccess;
    if (!m->mean_ptrs) e = dalloc(m, &m->mean_ptrs, 2 * kMeanMaxMembers);
    if (e == cudaSuccess && !m->bsum) e = dalloc(m, &m->bsum, kUmmaMaxN);
    if (e == cudaSuccess && m->wcat_elems < need) {
        e = dalloc(m, &m->wcat, need);
        if (e == cudaSuccess) m->wcat_elems = need;
    }
    if (e != cudaSuccess) return e;
    void *h[2 * kMeanMaxMembers] = {};
    for (int j = 0; j < count; j++) {
        h[j] = members[j]->wpk[L - 1];
        h[kMeanMaxMembers + j] = members[j]->w + members[j]->boff[L - 1];
    }
    e = cudaMemcpyAsync(m->mean_ptrs, h, sizeof(h), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    k_concat_weights<<<grid_for((long long)need), 256, 0, s>>>((const bf16 *const *)m->mean_ptrs, count, np, kh,
                                                               m->wcat);
    k_bias_sum<<<1, 256, 0, s>>>((const float *const *)(m->mean_ptrs + kMeanMaxMembers), count, N, m->bsum);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    MeanMaps maps;
    memset(&maps, 0, sizeof(maps));
    for (int j = 0; j < count; j++)
        if (!operand_map(&maps.a[j], members[j]->H[L - 1], B, kh, kh, kUmmaM, true)) return cudaErrorNotSupported;
    CUtensorMap mw;
    if (!operand_map(&mw, m->wcat, np, kh * count, (long long)kh * count, np, true)) return cudaErrorNotSupported;
    const int vec = ldy % 32 == 0 && ldy >= pad32(N) && reinterpret_cast<uintptr_t>(y) % 32 == 0;
    const int tiles = (B + kUmmaM - 1) / kUmmaM;
    const int grid = std::max(1, std::min(tiles, sm_count_mlp()));
    k_umma_mean_layer<kUmmaEpiWarps><<<grid, 32 * (2 + kUmmaEpiWarps), kMeanSmem, s>>>(
        maps, mw, B, kh, count, np, N, m->bsum, 1.0f / (float)count, y, ldy, vec, m->umma_err);
    return cudaGetLastError();
}

// One chunk of B rows of x (device) through every member, their mean into acc (row
// stride ldacc): the members' hidden layers, then one mean layer when it fits, else
// each member's last layer accumulating in its epilogue.
static cudaError_t ensemble_chunk(pt_mlp *const *members, int count, int B, const float *x, float *acc, int ldacc,
                                  cudaStream_t s)
{
    const bool fused = mean_layer_fits(members, count);
    const bf16 *x0 = nullptr;
    cudaError_t e = cudaSuccess;
    for (int j = 0; j < count && e == cudaSuccess; j++) {
        pt_mlp *q = members[j];
        const cudaStream_t own = q->stream;
        q->stream = s;
        e = forward_infer(q, B, x, &x0, acc, ldacc, 1.0f / (float)count, j == 0, fused);
        q->stream = own;
    }
    if (e != cudaSuccess || !fused || B == 0) return e;
    return mean_layer(members, count, B, acc, ldacc, s);
}

// A device wait of the tcgen05 path that gave up: reported once, then cleared.
static pt_status umma_check(pt_mlp *m)
{
    if (!m->umma_err) return PT_OK;
    int h = 0;
    MCK(cudaMemcpyAsync(&h, m->umma_err, sizeof(int), cudaMemcpyDeviceToHost, m->stream), "tcgen05 error word");
    MCK(cudaStreamSynchronize(m->stream), "sync");
    if (h) {
        cudaMemsetAsync(m->umma_err, 0, sizeof(int), m->stream);
        return mfail(m, PT_ERR_TIMEOUT, "a tcgen05 MMA completion wait gave up");
    }
    return PT_OK;
}

extern "C" {

pt_status pt_mlp_create(int layers, const int *widths, int max_batch, uint64_t seed, void *cuda_stream, pt_mlp **out)
{
    if (!widths || !out || layers < 1 || layers > 16 || max_batch < 1 || max_batch > (1 << 20))
        return mfail(nullptr, PT_ERR_ARG, "layers must be 1..16 and max_batch 1..2^20");
    for (int l = 0; l <= layers; l++)
        if (widths[l] < 1 || widths[l] > 4096) return mfail(nullptr, PT_ERR_ARG, "widths must be 1..4096");
    *out = nullptr;
    pt_mlp *m = new pt_mlp();
    m->L = layers;
    m->width.assign(widths, widths + layers + 1);
    m->max_batch = max_batch;
    m->stream = (cudaStream_t)cuda_stream;
    for (int l = 0; l < layers; l++) {
        m->woff.push_back(m->nparam);
        m->nparam += (long long)widths[l + 1] * widths[l];
        m->boff.push_back(m->nparam);
        m->nparam += widths[l + 1];
    }
    auto bad = [&](cudaError_t e, const char *what) {
        if (e == cudaSuccess) return false;
        mfail(nullptr, e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
        pt_mlp_destroy(m);
        return true;
    };
    const size_t P = (size_t)m->nparam;
    if (bad(dalloc(m, &m->w, P), "parameters") || bad(dalloc(m, &m->m, P), "adam m") ||
        bad(dalloc(m, &m->v, P), "adam v") || bad(dalloc(m, &m->grad, P), "gradients") ||
        bad(dalloc(m, &m->wb, P), "bf16 weights") || bad(dalloc(m, &m->loss, 1), "loss") ||
        bad(dalloc(m, &m->Ybatch, (size_t)max_batch * widths[layers]), "targets"))
        return PT_ERR_CUDA;
    m->H.resize(layers + 1);
    m->Z.resize(layers);
    m->dZf.resize(layers);
    m->dZb.resize(layers);
    for (int l = 0; l <= layers; l++)
        if (bad(dalloc(m, &m->H[l], (size_t)max_batch * widths[l]), "activations")) return PT_ERR_CUDA;
    for (int l = 0; l < layers; l++) {
        const size_t n = (size_t)max_batch * widths[l + 1];
        if (bad(dalloc(m, &m->Z[l], n), "pre-activations") || bad(dalloc(m, &m->dZf[l], n), "gradients") ||
            bad(dalloc(m, &m->dZb[l], n), "gradients"))
            return PT_ERR_CUDA;
    }
    // He-uniform weights (bound sqrt(6 / fan_in)), zero biases, from a seeded generator
    std::vector<float> init(P, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < layers; l++) {
        const float bound = std::sqrt(6.f / (float)widths[l]);
        std::uniform_real_distribution<float> U(-bound, bound);
        for (long long i = 0; i < (long long)widths[l + 1] * widths[l]; i++) init[m->woff[l] + i] = U(rng);
    }
    *out = m;
    return pt_mlp_set_params(m, init.data());
}

pt_status pt_mlp_param_count(const pt_mlp *m, int64_t *count)
{
    if (!m || !count) return PT_ERR_ARG;
    *count = m->nparam;
    return PT_OK;
}

pt_status pt_mlp_set_params(pt_mlp *m, const float *params)
{
    if (!m || !params) return PT_ERR_ARG;
    const size_t bytes = (size_t)m->nparam * sizeof(float);
    MCK(cudaMemcpyAsync(m->w, params, bytes, cudaMemcpyHostToDevice, m->stream), "parameters");
    MCK(cudaMemsetAsync(m->m, 0, bytes, m->stream), "adam m");
    MCK(cudaMemsetAsync(m->v, 0, bytes, m->stream), "adam v");
    k_to_bf16<<<grid_for(m->nparam), 256, 0, m->stream>>>(m->w, m->wb, m->nparam);
    MCK(cudaGetLastError(), "bf16 weights");
    MCK(cudaStreamSynchronize(m->stream), "sync");
    m->step = 0;
    m->packed_stale = true;
    return PT_OK;
}

pt_status pt_mlp_get_params(pt_mlp *m, float *params)
{
    if (!m || !params) return PT_ERR_ARG;
    MCK(cudaMemcpyAsync(params, m->w, (size_t)m->nparam * sizeof(float), cudaMemcpyDeviceToHost, m->stream), "copy");
    MCK(cudaStreamSynchronize(m->stream), "sync");
    return PT_OK;
}

pt_status pt_mlp_set_data(pt_mlp *m, const float *X, const float *Y, int n)
{
    if (!m || !X || !Y || n < 1) return PT_ERR_ARG;
    for (void *p : {(void *)m->X, (void *)m->Y, (void *)m->perm}) {
        if (!p) continue;
        cudaFree(p);
        m->allocs.erase(std::remove(m->allocs.begin(), m->allocs.end(), p), m->allocs.end());
    }
    m->X = m->Y = nullptr;
    m->perm = nullptr;
    const int din = m->width[0], dout = m->width[m->L];
    MCK(dalloc(m, &m->X, (size_t)n * din), "data");
    MCK(dalloc(m, &m->Y, (size_t)n * dout), "data");
    MCK(dalloc(m, &m->perm, (size_t)n), "data");
    MCK(cudaMemcpyAsync(m->X, X, (size_t)n * din * sizeof(float), cudaMemcpyHostToDevice, m->stream), "data");
    MCK(cudaMemcpyAsync(m->Y, Y, (size_t)n * dout * sizeof(float), cudaMemcpyHostToDevice, m->stream), "data");
    MCK(cudaStreamSynchronize(m->stream), "sync");
    m->n = n;
    return PT_OK;
}

pt_status pt_mlp_train(pt_mlp *m, int epochs, int batch, float lr, uint64_t shuffle_seed, float *epoch_loss)
{
    if (!m || epochs < 1 || batch < 1 || batch > m->max_batch || !(lr > 0.f)) return PT_ERR_ARG;
    if (!m->X) return mfail(m, PT_ERR_STATE, "pt_mlp_train before pt_mlp_set_data");
    const int din = m->width[0], dout = m->width[m->L];
    std::vector<int> perm(m->n);
    std::mt19937_64 rng(shuffle_seed);
    float last = 0.f;
    for (int ep = 0; ep < epochs; ep++) {
        std::iota(perm.begin(), perm.end(), 0);
        std::shuffle(perm.begin(), perm.end(), rng);
        MCK(cudaMemcpyAsync(m->perm, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice, m->stream),
            "permutation");
        double sum = 0.0;
        int steps = 0;
        for (int s0 = 0; s0 < m->n; s0 += batch) {
            const int B = std::min(batch, m->n - s0);
            k_gather<<<B, 128, 0, m->stream>>>(m->X, m->Y, m->perm + s0, B, din, dout, m->H[0], m->Ybatch);
            MCK(forward(m, B), "forward");
            MCK(backward(m, B), "backward");
            m->step++;
            m->packed_stale = true;
            const float c1 = 1.f - std::pow(0.9f, (float)m->step), c2 = 1.f - std::pow(0.999f, (float)m->step);
            k_adam<<<grid_for(m->nparam), 256, 0, m->stream>>>(m->w, m->m, m->v, m->grad, m->wb, m->nparam, lr, 0.9f,
                                                               0.999f, 1e-8f, c1, c2);
            MCK(cudaGetLastError(), "adam");
            if (ep == epochs - 1) {
                float l = 0.f;
                MCK(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream), "loss");
                MCK(cudaStreamSynchronize(m->stream), "sync");
                sum += l * B;
                steps += B;
            }
        }
        if (ep == epochs - 1) last = (float)(sum / std::max(steps, 1));
    }
    MCK(cudaStreamSynchronize(m->stream), "sync");
    if (epoch_loss) *epoch_loss = last;
    return PT_OK;
}

pt_status pt_mlp_gradients(pt_mlp *m, const float *X, const float *Y, int n, float *grads, float *loss)
{
    if (!m || !X || !Y || !grads || n < 1 || n > m->max_batch) return PT_ERR_ARG;
    const int din = m->width[0], dout = m->width[m->L];
    float *dX = nullptr, *dY = nullptr;
    MCK(cudaMalloc(&dX, (size_t)n * din * sizeof(float)), "batch");
    cudaError_t e = cudaMalloc(&dY, (size_t)n * dout * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dX, X, (size_t)n * din * sizeof(float), cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dY, Y, (size_t)n * dout * sizeof(float), cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) {
        k_gather<<<n, 128, 0, m->stream>>>(dX, dY, nullptr, n, din, dout, m->H[0], m->Ybatch);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = forward(m, n);
    if (e == cudaSuccess) e = backward(m, n);
    float l = 0.f;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(grads, m->grad, (size_t)m->nparam * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    cudaFree(dX);
    cudaFree(dY);
    MCK(e, "gradients");
    if (loss) *loss = l;
    return PT_OK;
}

pt_status pt_mlp_predict(pt_mlp *m, const float *X, int n, float *Y)
{
    if (!m || !X || !Y || n < 0) return PT_ERR_ARG;
    const int din = m->width[0], dout = m->width[m->L];
    const int chunk = m->max_batch;
    MCK(ensure_zout(m), "inference buffers");
    float *dX = m->xin;
    cudaError_t e = cudaSuccess;
    for (int s0 = 0; s0 < n && e == cudaSuccess; s0 += chunk) {
        const int B = std::min(chunk, n - s0);
        e = cudaMemcpyAsync(dX, X + (size_t)s0 * din, (size_t)B * din * sizeof(float), cudaMemcpyHostToDevice,
                            m->stream);
        if (e != cudaSuccess) break;
        const bf16 *x0 = nullptr;
        e = forward_infer(m, B, dX, &x0, m->zout, m->ldz, 1.0f, true);
        if (e != cudaSuccess) break;
        e = copy_out(m->zout, m->ldz, m->Z[m->L - 1], B, dout, Y + (size_t)s0 * dout, cudaMemcpyDeviceToHost,
                     m->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    MCK(e, "predict");
    return umma_check(m);
}

pt_status pt_mlp_set_tcgen05(pt_mlp *m, int enabled)
{
    if (!m) return PT_ERR_ARG;
    m->use_umma = enabled ? 1 : 0;
    return PT_OK;
}

pt_status pt_mlp_predict_ensemble(pt_mlp *const *members, int count, const float *X, int n, float *Y)
{
    if (!members || count < 1 || !X || !Y || n < 0) return PT_ERR_ARG;
    pt_mlp *m = members[0];
    if (!m) return PT_ERR_ARG;
    int chunk = m->max_batch;
    for (int j = 0; j < count; j++) {
        pt_mlp *q = members[j];
        if (!q) return PT_ERR_ARG;
        if (q->L != m->L) return mfail(m, PT_ERR_ARG, "ensemble members differ in depth");
        for (int l = 0; l <= m->L; l++)
            if (q->width[l] != m->width[l]) return mfail(m, PT_ERR_ARG, "ensemble members differ in widths");
        chunk = std::min(chunk, q->max_batch);
    }
    const int din = m->width[0], dout = m->width[m->L];
    const cudaStream_t s = m->stream;
    // every member runs on the first member's stream: finish what is queued on its own
    for (int j = 1; j < count; j++)
        if (members[j]->stream != s) MCK(cudaStreamSynchronize(members[j]->stream), "ensemble member stream");
    // the members' mean accumulates in the first member's padded output buffer
    MCK(ensure_zout(m), "inference buffers");
    float *dX = m->xin, *acc = m->zout;   // chunk <= m->max_batch rows
    cudaError_t e = cudaSuccess;
    for (int s0 = 0; s0 < n && e == cudaSuccess; s0 += chunk) {
        const int B = std::min(chunk, n - s0);
        e = cudaMemcpyAsync(dX, X + (size_t)s0 * din, (size_t)B * din * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = ensemble_chunk(members, count, B, dX, acc, m->ldz, s);
        if (e == cudaSuccess)
            e = copy_out(acc, m->ldz, m->Z[m->L - 1], B, dout, Y + (size_t)s0 * dout, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    MCK(e, "ensemble predict");
    for (int j = 0; j < count; j++) {
        const pt_status st = umma_check(members[j]);
        if (st != PT_OK) return st;
    }
    return PT_OK;
}

pt_status pt_mlp_predict_ensemble_device(pt_mlp *const *members, int count, const float *X, int n, float *Y)
{
    if (!members || count < 1 || !X || !Y || n < 0) return PT_ERR_ARG;
    pt_mlp *m = members[0];
    if (!m) return PT_ERR_ARG;
    int chunk = m->max_batch;
    for (int j = 0; j < count; j++) {
        pt_mlp *q = members[j];
        if (!q) return PT_ERR_ARG;
        if (q->L != m->L) return mfail(m, PT_ERR_ARG, "ensemble members differ in depth");
        for (int l = 0; l <= m->L; l++)
            if (q->width[l] != m->width[l]) return mfail(m, PT_ERR_ARG, "ensemble members differ in widths");
        chunk = std::min(chunk, q->max_batch);
    }
    const int din = m->width[0], dout = m->width[m->L];
    const cudaStream_t s = m->stream;
    for (int j = 1; j < count; j++)
        if (members[j]->stream != s) MCK(cudaStreamSynchronize(members[j]->stream), "ensemble member stream");
    MCK(ensure_zout(m), "inference output");
    for (int s0 = 0; s0 < n; s0 += chunk) {
        const int B = std::min(chunk, n - s0);
        MCK(ensemble_chunk(members, count, B, X + (size_t)s0 * din, m->zout, m->ldz, s), "ensemble predict (device)");
        // the mean, from the padded accumulator into y's rows
        MCK(copy_out(m->zout, m->ldz, nullptr, B, dout, Y + (size_t)s0 * dout, cudaMemcpyDeviceToDevice, s),
            "ensemble mean");
    }
    return PT_OK;
}

void pt_mlp_destroy(pt_mlp *m)
{
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    else cudaDeviceSynchronize();
    for (void *p : m->allocs) cudaFree(p);
    delete m;
}

const char *pt_mlp_last_error(const pt_mlp *m) { return m ? m->err.c_str() : g_mlp_create_error.c_str(); }

}  // extern "C"
