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

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float z)
{
    // d/dz [z Phi(z)] = Phi(z) + z phi(z)
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
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
// Forward layers for inference on the fifth-generation tensor cores: tcgen05.mma
// (kind::f16, BF16 operands, FP32 accumulator in tensor memory), issued by one thread,
// with both operands K-major in shared memory and the accumulator read back with
// tcgen05.ld for the bias + GELU epilogue.  One CTA per SM (persistent): it keeps the
// layer's whole weight matrix (Np x Kp BF16, at most 256 x 256 = 128 KB) in shared
// memory and walks 128-row tiles of the batch: load the tile (128 x Kp BF16), one
// MMA per 16 columns of K into a 128 x Np accumulator, epilogue.
//
// Shared-memory operand layout (no swizzle, K-major): 8-row x 16-byte core matrices,
// core (row group g, K group c) at byte (g * KG + c) * 128 with KG = Kp / 8, row r of
// a core at +16 r.  So the K-direction core stride (the descriptor's leading byte
// offset) is 128 B and the row-group stride (stride byte offset) is KG * 128 B; the
// MMA over K columns [16 s, 16 s + 16) starts at +256 s.
constexpr int kUmmaM = 128;           // rows per tile (the MMA's M)
constexpr int kUmmaThreads = 512;     // sixteen warps: warp w reads accumulator lanes 32 (w % 4).. + 31,
                                      // the 32-column chunks c with c % 4 == w / 4
constexpr int kUmmaColGroups = kUmmaThreads / 128;
constexpr int kUmmaMaxN = 256, kUmmaMaxK = 256;
constexpr int kUmmaSmem = 1024 + (kUmmaMaxN + kUmmaM) * kUmmaMaxK * 2;   // barrier page + B + A
constexpr long long kUmmaSpin = 1ll << 22;   // polls of the MMA-completion barrier before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte offset
// >> 4 (16-29), stride byte offset >> 4 (32-45), the fixed 0b001 (46-48), no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 (17-22), M >> 4 (24-28).
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Copies rows [r0, r0 + R) x Kp BF16 (row stride ld elements) into the core-matrix
// layout at dst with asynchronous 16-byte copies (every thread issues all of its
// copies before waiting, so the whole tile is in flight at once); rows at or past
// `rows` are zero-filled.  The caller waits with umma_fill_wait.
__device__ __forceinline__ void umma_fill(uint8_t *dst, const bf16 *src, long long ld, int r0, int R, int rows, int Kp)
{
    const int KG = Kp / 8, chunks = R * KG;
    for (int q = threadIdx.x; q < chunks; q += blockDim.x) {
        const int r = q / KG, c = q % KG;
        const bool in = r0 + r < rows;
        const bf16 *g = in ? src + (long long)(r0 + r) * ld + 8 * c : src;
        const uint32_t s = smem_u32(dst + ((r >> 3) * KG + c) * 128 + (r & 7) * 16);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(s), "l"(g), "r"(in ? 16 : 0) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void umma_fill_wait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// One layer: out = act(A W^T + bias) over M rows.  A: M x Kp BF16 (row stride lda);
// W: Np x Kp BF16 (zero rows past N); Kp a multiple of 16, Np of 16, both <= 256.
// Hidden layers (H set) store BF16 activations (row stride ldh); the last layer
// (Z set) stores FP32 outputs (row stride N).  error: set when a wait gives up.
__global__ void __launch_bounds__(kUmmaThreads, 1)
    k_umma_layer(const bf16 *A, long long lda, int M, int Kp, const bf16 *W, int Np, int N, const float *bias, int gelu,
                 bf16 *H, long long ldh, float *Z, int *error)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 64);
    uint8_t *sB = smem + 1024;
    uint8_t *sA = sB + (size_t)Np * Kp * 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    umma_fill(sB, W, Kp, 0, Np, Np, Kp);   // waited for with the first tile's fill
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    const uint32_t KG = (uint32_t)Kp / 8;
    const uint32_t idesc = umma_idesc(kUmmaM, Np);
    const int tiles = (M + kUmmaM - 1) / kUmmaM;
    uint32_t phase = 0;
    bool failed = false;
    for (int t = blockIdx.x; t < tiles && !failed; t += gridDim.x) {
        const int m0 = t * kUmmaM;
        umma_fill(sA, A, lda, m0, kUmmaM, M, Kp);
        umma_fill_wait();
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (threadIdx.x == 0) {
            const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
            for (int s = 0; s < Kp / 16; s++) {
                const uint64_t ad = umma_desc(a0 + 256u * s, 128u, KG * 128u);
                const uint64_t bd = umma_desc(b0 + 256u * s, 128u, KG * 128u);
                const uint32_t acc = s > 0 ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(bar)));
        }
        // wait for the MMAs (bounded; the outcome is made uniform over the block)
        long long spins = 0;
        uint32_t done = 0;
        while (!done) {
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(smem_u32(bar)), "r"(phase));
            if (!done && ++spins > kUmmaSpin) break;
        }
        if (__syncthreads_or(!done)) {
            if (threadIdx.x == 0) atomicExch(error, 1);
            failed = true;
            break;
        }
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;");
        // epilogue: warp w reads accumulator lanes (rows) 32 (w % 4) .. + 31, 32 columns at
        // a time, every kUmmaColGroups-th chunk from chunk w / 4
        const int quarter = warp & 3;
        const int row = m0 + 32 * quarter + lane;
        for (int c0 = 32 * (warp >> 2); c0 < Np; c0 += 32 * kUmmaColGroups) {
            uint32_t v[32];
            const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
                  "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
                  "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                  "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            if (row >= M) continue;
            if (H) {
                uint32_t packed[16];
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                    const int c = c0 + j;
                    float z0 = __uint_as_float(v[j]) + (c < N ? bias[c] : 0.f);
                    float z1 = __uint_as_float(v[j + 1]) + (c + 1 < N ? bias[c + 1] : 0.f);
                    if (gelu) {
                        z0 = 0.5f * z0 * (1.f + erff(z0 * 0.70710678118654752f));
                        z1 = 0.5f * z1 * (1.f + erff(z1 * 0.70710678118654752f));
                    }
                    packed[j / 2] = pack2(__float2bfloat16(z0), __float2bfloat16(z1));
                }
                // N is a multiple of 32 for hidden layers: whole 64-byte runs
                uint4 *dst = reinterpret_cast<uint4 *>(H + (long long)row * ldh + c0);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
            } else {
                float *dst = Z + (long long)row * N;
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const int c = c0 + j;
                    if (c < N) dst[c] = __uint_as_float(v[j]) + bias[c];
                }
            }
        }
        // the next tile's MMA overwrites the accumulator and its fill the A operand
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
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

// acc = (first ? 0 : acc) + scale * z over n values
__global__ void k_accumulate(float *acc, const float *z, long long n, float scale, int first)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        acc[i] = first ? scale * z[i] : acc[i] + scale * z[i];
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

// forward pass for inference over the B rows in H[0]: tcgen05 layers when the shapes
// fit (Z[L-1] receives the outputs, hidden H[l] the activations), else forward().
static cudaError_t forward_infer(pt_mlp *m, int B)
{
    if (!m->use_umma || !umma_fits(m)) return forward(m, B);
    cudaError_t e = cudaSuccess;
    if (m->wpk.empty()) {
        static const cudaError_t attr =
            cudaFuncSetAttribute(k_umma_layer, cudaFuncAttributeMaxDynamicSharedMemorySize, kUmmaSmem);
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
    }
    k_pad_bf16<<<grid_for((long long)B * m->kpad[0]), 256, 0, m->stream>>>(m->H[0], B, m->width[0], m->h0p, B,
                                                                           m->kpad[0]);
    const int tiles = (B + kUmmaM - 1) / kUmmaM;
    for (int l = 0; l < m->L; l++) {
        const int Kp = m->kpad[l], Np = m->npad[l];
        const bool last = l + 1 == m->L;
        // at least 80 KB per CTA: two CTAs per SM at most, within the 512 TMEM columns
        const int smem = std::max(1024 + (Np + kUmmaM) * Kp * 2, 80 * 1024);
        const int per_sm = smem > 114 * 1024 ? 1 : 2;
        const int grid = std::max(1, std::min(tiles, per_sm * sm_count_mlp()));
        const bf16 *A = l == 0 ? m->h0p : m->H[l];
        const long long lda = l == 0 ? m->kpad[0] : m->width[l];
        k_umma_layer<<<grid, kUmmaThreads, smem, m->stream>>>(A, lda, B, Kp, m->wpk[l], Np, m->width[l + 1],
                                                             m->w + m->boff[l], last ? 0 : 1,
                                                             last ? nullptr : m->H[l + 1], m->width[l + 1],
                                                             last ? m->Z[l] : nullptr, m->umma_err);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
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
    float *dX = nullptr;
    const int chunk = m->max_batch;
    MCK(cudaMalloc(&dX, (size_t)std::max(1, std::min(n, chunk)) * din * sizeof(float)), "batch");
    cudaError_t e = cudaSuccess;
    for (int s0 = 0; s0 < n && e == cudaSuccess; s0 += chunk) {
        const int B = std::min(chunk, n - s0);
        e = cudaMemcpyAsync(dX, X + (size_t)s0 * din, (size_t)B * din * sizeof(float), cudaMemcpyHostToDevice,
                            m->stream);
        if (e != cudaSuccess) break;
        k_gather<<<B, 128, 0, m->stream>>>(dX, nullptr, nullptr, B, din, dout, m->H[0], nullptr);
        e = forward_infer(m, B);
        if (e != cudaSuccess) break;
        e = cudaMemcpyAsync(Y + (size_t)s0 * dout, m->Z[m->L - 1], (size_t)B * dout * sizeof(float),
                            cudaMemcpyDeviceToHost, m->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    cudaFree(dX);
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
    float *dX = nullptr, *acc = nullptr;
    const size_t rows = (size_t)std::max(1, std::min(n, chunk));
    MCK(cudaMalloc(&dX, rows * din * sizeof(float)), "batch");
    cudaError_t e = cudaMalloc(&acc, rows * dout * sizeof(float));
    for (int s0 = 0; s0 < n && e == cudaSuccess; s0 += chunk) {
        const int B = std::min(chunk, n - s0);
        e = cudaMemcpyAsync(dX, X + (size_t)s0 * din, (size_t)B * din * sizeof(float), cudaMemcpyHostToDevice, s);
        for (int j = 0; j < count && e == cudaSuccess; j++) {
            pt_mlp *q = members[j];
            const cudaStream_t own = q->stream;
            q->stream = s;
            k_gather<<<B, 128, 0, s>>>(dX, nullptr, nullptr, B, din, dout, q->H[0], nullptr);
            e = forward_infer(q, B);
            if (e == cudaSuccess) {
                const long long total = (long long)B * dout;
                k_accumulate<<<(int)std::min<long long>((total + 255) / 256, 4096), 256, 0, s>>>(
                    acc, q->Z[q->L - 1], total, 1.0f / (float)count, j == 0);
                e = cudaGetLastError();
            }
            q->stream = own;
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(Y + (size_t)s0 * dout, acc, (size_t)B * dout * sizeof(float), cudaMemcpyDeviceToHost,
                                s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dX);
    if (acc) cudaFree(acc);
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
    for (int s0 = 0; s0 < n; s0 += chunk) {
        const int B = std::min(chunk, n - s0);
        for (int j = 0; j < count; j++) {
            pt_mlp *q = members[j];
            const cudaStream_t own = q->stream;
            q->stream = s;
            k_gather<<<B, 128, 0, s>>>(X + (size_t)s0 * din, nullptr, nullptr, B, din, dout, q->H[0], nullptr);
            cudaError_t e = forward_infer(q, B);
            if (e == cudaSuccess) {
                const long long total = (long long)B * dout;
                k_accumulate<<<(int)std::min<long long>((total + 255) / 256, 4096), 256, 0, s>>>(
                    Y + (size_t)s0 * dout, q->Z[q->L - 1], total, 1.0f / (float)count, j == 0);
                e = cudaGetLastError();
            }
            q->stream = own;
            MCK(e, "ensemble predict (device)");
        }
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
