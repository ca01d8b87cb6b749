// pt_mlp.cu - the surrogate's multilayer perceptron: BF16 weights and activations,
// FP32 accumulation, FP32 master weights and Adam, all in hand-written kernels.
//
// Layers l = 0..L-1 map width[l] -> width[l+1]; hidden layers apply GELU, the last
// is linear.  Parameters live in one FP32 array, layer by layer: W_l (width[l+1] x
// width[l], row-major) then b_l (width[l+1]); a BF16 copy of every weight feeds the
// tensor cores.  The library owns all device memory; callers pass host arrays.
//
// GEMMs are small (at most a few thousand rows by 256), so they run on the warp-level
// tensor-core instruction mma.sync m16n8k16 (BF16 in, FP32 accumulate): one kernel
// with strided operands serves the forward product X W^T, the data gradient dZ W and
// the weight gradient dZ^T X.
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
        e = forward(m, B);
        if (e != cudaSuccess) break;
        e = cudaMemcpyAsync(Y + (size_t)s0 * dout, m->Z[m->L - 1], (size_t)B * dout * sizeof(float),
                            cudaMemcpyDeviceToHost, m->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    cudaFree(dX);
    MCK(e, "predict");
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
            e = forward(q, B);
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
            cudaError_t e = forward(q, B);
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
