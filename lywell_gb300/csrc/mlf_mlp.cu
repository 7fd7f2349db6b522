// Small MLP for the learned near-field preconditioner: hand-written forward,
// backward and Adam kernels.  The forward of inference runs on tcgen05 tensor
// cores (BF16 operands, FP32 accumulation in TMEM); training's forward and
// backward run on FP32 FMAs over the same BF16 values.
//
// Network: 16 inputs -> 128 (ReLU) -> 128 (ReLU) -> 2 outputs, one token per
// row.  Parameters are kept as an FP32 master copy (Adam state beside it) and
// a BF16 copy that the forward and backward kernels read; hidden activations
// are stored in BF16; every product and sum accumulates in FP32.  Inputs are
// normalised in the kernel as (x - mu) / sd.
//
// Parameter vector layout (FP32 and BF16 copies alike):
//   W1[16][128] b1[128] W2[128][128] b2[128] W3[128][2] b3[2]   (W[in][out])
//
// Training loss: mean over tokens and outputs of (out - target)^2.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/lywell_mlfma.h"
#include "mlf_tcgen05.h"

namespace mlp {

constexpr int IN = 16, H = 128, OUT = 2, TT = 64;
constexpr int OW1 = 0, OB1 = OW1 + IN * H, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + H * OUT,
              NPARAM = OB3 + OUT;

struct Net {
    int dev = 0;
    cudaStream_t stream = nullptr;
    float* P = nullptr;            // FP32 master
    __nv_bfloat16* Pb = nullptr;   // BF16 copy
    float *G = nullptr, *M1 = nullptr, *M2 = nullptr;
    float* norm = nullptr;         // mu[16], sd[16]
    double* dloss = nullptr;
    int* derr = nullptr;           // set when a tensor-core forward CTA gave up a wait
    int adam_t = 0;
    std::string err;
};

// shared-memory image of one tile
struct Smem {
    float W1[IN * H], b1[H], W2[H * H], b2[H], W3[H * OUT], b3[OUT];
    float X[TT * IN];
    __nv_bfloat16 H1[TT * H], H2[TT * H];
    float out[TT * OUT];
    float dH2[TT * H], dH1[TT * H];
};

__device__ __forceinline__ float bf(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ void load_weights(Smem& s, const __nv_bfloat16* __restrict__ Pb) {
    for (int q = threadIdx.x; q < IN * H; q += blockDim.x) s.W1[q] = __bfloat162float(Pb[OW1 + q]);
    for (int q = threadIdx.x; q < H * H; q += blockDim.x) s.W2[q] = __bfloat162float(Pb[OW2 + q]);
    for (int q = threadIdx.x; q < H * OUT; q += blockDim.x) s.W3[q] = __bfloat162float(Pb[OW3 + q]);
    for (int q = threadIdx.x; q < H; q += blockDim.x) {
        s.b1[q] = __bfloat162float(Pb[OB1 + q]);
        s.b2[q] = __bfloat162float(Pb[OB2 + q]);
    }
    if (threadIdx.x < OUT) s.b3[threadIdx.x] = __bfloat162float(Pb[OB3 + threadIdx.x]);
}

// forward of one tile of nt <= TT tokens starting at token t0 (rows past nt are zero)
__device__ void forward_tile(Smem& s, const float* __restrict__ X, const float* __restrict__ norm, long long t0,
                             int nt) {
    for (int q = threadIdx.x; q < TT * IN; q += blockDim.x) {
        const int t = q / IN, i = q - t * IN;
        s.X[q] = t < nt ? (X[(t0 + t) * IN + i] - norm[i]) / norm[IN + i] : 0.f;
    }
    __syncthreads();
    // 256 threads: token group tg = tid / 16 (4 tokens), neuron group ng = tid % 16 (8 neurons)
    const int tg = threadIdx.x >> 4, ng = threadIdx.x & 15;
    {
        float acc[4][8];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[a][u] = s.b1[ng * 8 + u];
        for (int i = 0; i < IN; ++i) {
            float w[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) w[u] = s.W1[i * H + ng * 8 + u];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float x = s.X[(tg * 4 + a) * IN + i];
#pragma unroll
                for (int u = 0; u < 8; ++u) acc[a][u] = fmaf(x, w[u], acc[a][u]);
            }
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int u = 0; u < 8; ++u) s.H1[(tg * 4 + a) * H + ng * 8 + u] = __float2bfloat16_rn(fmaxf(acc[a][u], 0.f));
    }
    __syncthreads();
    {
        float acc[4][8];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[a][u] = s.b2[ng * 8 + u];
        for (int k = 0; k < H; ++k) {
            float w[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) w[u] = s.W2[k * H + ng * 8 + u];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float h = __bfloat162float(s.H1[(tg * 4 + a) * H + k]);
#pragma unroll
                for (int u = 0; u < 8; ++u) acc[a][u] = fmaf(h, w[u], acc[a][u]);
            }
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int u = 0; u < 8; ++u) s.H2[(tg * 4 + a) * H + ng * 8 + u] = __float2bfloat16_rn(fmaxf(acc[a][u], 0.f));
    }
    __syncthreads();
    if (threadIdx.x < TT * OUT) {
        const int t = threadIdx.x / OUT, o = threadIdx.x - t * OUT;
        float acc = s.b3[o];
        for (int k = 0; k < H; ++k) acc = fmaf(__bfloat162float(s.H2[t * H + k]), s.W3[k * OUT + o], acc);
        s.out[threadIdx.x] = acc;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Forward on the fifth-generation tensor cores (inference: mlf_mlp_forward, and
// so mlf_lp_install).  One tile = 128 tokens = the MMA's M.  The 128 x 128
// hidden layer, 86 % of the flops, is tcgen05.mma .kind::f16: A = H1 (BF16,
// 128 tokens x 128), B = W2^T (BF16, row n = neuron n's weights), both written
// by the threads into K-major 128-byte-swizzled tiles, FP32 accumulator in
// TMEM.  Layer 1 (K = 16, on FP32 normalised inputs, which BF16 operands
// would round) and layer 3 (two outputs) are per-token FP32 dot products in
// registers.  Thread t owns token t: it writes its row of H1 and reads its
// TMEM lane back.  The arithmetic is the CUDA-core path's -- BF16 values, FP32
// sums, H1 and H2 rounded to BF16 -- in another summation order.
// ---------------------------------------------------------------------------
constexpr int TQ = 128;
constexpr uint32_t MLP_SPIN = 1u << 20;   // mbarrier polls before a wait gives up

struct TcMlpSmem {
    alignas(1024) unsigned char H1[2 * TQ * 128];   // layer-2 A: 128 BF16 per token, two K-blocks of 64
    alignas(1024) unsigned char W2t[2 * H * 128];   // layer-2 B: W2^T, two K-blocks
    float W1[IN * H], b1[H], b2[H], W3[H * OUT], b3[OUT], mu[IN], sd[IN];
    uint64_t bar;
    uint32_t tmem;
    int fail;
};

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(a, b);   // a at the lower address
    return *reinterpret_cast<const uint32_t*>(&p);
}

__global__ void __launch_bounds__(TQ, 2) k_mlp_forward_tc(long long ntok, const float* __restrict__ X,
                                                         const float* __restrict__ norm,
                                                         const __nv_bfloat16* __restrict__ Pb, float* __restrict__ Y,
                                                         int* __restrict__ err) {
    namespace tc = mlf::tc;
    extern __shared__ unsigned char mlp_raw[];
    const uint32_t raw = tc::smem_u32(mlp_raw);
    TcMlpSmem& s = *reinterpret_cast<TcMlpSmem*>(mlp_raw + (((raw + 1023u) & ~1023u) - raw));
    const int tid = threadIdx.x, warp = tid >> 5;
    // layer-2 B operand (thread = neuron n), layer 1, biases, the output layer, the normalisation
    for (int q = tid; q < IN * H; q += TQ) s.W1[q] = __bfloat162float(Pb[OW1 + q]);
    for (int c = 0; c < 16; ++c) {
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int k = c * 8 + 2 * q;
            w[q] = pack_bf2(__bfloat162float(Pb[OW2 + k * H + tid]), __bfloat162float(Pb[OW2 + (k + 1) * H + tid]));
        }
        *reinterpret_cast<uint4*>(s.W2t + (c >> 3) * (H * 128) + tc::sw128_offset(tid, c & 7)) =
            make_uint4(w[0], w[1], w[2], w[3]);
    }
    s.b1[tid] = __bfloat162float(Pb[OB1 + tid]);
    s.b2[tid] = __bfloat162float(Pb[OB2 + tid]);
    s.W3[2 * tid] = __bfloat162float(Pb[OW3 + 2 * tid]);
    s.W3[2 * tid + 1] = __bfloat162float(Pb[OW3 + 2 * tid + 1]);
    if (tid < OUT) s.b3[tid] = __bfloat162float(Pb[OB3 + tid]);
    if (tid < IN) {
        s.mu[tid] = norm[tid];
        s.sd[tid] = norm[IN + tid];
    }
    if (tid == 0) {
        tc::mbar_init(&s.bar, 1);
        s.fail = 0;
        tc::fence_barrier_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(&s.tmem, 128);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before_sync();
    __syncthreads();
    tc::tc_fence_after_sync();
    const uint32_t tmem = s.tmem, lane_base = (uint32_t)(32 * warp) << 16;
    const uint32_t idesc = tc::instr_desc_f32acc(tc::FMT_BF16, TQ, H);
    const uint32_t aH = tc::smem_u32(s.H1), aW2 = tc::smem_u32(s.W2t);
    uint32_t phase = 0;
    for (long long t0 = (long long)blockIdx.x * TQ; t0 < ntok; t0 += (long long)gridDim.x * TQ) {
        const long long tok = t0 + tid;
        const bool live = tok < ntok;
        // layer 1 (K = 16) in FP32 on the token's normalised inputs; H1 = relu(.)
        // rounded to BF16, this token's row of the layer-2 operand
        float xn[IN];
#pragma unroll
        for (int i = 0; i < IN; ++i) xn[i] = live ? (X[tok * IN + i] - s.mu[i]) / s.sd[i] : 0.f;
        for (int c = 0; c < 16; ++c) {   // 16-byte chunk c = neurons 8c .. 8c+7
            float acc[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[u] = s.b1[8 * c + u];
#pragma unroll
            for (int i = 0; i < IN; ++i)
#pragma unroll
                for (int u = 0; u < 8; ++u) acc[u] = fmaf(xn[i], s.W1[i * H + 8 * c + u], acc[u]);
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = pack_bf2(fmaxf(acc[2 * q], 0.f), fmaxf(acc[2 * q + 1], 0.f));
            *reinterpret_cast<uint4*>(s.H1 + (c >> 3) * (TQ * 128) + tc::sw128_offset(tid, c & 7)) =
                make_uint4(w[0], w[1], w[2], w[3]);
        }
        tc::fence_proxy_async_smem();
        tc::tc_fence_before_sync();   // the previous tile's TMEM reads are done
        __syncthreads();
        if (tid == 0) {
            tc::tc_fence_after_sync();
#pragma unroll
            for (int kb = 0; kb < 2; ++kb)
#pragma unroll
                for (int q = 0; q < 4; ++q)   // K steps of 16 BF16 = 32 bytes of the 128-byte rows
                    tc::mma_f16(tmem, tc::kmajor_sw128_desc(aH + kb * (TQ * 128) + 32 * q),
                                tc::kmajor_sw128_desc(aW2 + kb * (H * 128) + 32 * q), idesc, (kb | q) != 0);
            tc::mma_commit(&s.bar);
            if (!tc::mbar_wait(&s.bar, phase, MLP_SPIN)) s.fail = 1;
        }
        phase ^= 1;
        __syncthreads();
        tc::tc_fence_after_sync();
        if (s.fail) break;
        // out = W3^T H2 + b3, H2 = relu(D2 + b2) rounded to BF16
        float o0 = s.b3[0], o1 = s.b3[1];
        for (int c0 = 0; c0 < H; c0 += 32) {
            float v[32];
            tc::tmem_ld_32x32b_x32(tmem + lane_base + (uint32_t)c0, v);
#pragma unroll
            for (int k = 0; k < 32; ++k) {
                const float h = bf(fmaxf(v[k] + s.b2[c0 + k], 0.f));
                o0 = fmaf(h, s.W3[(c0 + k) * OUT], o0);
                o1 = fmaf(h, s.W3[(c0 + k) * OUT + 1], o1);
            }
        }
        if (live) {
            Y[tok * OUT] = o0;
            Y[tok * OUT + 1] = o1;
        }
    }
    if (tid == 0 && s.fail) atomicExch(err, 1);
    tc::tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

// Forward + loss + backward over tokens idx[0..ntok) (idx NULL: 0..ntok-1);
// gradients of the mean loss (scale = 1 / (ntok_total * OUT)) added into G,
// the loss sum into *loss.
__global__ void __launch_bounds__(256) k_mlp_grad(long long ntok, const long long* __restrict__ idx,
                                                  const float* __restrict__ X, const float* __restrict__ T,
                                                  const float* __restrict__ norm,
                                                  const __nv_bfloat16* __restrict__ Pb, float scale,
                                                  float* __restrict__ G, double* __restrict__ loss,
                                                  float* __restrict__ Xg, float* __restrict__ Tg) {
    extern __shared__ __align__(16) unsigned char smraw[];
    Smem& s = *reinterpret_cast<Smem*>(smraw);
    load_weights(s, Pb);
    const int tg = threadIdx.x >> 4, ng = threadIdx.x & 15;
    // gathered copies of this CTA's tokens (rows blockIdx.x * TT ..) when idx is given
    for (long long t0 = (long long)blockIdx.x * TT; t0 < ntok; t0 += (long long)gridDim.x * TT) {
        const int nt = (int)((ntok - t0) < TT ? (ntok - t0) : TT);
        const float* Xs = X;
        const float* Ts = T;
        long long base = t0;
        if (idx) {
            float* xg = Xg + (size_t)blockIdx.x * TT * IN;
            float* tgb = Tg + (size_t)blockIdx.x * TT * OUT;
            for (int q = threadIdx.x; q < nt * IN; q += blockDim.x) {
                const int t = q / IN, i = q - t * IN;
                xg[q] = X[idx[t0 + t] * IN + i];
            }
            for (int q = threadIdx.x; q < nt * OUT; q += blockDim.x) {
                const int t = q / OUT, o = q - t * OUT;
                tgb[q] = T[idx[t0 + t] * OUT + o];
            }
            __syncthreads();
            Xs = xg;
            Ts = tgb;
            base = 0;
        }
        forward_tile(s, Xs, norm, base, nt);
        // dOut in s.out (in place) and the loss
        float lsum = 0.f;
        if (threadIdx.x < TT * OUT) {
            const int t = threadIdx.x / OUT;
            float d = 0.f;
            if (t < nt) {
                d = s.out[threadIdx.x] - Ts[base * OUT + threadIdx.x];
                lsum = d * d;
            }
            s.out[threadIdx.x] = 2.f * scale * d;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffff, lsum, o);
        if ((threadIdx.x & 31) == 0 && threadIdx.x < TT * OUT) atomicAdd(loss, (double)lsum);
        __syncthreads();
        // dW3, db3
        {
            const int k = threadIdx.x >> 1, o = threadIdx.x & 1;   // 256 = 128 x 2
            float g = 0.f;
            for (int t = 0; t < TT; ++t) g = fmaf(__bfloat162float(s.H2[t * H + k]), s.out[t * OUT + o], g);
            atomicAdd(&G[OW3 + k * OUT + o], g);
            if (threadIdx.x < OUT) {
                float gb = 0.f;
                for (int t = 0; t < TT; ++t) gb += s.out[t * OUT + threadIdx.x];
                atomicAdd(&G[OB3 + threadIdx.x], gb);
            }
        }
        // dH2 = relu'(H2) * dOut W3^T
        for (int q = threadIdx.x; q < TT * H; q += blockDim.x) {
            const int t = q / H, k = q - t * H;
            const float h = __bfloat162float(s.H2[q]);
            s.dH2[q] = h > 0.f ? s.out[t * OUT] * s.W3[k * OUT] + s.out[t * OUT + 1] * s.W3[k * OUT + 1] : 0.f;
        }
        __syncthreads();
        // dW2[k][n] = sum_t H1[t][k] dH2[t][n]: thread (kg = tid / 16: 8 k's, ng: 8 n's)
        {
            float acc[8][8];
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int u = 0; u < 8; ++u) acc[a][u] = 0.f;
            for (int t = 0; t < TT; ++t) {
                float d[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) d[u] = s.dH2[t * H + ng * 8 + u];
#pragma unroll
                for (int a = 0; a < 8; ++a) {
                    const float h = __bfloat162float(s.H1[t * H + tg * 8 + a]);
#pragma unroll
                    for (int u = 0; u < 8; ++u) acc[a][u] = fmaf(h, d[u], acc[a][u]);
                }
            }
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int u = 0; u < 8; ++u) atomicAdd(&G[OW2 + (tg * 8 + a) * H + ng * 8 + u], acc[a][u]);
        }
        if (threadIdx.x < H) {
            float gb = 0.f;
            for (int t = 0; t < TT; ++t) gb += s.dH2[t * H + threadIdx.x];
            atomicAdd(&G[OB2 + threadIdx.x], gb);
        }
        // dH1 = relu'(H1) * dH2 W2^T
        {
            float acc[4][8];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int u = 0; u < 8; ++u) acc[a][u] = 0.f;
            for (int n = 0; n < H; ++n) {
                float w[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) w[u] = s.W2[(ng * 8 + u) * H + n];
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const float d = s.dH2[(tg * 4 + a) * H + n];
#pragma unroll
                    for (int u = 0; u < 8; ++u) acc[a][u] = fmaf(d, w[u], acc[a][u]);
                }
            }
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int q = (tg * 4 + a) * H + ng * 8 + u;
                    s.dH1[q] = __bfloat162float(s.H1[q]) > 0.f ? acc[a][u] : 0.f;
                }
        }
        __syncthreads();
        // dW1[i][n] = sum_t X[t][i] dH1[t][n]: 2048 = 256 x 8
        {
            const int i = threadIdx.x >> 4;
            float acc[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[u] = 0.f;
            for (int t = 0; t < TT; ++t) {
                const float x = s.X[t * IN + i];
#pragma unroll
                for (int u = 0; u < 8; ++u) acc[u] = fmaf(x, s.dH1[t * H + ng * 8 + u], acc[u]);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) atomicAdd(&G[OW1 + i * H + ng * 8 + u], acc[u]);
        }
        if (threadIdx.x < H) {
            float gb = 0.f;
            for (int t = 0; t < TT; ++t) gb += s.dH1[t * H + threadIdx.x];
            atomicAdd(&G[OB1 + threadIdx.x], gb);
        }
        __syncthreads();
    }
}

__global__ void k_adam(int n, float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M1,
                       float* __restrict__ M2, __nv_bfloat16* __restrict__ Pb, float lr, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float m = 0.9f * M1[i] + 0.1f * g;
    const float v = 0.999f * M2[i] + 0.001f * g * g;
    M1[i] = m;
    M2[i] = v;
    const float p = P[i] - lr * (m * c1) / (sqrtf(v * c2) + 1e-8f);
    P[i] = p;
    Pb[i] = __float2bfloat16_rn(p);
}

__global__ void k_to_bf16(int n, const float* __restrict__ P, __nv_bfloat16* __restrict__ Pb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) Pb[i] = __float2bfloat16_rn(P[i]);
}

// batch indices: idx[b] = hash(seed, step, b) mod ntok
__global__ void k_batch_idx(int nb, long long ntok, unsigned long long seed, int step, long long* __restrict__ idx) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(step * 1000003ll + b + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    idx[b] = (long long)(z % (unsigned long long)ntok);
}

static bool ok(Net* n, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    n->err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

#define NCK(call)                                          \
    do {                                                   \
        if (!ok(n, (call), #call)) return MLF_E_CUDA;      \
    } while (0)

static int grid_for(long long ntok) {
    const long long tiles = (ntok + TT - 1) / TT;
    return (int)std::min<long long>(tiles, 152 * 8);
}

}  // namespace mlp

using namespace mlp;

struct mlf_mlp {
    Net n;
};

extern "C" {

int mlf_mlp_create(mlf_mlp** out, int device, unsigned long long seed) {
    if (!out) return MLF_E_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return MLF_E_NO_DEVICE;
    auto* h = new mlf_mlp();
    Net* n = &h->n;
    n->dev = device;
    auto fail = [&](int st) { mlf_mlp_free(h); return st; };
    if (!ok(n, cudaSetDevice(device), "cudaSetDevice")) return fail(MLF_E_CUDA);
    if (!ok(n, cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking), "stream")) return fail(MLF_E_CUDA);
    if (!ok(n, cudaMalloc(&n->P, NPARAM * sizeof(float)), "alloc") ||
        !ok(n, cudaMalloc(&n->Pb, NPARAM * sizeof(__nv_bfloat16)), "alloc") ||
        !ok(n, cudaMalloc(&n->G, NPARAM * sizeof(float)), "alloc") ||
        !ok(n, cudaMalloc(&n->M1, NPARAM * sizeof(float)), "alloc") ||
        !ok(n, cudaMalloc(&n->M2, NPARAM * sizeof(float)), "alloc") ||
        !ok(n, cudaMalloc(&n->norm, 2 * IN * sizeof(float)), "alloc") ||
        !ok(n, cudaMalloc(&n->dloss, sizeof(double)), "alloc") ||
        !ok(n, cudaMalloc(&n->derr, sizeof(int)), "alloc") || !ok(n, cudaMemset(n->derr, 0, sizeof(int)), "memset"))
        return fail(MLF_E_CUDA);
    if (!ok(n, cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(TcMlpSmem) + 1024)),
            "smem") ||
        !ok(n, cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(Smem)), "smem"))
        return fail(MLF_E_CUDA);
    // Glorot-uniform weights, zero biases
    std::vector<float> P(NPARAM, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fin, int fout) {
        const float a = std::sqrt(6.f / (fin + fout));
        std::uniform_real_distribution<float> U(-a, a);
        for (int q = 0; q < fin * fout; ++q) P[off + q] = U(rng);
    };
    fill(OW1, IN, H);
    fill(OW2, H, H);
    fill(OW3, H, OUT);
    std::vector<float> nm(2 * IN, 0.f);
    for (int i = 0; i < IN; ++i) nm[IN + i] = 1.f;
    if (!ok(n, cudaMemcpy(n->P, P.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice), "copy") ||
        !ok(n, cudaMemcpy(n->norm, nm.data(), 2 * IN * sizeof(float), cudaMemcpyHostToDevice), "copy") ||
        !ok(n, cudaMemset(n->M1, 0, NPARAM * sizeof(float)), "memset") ||
        !ok(n, cudaMemset(n->M2, 0, NPARAM * sizeof(float)), "memset"))
        return fail(MLF_E_CUDA);
    k_to_bf16<<<(NPARAM + 255) / 256, 256, 0, n->stream>>>(NPARAM, n->P, n->Pb);
    if (!ok(n, cudaStreamSynchronize(n->stream), "init")) return fail(MLF_E_CUDA);
    *out = h;
    return MLF_OK;
}

void mlf_mlp_free(mlf_mlp* h) {
    if (!h) return;
    Net* n = &h->n;
    cudaSetDevice(n->dev);
    for (void* p : {(void*)n->P, (void*)n->Pb, (void*)n->G, (void*)n->M1, (void*)n->M2, (void*)n->norm,
                    (void*)n->dloss, (void*)n->derr})
        if (p) cudaFree(p);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete h;
}

const char* mlf_mlp_last_error(mlf_mlp* h) { return h ? h->n.err.c_str() : "null network"; }

int mlf_mlp_nparam(void) { return NPARAM; }

int mlf_mlp_set_params(mlf_mlp* h, const float* params, const float* norm) {
    if (!h) return MLF_E_ARG;
    Net* n = &h->n;
    NCK(cudaSetDevice(n->dev));
    if (params) {
        NCK(cudaMemcpy(n->P, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
        k_to_bf16<<<(NPARAM + 255) / 256, 256, 0, n->stream>>>(NPARAM, n->P, n->Pb);
        NCK(cudaMemset(n->M1, 0, NPARAM * sizeof(float)));
        NCK(cudaMemset(n->M2, 0, NPARAM * sizeof(float)));
        n->adam_t = 0;
    }
    if (norm) NCK(cudaMemcpy(n->norm, norm, 2 * IN * sizeof(float), cudaMemcpyHostToDevice));
    NCK(cudaStreamSynchronize(n->stream));
    return MLF_OK;
}

int mlf_mlp_get_params(mlf_mlp* h, float* params, float* norm) {
    if (!h) return MLF_E_ARG;
    Net* n = &h->n;
    NCK(cudaSetDevice(n->dev));
    if (params) NCK(cudaMemcpy(params, n->P, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    if (norm) NCK(cudaMemcpy(norm, n->norm, 2 * IN * sizeof(float), cudaMemcpyDeviceToHost));
    return MLF_OK;
}

// Y[ntok][2] = net(X[ntok][16]); device pointers; stream NULL = the network's own
int mlf_mlp_forward(mlf_mlp* h, const float* X, long long ntok, float* Y, void* stream) {
    if (!h || !X || !Y || ntok < 0) return MLF_E_ARG;
    Net* n = &h->n;
    NCK(cudaSetDevice(n->dev));
    cudaStream_t s = stream ? (cudaStream_t)stream : n->stream;
    if (ntok) {
        int nsm = 0;
        NCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, n->dev));
        const long long tiles = (ntok + TQ - 1) / TQ;
        const int grid = (int)std::min<long long>(tiles, 2LL * nsm);
        k_mlp_forward_tc<<<grid, TQ, sizeof(TcMlpSmem) + 1024, s>>>(ntok, X, n->norm, n->Pb, Y, n->derr);
    }
    NCK(cudaGetLastError());
    if (!stream) {
        NCK(cudaStreamSynchronize(s));
        int e = 0;
        NCK(cudaMemcpy(&e, n->derr, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) {
            cudaMemset(n->derr, 0, sizeof(int));
            n->err = "tensor-core forward: an mbarrier wait gave up";
            return MLF_E_CUDA;
        }
    }
    return MLF_OK;
}

// Full-batch gradient of the mean loss over all ntok tokens (device X, T);
// grad (host, NPARAM) and *loss (host) receive the result.
int mlf_mlp_grad(mlf_mlp* h, const float* X, const float* T, long long ntok, float* grad, double* loss) {
    if (!h || !X || !T || ntok <= 0) return MLF_E_ARG;
    Net* n = &h->n;
    NCK(cudaSetDevice(n->dev));
    NCK(cudaMemsetAsync(n->G, 0, NPARAM * sizeof(float), n->stream));
    NCK(cudaMemsetAsync(n->dloss, 0, sizeof(double), n->stream));
    const float scale = (float)(1.0 / ((double)ntok * OUT));
    k_mlp_grad<<<grid_for(ntok), 256, sizeof(Smem), n->stream>>>(ntok, nullptr, X, T, n->norm, n->Pb, scale, n->G,
                                                                 n->dloss, nullptr, nullptr);
    NCK(cudaGetLastError());
    if (grad) NCK(cudaMemcpyAsync(grad, n->G, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    double l = 0;
    NCK(cudaMemcpyAsync(&l, n->dloss, sizeof(double), cudaMemcpyDeviceToHost, n->stream));
    NCK(cudaStreamSynchronize(n->stream));
    if (loss) *loss = l / ((double)ntok * OUT);
    return MLF_OK;
}

// Adam on minibatches of `batch` tokens drawn (hashed, with replacement) from
// X[ntok][16], T[ntok][2] (device); loss_hist[steps] (host, optional) gets
// each step's minibatch loss.
int mlf_mlp_train(mlf_mlp* h, const float* X, const float* T, long long ntok, int steps, int batch, float lr,
                  unsigned long long seed, float* loss_hist) {
    if (!h || !X || !T || ntok <= 0 || steps <= 0 || batch <= 0 || !(lr > 0)) return MLF_E_ARG;
    Net* n = &h->n;
    NCK(cudaSetDevice(n->dev));
    long long* idx = nullptr;
    float *xg = nullptr, *tg = nullptr;
    double* dl = nullptr;
    const int grid = grid_for(batch);
    NCK(cudaMalloc(&idx, batch * sizeof(long long)));
    NCK(cudaMalloc(&xg, (size_t)grid * TT * IN * sizeof(float)));
    NCK(cudaMalloc(&tg, (size_t)grid * TT * OUT * sizeof(float)));
    NCK(cudaMalloc(&dl, steps * sizeof(double)));
    NCK(cudaMemsetAsync(dl, 0, steps * sizeof(double), n->stream));
    const float scale = (float)(1.0 / ((double)batch * OUT));
    for (int st = 0; st < steps; ++st) {
        k_batch_idx<<<(batch + 255) / 256, 256, 0, n->stream>>>(batch, ntok, seed, st, idx);
        cudaMemsetAsync(n->G, 0, NPARAM * sizeof(float), n->stream);
        k_mlp_grad<<<grid, 256, sizeof(Smem), n->stream>>>(batch, idx, X, T, n->norm, n->Pb, scale, n->G, dl + st, xg,
                                                           tg);
        ++n->adam_t;
        const float c1 = 1.f / (1.f - std::pow(0.9f, (float)n->adam_t));
        const float c2 = 1.f / (1.f - std::pow(0.999f, (float)n->adam_t));
        k_adam<<<(NPARAM + 255) / 256, 256, 0, n->stream>>>(NPARAM, n->P, n->G, n->M1, n->M2, n->Pb, lr, c1, c2);
    }
    NCK(cudaGetLastError());
    std::vector<double> lh(steps);
    NCK(cudaMemcpyAsync(lh.data(), dl, steps * sizeof(double), cudaMemcpyDeviceToHost, n->stream));
    NCK(cudaStreamSynchronize(n->stream));
    if (loss_hist)
        for (int st = 0; st < steps; ++st) loss_hist[st] = (float)(lh[st] / ((double)batch * OUT));
    cudaFree(idx);
    cudaFree(xg);
    cudaFree(tg);
    cudaFree(dl);
    return MLF_OK;
}

}  // extern "C"
