// Surrogate MLP of the force-indentation curve (C ABI nfx_mlp_*): material parameters ->
// curve samples, layers n_in -> width x depth -> n_out with SiLU between them. Weights and
// activations are BF16, every product is accumulated in FP32 by warp-level tensor-core MMAs
// (mma.sync m16n8k16, BF16 inputs, FP32 accumulators), the optimizer keeps FP32 master weights
// (AdamW). The reference has no learned part; this is the project's own.
//
// Every matrix product is one "TN" kernel, C[M,N] = A[M,K] * B[N,K]^T, whose two operands are
// stored with the reduction index contiguous. Forward and backward keep the layouts that make
// all three products of a layer TN:
//   forward        Z = X W^T + b        A = X   [M,K]   B = W   [N,K]
//   input grad     dX = dZ W            A = dZ  [M,N]   B = W^T [K,N]   (W^T kept beside W)
//   weight grad    dW = dZ^T X          A = dZ^T[N,M]   B = X^T [K,M]   (transposed copies
//                                                                        written by epilogues)
// so the epilogues write activations and gradients in both layouts.
//
// Optional output gain: y = exp(alpha * x_k) * (W_L a + b_L) for one input k (nfx_mlp_set_output_gain).
// With x_k the logarithm of a scale the curves are proportional to, the network itself only has
// to learn the scale-free shape, while outputs and input gradients stay those of y.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/nfx.h"
#include "nfx_internal.h"

namespace {

using bf16 = __nv_bfloat16;

int mfail(int code, const std::string& msg) {
    nfx::set_error(msg);
    return code;
}

#define MCUDA(expr)                                                                                         \
    do {                                                                                                    \
        cudaError_t e_ = (expr);                                                                            \
        if (e_ != cudaSuccess) return mfail(NFX_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define MARG(cond, msg)                              \
    do {                                             \
        if (!(cond)) return mfail(NFX_ERR_ARG, msg); \
    } while (0)

constexpr int MLP_MAX_LAYERS = 8;
constexpr int MLP_MAX_WIDTH = 1024;

// ---------------------------------------------------------------------------------------
// GEMM: C[M,N] = A[M,K] B[N,K]^T, BF16 operands, FP32 accumulation, fused epilogue.
// A block of 4 warps covers 64 rows x 64 columns, each warp 32 x 32 (two m16 row groups x four
// n8 column groups of mma.sync m16n8k16). K advances in chunks of 64 through two shared-memory
// stages filled by cp.async (16-byte copies, zero-filled past M, N or K), so a chunk's global
// loads overlap the previous chunk's MMAs. lda/ldb must be multiples of 8 and the operands
// 16-byte aligned. Any K works: columns at or past K read as zero (the weight-gradient products
// reduce over the batch, whose transposed buffers hold stale columns beyond it).
// ---------------------------------------------------------------------------------------
enum Epi : int {
    EPI_HIDDEN = 0,       // z = acc + b: Z (f32) stored; a = silu(z) stored as bf16 [M,N] and [N,M]
    EPI_OUTPUT = 1,       // y = acc + b stored as f32 [M,N]
    EPI_GRAD_HIDDEN = 2,  // g = acc * silu'(Zp[m,n]) stored as bf16 [M,N] and [N,M]
    EPI_GRAD_INPUT = 3,   // acc stored as f32 [M,N]
    EPI_WGRAD = 4,        // acc stored as f32 [M,N]; with bias_out, column bias_col to bias_out[M]
};

struct EpiArgs {
    const float* bias;  // [N]
    const float* zp;    // [M,N] pre-activations (EPI_GRAD_HIDDEN)
    float* out_f;       // [M,N]
    bf16* out_b;        // [M,N]
    bf16* out_bt;       // [N,M]
    int ldo, ldot;      // leading dimensions of out and its transpose
    const float* gain_x;  // EPI_OUTPUT: inputs [M, gain_ld]; null: no gain
    int gain_ld, gain_k;
    float gain_alpha;
    const float* gain_dx;  // EPI_GRAD_INPUT: per-row term added to column gain_k; null: none
    float* bias_out;       // EPI_WGRAD: column bias_col goes to bias_out[m] (the bias gradient)
    int bias_col;
};

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

constexpr int GB_M = 64, GB_N = 64, GB_K = 64;
// Staged rows are padded to 72 elements (144 B): a warp's fragment loads (rows g = 0..7, pairs
// q = 0..3 at word 36 g + q) then fall on 32 distinct banks.
constexpr int GB_LD = GB_K + 8;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Stage rows [r0, r0 + 64) x columns [k0, k0 + GB_K) of a row-major BF16 matrix (rows x K, leading
// dimension ld) into s[64][GB_LD]: 512 copies of 8 elements, 4 per thread. Copies past the matrix
// read nothing (source size 0, from the matrix's own aligned base) and fill zeros.
__device__ __forceinline__ void stage_tile(bf16* s, const bf16* g, int ld, int r0, int rows, int k0, int K) {
#pragma unroll
    for (int c = threadIdx.x; c < 64 * (GB_K / 8); c += 128) {
        const int r = c / (GB_K / 8), kc = (c % (GB_K / 8)) * 8;
        const int row = r0 + r, k = k0 + kc;
        int bytes = 0;
        const bf16* src = g;
        if (row < rows && k < K) {
            bytes = min(8, K - k) * 2;
            src = g + (size_t)row * ld + k;
        }
        cp_async16(s + r * GB_LD + kc, src, bytes);
    }
}

__device__ __forceinline__ unsigned lds_pair(const bf16* p) { return *reinterpret_cast<const unsigned*>(p); }

__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void epi_store(int epi, const EpiArgs& e, int m, int n, int M, int N, float acc) {
    if (m >= M || n >= N) return;
    switch (epi) {
        case EPI_HIDDEN: {
            const float z = acc + e.bias[n];
            e.out_f[(size_t)m * e.ldo + n] = z;
            const bf16 a = __float2bfloat16_rn(silu_f(z));
            e.out_b[(size_t)m * e.ldo + n] = a;
            e.out_bt[(size_t)n * e.ldot + m] = a;
            break;
        }
        case EPI_OUTPUT: {
            float y = acc + e.bias[n];
            if (e.gain_x) y *= expf(e.gain_alpha * e.gain_x[(size_t)m * e.gain_ld + e.gain_k]);
            e.out_f[(size_t)m * e.ldo + n] = y;
            break;
        }
        case EPI_GRAD_INPUT: {
            float g = acc;
            if (e.gain_dx && n == e.gain_k) g += e.gain_dx[m];
            e.out_f[(size_t)m * e.ldo + n] = g;
            break;
        }
        case EPI_GRAD_HIDDEN: {
            const bf16 g = __float2bfloat16_rn(acc * silu_grad(e.zp[(size_t)m * e.ldo + n]));
            e.out_b[(size_t)m * e.ldo + n] = g;
            e.out_bt[(size_t)n * e.ldot + m] = g;
            break;
        }
        default:
            if (e.bias_out && n == e.bias_col)
                e.bias_out[m] = acc;
            else
                e.out_f[(size_t)m * e.ldo + n] = acc;
            break;
    }
}

__global__ void __launch_bounds__(128) k_gemm_tn(int M, int N, int K, const bf16* __restrict__ A, int lda,
                                                 const bf16* __restrict__ B, int ldb, int epi, EpiArgs e) {
    __shared__ __align__(16) bf16 sA[2][GB_M * GB_LD];
    __shared__ __align__(16) bf16 sB[2][GB_N * GB_LD];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, q = lane & 3;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int m0 = blockIdx.x * GB_M, n0 = blockIdx.y * GB_N;
    float c[2][4][4] = {};
    const int nk = (K + GB_K - 1) / GB_K;
    stage_tile(sA[0], A, lda, m0, M, 0, K);
    stage_tile(sB[0], B, ldb, n0, N, 0, K);
    cp_async_commit();
    for (int kc = 0; kc < nk; kc++) {
        const int cur = kc & 1;
        if (kc + 1 < nk) {
            stage_tile(sA[cur ^ 1], A, lda, m0, M, (kc + 1) * GB_K, K);
            stage_tile(sB[cur ^ 1], B, ldb, n0, N, (kc + 1) * GB_K, K);
        }
        cp_async_commit();
        cp_async_wait_prev();  // every group but the newest has landed: chunk kc is staged
        __syncthreads();
        const bf16* as = sA[cur];
        const bf16* bs = sB[cur];
#pragma unroll
        for (int ks = 0; ks < GB_K; ks += 16) {
            unsigned af[2][4];
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const bf16* r0 = as + (wm + i * 16 + g) * GB_LD + ks + 2 * q;
                const bf16* r8 = r0 + 8 * GB_LD;
                af[i][0] = lds_pair(r0);
                af[i][1] = lds_pair(r8);
                af[i][2] = lds_pair(r0 + 8);
                af[i][3] = lds_pair(r8 + 8);
            }
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const bf16* rb = bs + (wn + t * 8 + g) * GB_LD + ks + 2 * q;
                const unsigned b0 = lds_pair(rb), b1 = lds_pair(rb + 8);
                mma_bf16(c[0][t], af[0], b0, b1);
                mma_bf16(c[1][t], af[1], b0, b1);
            }
        }
        __syncthreads();  // the stage is read out before the next iteration refills it
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const int ra = m0 + wm + i * 16 + g, rb = ra + 8;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int n = n0 + wn + t * 8 + 2 * q;
            epi_store(epi, e, ra, n, M, N, c[i][t][0]);
            epi_store(epi, e, ra, n + 1, M, N, c[i][t][1]);
            epi_store(epi, e, rb, n, M, N, c[i][t][2]);
            epi_store(epi, e, rb, n + 1, M, N, c[i][t][3]);
        }
    }
}

// The training loop's step index: *base + k, where base is a device counter that a captured
// chunk of k = 0 .. G-1 steps advances at its end (so one CUDA graph serves every chunk).
__device__ __forceinline__ long long train_step(const long long* base, int k) { return *base + k; }

__global__ void k_advance_counter(long long* base, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *base += n;
}

__global__ void k_fill_bf16(bf16* p, int n, float v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = __float2bfloat16_rn(v);
}

// One training step's minibatch: rows idx[s * M + r] of the dataset's inputs, targets and weights
// into the staged batch, and the inputs packed as layer 0's BF16 operands X [M, kp] and X^T
// [kp, ldt] (zero-padded), in one launch. One thread per (row, column) of kp + n_out + 1 columns.
__global__ void k_gather_pack(int M, int n_in, int kp, int n_out, const int* __restrict__ idx,
                              const long long* __restrict__ base, int k, const float* __restrict__ x_all,
                              const float* __restrict__ t_all, const float* __restrict__ w_all, float* __restrict__ xin,
                              float* __restrict__ tgt, float* __restrict__ wts, bf16* __restrict__ X,
                              bf16* __restrict__ Xt, int ldt) {
    const int cols = kp + n_out + 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * cols) return;
    const int r = i / cols, c = i % cols;
    const long long row = idx[train_step(base, k) * M + r];
    if (c < kp) {
        const float v = c < n_in ? x_all[row * n_in + c] : 0.f;
        if (c < n_in) xin[(size_t)r * n_in + c] = v;
        const bf16 b = __float2bfloat16_rn(v);
        X[(size_t)r * kp + c] = b;
        Xt[(size_t)c * ldt + r] = b;
    } else if (c < kp + n_out) {
        tgt[(size_t)r * n_out + (c - kp)] = t_all[row * n_out + (c - kp)];
    } else {
        wts[r] = w_all[row];
    }
}

// Inputs: x f32 [M, n_in] (row stride n_in) -> X bf16 [M, kp] and X^T [kp, ldt], zero-padded.
__global__ void k_pack_input(int M, int n_in, int kp, const float* __restrict__ x, bf16* __restrict__ X,
                             bf16* __restrict__ Xt, int ldt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * kp) return;
    const int m = i / kp, k = i % kp;
    const bf16 v = __float2bfloat16_rn(k < n_in ? x[(size_t)m * n_in + k] : 0.f);
    X[i] = v;
    Xt[(size_t)k * ldt + m] = v;
}

// Weighted squared error per sample, loss_s = w_s * sum_j (y_sj - t_sj)^2, and the gradient of
// scale * loss with respect to the last layer's output z as bf16 [M, N] and [N, M]: dL/dy =
// scale * 2 w_s (y - t), times the row's gain exp(alpha x_k) when there is one, in which case
// gdx[m] = alpha * sum_j y_j dL/dy_j (the gain's own input gradient) is written too. One warp
// per sample.
__global__ void k_loss_grad(int M, int N, const float* __restrict__ y, const float* __restrict__ tgt,
                            const float* __restrict__ w, float scale, float* __restrict__ loss, bf16* __restrict__ dy,
                            bf16* __restrict__ dyt, int ldt, const float* __restrict__ gain_x, int gain_ld, int gain_k,
                            float gain_alpha, float* __restrict__ gdx, float* __restrict__ hist,
                            const long long* __restrict__ base, int k) {
    const int m = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (m >= M) return;
    const float ws = w ? w[m] : 1.0f;
    const float gm = gain_x ? expf(gain_alpha * gain_x[(size_t)m * gain_ld + gain_k]) : 1.0f;
    float s = 0.f, sg = 0.f;
    for (int n = lane; n < N; n += 32) {
        const float yv = y[(size_t)m * N + n];
        const float d = yv - tgt[(size_t)m * N + n];
        s += d * d;
        const float dl = scale * 2.0f * ws * d;
        sg += yv * dl;
        const bf16 g = __float2bfloat16_rn(dl * gm);
        dy[(size_t)m * N + n] = g;
        dyt[(size_t)n * ldt + m] = g;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        sg += __shfl_xor_sync(0xffffffffu, sg, o);
    }
    if (lane == 0) {
        loss[m] = ws * s;
        if (hist) hist[train_step(base, k) * M + m] = ws * s;  // the training loop's loss history
        if (gain_x) gdx[m] = gain_alpha * sg;
    }
}

// AdamW on every parameter tensor of the network in one launch: a table of segments (each layer's
// weight matrix and bias vector), the grid running over their concatenation. The learning rate
// and the bias corrections either come from the host (sched = 0) or follow the training loop's
// cosine schedule at step *base + k (sched = 1): lr = lr_min + (lr0 - lr_min)(1 + cos(pi s /
// (steps - 1))) / 2, Adam step t = t0 + s + 1.
struct AdamSeg {
    float *p, *m1, *m2;
    const float* g;
    bf16 *W, *Wt;
    int N, K, kl;
    float wd;
    long long begin;  // first element in the concatenation
};
struct AdamTable {
    int nseg;
    AdamSeg seg[2 * MLP_MAX_LAYERS];
    long long total;
};
struct AdamHyper {
    float lr, b1, b2, eps, c1, c2;  // host-given values (sched = 0)
    int sched;
    float lr0, lr_min;
    long long steps, t0;
    const long long* base;
    int k;
};
__global__ void k_adamw_all(AdamTable tab, AdamHyper hp) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tab.total) return;
    int q = 0;
    while (q + 1 < tab.nseg && i >= tab.seg[q + 1].begin) q++;
    const AdamSeg& S = tab.seg[q];
    const int j = (int)(i - S.begin);
    const int n = j / S.K, kk = j % S.K;
    if (kk >= S.kl) return;
    float lr = hp.lr, c1 = hp.c1, c2 = hp.c2;
    if (hp.sched) {
        const long long st = train_step(hp.base, hp.k);
        const double frac = hp.steps > 1 ? (double)st / (double)(hp.steps - 1) : 0.0;
        lr = (float)(hp.lr_min + 0.5 * (hp.lr0 - hp.lr_min) * (1.0 + cos(3.14159265358979323846 * frac)));
        const float t = (float)(hp.t0 + st + 1);
        c1 = 1.f - powf(hp.b1, t);
        c2 = 1.f - powf(hp.b2, t);
    }
    const float g = S.g[j];
    const float a = hp.b1 * S.m1[j] + (1.f - hp.b1) * g;
    const float b = hp.b2 * S.m2[j] + (1.f - hp.b2) * g * g;
    S.m1[j] = a;
    S.m2[j] = b;
    float w = S.p[j] * (1.f - lr * S.wd);
    w -= lr * (a / c1) / (sqrtf(b / c2) + hp.eps);
    S.p[j] = w;
    if (S.W) {
        const bf16 v = __float2bfloat16_rn(w);
        S.W[j] = v;
        S.Wt[(size_t)kk * S.N + n] = v;
    }
}

__global__ void k_refresh_bf16(int N, int K, const float* __restrict__ p, bf16* __restrict__ W, bf16* __restrict__ Wt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * K) return;
    const int n = i / K, k = i % K;
    const bf16 v = __float2bfloat16_rn(p[i]);
    W[i] = v;
    Wt[(size_t)k * N + n] = v;
}

// Input-space Adam step for the inverse fit: free inputs move, fixed ones stay, all are clamped
// to [lo, hi].
__global__ void k_input_adam(int B, int n_in, float* __restrict__ x, const float* __restrict__ g, int ldg,
                             float* __restrict__ m1, float* __restrict__ m2, const unsigned char* __restrict__ free_mask,
                             const float* __restrict__ lo, const float* __restrict__ hi, float lr, float b1, float b2,
                             float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * n_in) return;
    const int r = i / n_in, k = i % n_in;
    if (!free_mask[k]) return;
    const float gg = g[(size_t)r * ldg + k];
    const float a = b1 * m1[i] + (1.f - b1) * gg;
    const float b = b2 * m2[i] + (1.f - b2) * gg * gg;
    m1[i] = a;
    m2[i] = b;
    float v = x[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    x[i] = fminf(fmaxf(v, lo[k]), hi[k]);
}

int round_up(int x, int a) { return (x + a - 1) / a * a; }

}  // namespace

// ---------------------------------------------------------------------------------------
// Handle
// ---------------------------------------------------------------------------------------
struct nfx_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    int n_in = 0, n_out = 0, width = 0, depth = 0;
    int nl = 0;                  // layers = depth + 1
    int kin[MLP_MAX_LAYERS] = {};   // stored input width of layer l (layer 0 padded to 16)
    int kl[MLP_MAX_LAYERS] = {};    // logical input width
    int nout[MLP_MAX_LAYERS] = {};  // output width
    int max_batch = 0, mb = 0;      // capacity, padded to 64
    std::vector<void*> allocs;
    // per layer: fp32 master weights/biases, grads, Adam moments; bf16 W and W^T
    float *w[MLP_MAX_LAYERS] = {}, *b[MLP_MAX_LAYERS] = {};
    float *gw[MLP_MAX_LAYERS] = {}, *gb[MLP_MAX_LAYERS] = {};
    float *mw[MLP_MAX_LAYERS] = {}, *vw[MLP_MAX_LAYERS] = {}, *mbias[MLP_MAX_LAYERS] = {}, *vbias[MLP_MAX_LAYERS] = {};
    bf16 *wb[MLP_MAX_LAYERS] = {}, *wbt[MLP_MAX_LAYERS] = {};
    // activations: X_l bf16 [mb, kin] and X_l^T [kin + 1, mb] (its last row all ones); Z_l f32
    // [mb, nout] (hidden layers)
    bf16 *x[MLP_MAX_LAYERS + 1] = {}, *xt[MLP_MAX_LAYERS + 1] = {};
    float* z[MLP_MAX_LAYERS] = {};
    float* y = nullptr;            // [mb, n_out]
    bf16 *dz = nullptr, *dzt = nullptr, *dz2 = nullptr, *dz2t = nullptr;  // ping-pong [mb, width]
    float* dx = nullptr;           // [mb, 16] input gradient
    int gain_k = -1;               // output gain exp(gain_alpha * x[gain_k]); -1: none
    float gain_alpha = 0.f;
    float* gdx = nullptr;          // [mb] the gain's input gradient
    float* loss = nullptr;         // [mb]
    float *xin = nullptr, *tgt = nullptr, *wts = nullptr;  // staged batch inputs
    long long adam_t = 0;
};

namespace {

template <class T>
int malloc_dev(nfx_mlp* h, T** p, size_t n) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return mfail(NFX_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    h->allocs.push_back(q);
    *p = (T*)q;
    return NFX_OK;
}

cudaError_t gemm(cudaStream_t st, int M, int N, int K, const bf16* A, int lda, const bf16* B, int ldb, int epi,
                 const EpiArgs& e) {
    // the staged loads copy 16-byte pieces of rows
    if (lda % 8 || ldb % 8 || (reinterpret_cast<uintptr_t>(A) & 15u) || (reinterpret_cast<uintptr_t>(B) & 15u))
        return cudaErrorMisalignedAddress;
    const dim3 grid((unsigned)((M + GB_M - 1) / GB_M), (unsigned)((N + GB_N - 1) / GB_N));
    k_gemm_tn<<<grid, 128, 0, st>>>(M, N, K, A, lda, B, ldb, epi, e);
    return cudaGetLastError();
}

// Forward over a batch already packed into x[0]/xt[0]; output in h->y.
int forward_dev(nfx_mlp* h, int M) {
    for (int l = 0; l < h->nl; l++) {
        EpiArgs e{};
        e.bias = h->b[l];
        const bool last = l == h->nl - 1;
        e.ldo = h->nout[l];
        e.ldot = h->mb;
        if (last) {
            e.out_f = h->y;
            if (h->gain_k >= 0) {
                e.gain_x = h->xin;
                e.gain_ld = h->n_in;
                e.gain_k = h->gain_k;
                e.gain_alpha = h->gain_alpha;
            }
        } else {
            e.out_f = h->z[l];
            e.out_b = h->x[l + 1];
            e.out_bt = h->xt[l + 1];
        }
        MCUDA(gemm(h->stream, M, h->nout[l], h->kin[l], h->x[l], h->kin[l], h->wb[l], h->kin[l],
                   last ? EPI_OUTPUT : EPI_HIDDEN, e));
    }
    return NFX_OK;
}

// Backward from the output gradient in dz/dzt ([M, n_out] and [n_out, mb]): weight and bias
// gradients of every layer and, when want_dx, the input gradient in h->dx.
int backward_dev(nfx_mlp* h, int M, bool want_params, bool want_dx) {
    bf16 *g = h->dz, *gt = h->dzt, *g2 = h->dz2, *g2t = h->dz2t;
    for (int l = h->nl - 1; l >= 0; l--) {
        const int N = h->nout[l], K = h->kin[l];
        if (want_params) {
            // dW = dZ^T X and, from the ones row K of X^T, the bias gradient db = dZ^T 1
            EpiArgs e{};
            e.out_f = h->gw[l];
            e.ldo = K;
            e.bias_out = h->gb[l];
            e.bias_col = K;
            MCUDA(gemm(h->stream, N, K + 1, M, gt, h->mb, h->xt[l], h->mb, EPI_WGRAD, e));
        }
        if (l > 0) {
            EpiArgs e{};
            e.zp = h->z[l - 1];
            e.out_b = g2;
            e.out_bt = g2t;
            e.ldo = K;
            e.ldot = h->mb;
            MCUDA(gemm(h->stream, M, K, N, g, N, h->wbt[l], N, EPI_GRAD_HIDDEN, e));
            std::swap(g, g2);
            std::swap(gt, g2t);
        } else if (want_dx) {
            EpiArgs e{};
            e.out_f = h->dx;
            e.ldo = K;
            if (h->gain_k >= 0) {
                e.gain_dx = h->gdx;
                e.gain_k = h->gain_k;
            }
            MCUDA(gemm(h->stream, M, K, N, g, N, h->wbt[0], N, EPI_GRAD_INPUT, e));
        }
    }
    return NFX_OK;
}

// The staged inputs h->xin [M, n_in] -> layer 0's operands.
int pack_input(nfx_mlp* h, int M) {
    const int n = M * h->kin[0];
    k_pack_input<<<(n + 255) / 256, 256, 0, h->stream>>>(M, h->n_in, h->kin[0], h->xin, h->x[0], h->xt[0], h->mb);
    MCUDA(cudaGetLastError());
    return NFX_OK;
}

// hist/base/k: the training loop's loss history, indexed by its device step counter (null: none).
int loss_grad(nfx_mlp* h, int M, const float* tgt_dev, const float* w_dev, float scale, float* hist = nullptr,
              const long long* base = nullptr, int k = 0) {
    const bool gain = h->gain_k >= 0;
    k_loss_grad<<<(M + 7) / 8, 256, 0, h->stream>>>(M, h->n_out, h->y, tgt_dev, w_dev, scale, h->loss, h->dz, h->dzt,
                                                    h->mb, gain ? h->xin : nullptr, h->n_in, h->gain_k,
                                                    h->gain_alpha, h->gdx, hist, base, k);
    MCUDA(cudaGetLastError());
    return NFX_OK;
}

// The segment table of every parameter tensor (weights with decay wd, biases without).
AdamTable adam_table(nfx_mlp* h, float wd) {
    AdamTable t{};
    long long pos = 0;
    for (int l = 0; l < h->nl; l++) {
        const int N = h->nout[l], K = h->kin[l];
        t.seg[t.nseg++] = AdamSeg{h->w[l], h->mw[l], h->vw[l], h->gw[l], h->wb[l], h->wbt[l], N, K, h->kl[l], wd, pos};
        pos += (long long)N * K;
        t.seg[t.nseg++] = AdamSeg{h->b[l], h->mbias[l], h->vbias[l], h->gb[l], nullptr, nullptr, N, 1, 1, 0.f, pos};
        pos += N;
    }
    t.total = pos;
    return t;
}

int adamw_launch(nfx_mlp* h, const AdamTable& t, const AdamHyper& hp) {
    k_adamw_all<<<(unsigned)((t.total + 255) / 256), 256, 0, h->stream>>>(t, hp);
    MCUDA(cudaGetLastError());
    return NFX_OK;
}

int adamw_dev(nfx_mlp* h, float lr, float b1, float b2, float eps, float wd) {
    h->adam_t++;
    AdamHyper hp{};
    hp.lr = lr;
    hp.b1 = b1;
    hp.b2 = b2;
    hp.eps = eps;
    hp.c1 = 1.f - std::pow(b1, (float)h->adam_t);
    hp.c2 = 1.f - std::pow(b2, (float)h->adam_t);
    return adamw_launch(h, adam_table(h, wd), hp);
}

int check_batch(nfx_mlp* h, int64_t B) {
    MARG(B > 0 && B <= h->max_batch, "batch size must be in 1..max_batch");
    return NFX_OK;
}

}  // namespace

extern "C" {

int nfx_mlp_create(int device, int n_in, int width, int depth, int n_out, int64_t max_batch, nfx_mlp** out) {
    MARG(out, "out is null");
    *out = nullptr;
    MARG(n_in >= 1 && n_in <= 16, "n_in must be 1..16");
    MARG(width >= 16 && width <= MLP_MAX_WIDTH && width % 16 == 0, "width must be a multiple of 16 in 16..1024");
    MARG(depth >= 1 && depth + 1 <= MLP_MAX_LAYERS, "depth (hidden layers) must be 1..7");
    MARG(n_out >= 8 && n_out <= MLP_MAX_WIDTH && n_out % 8 == 0, "n_out must be a multiple of 8 in 8..1024");
    MARG(max_batch >= 1 && max_batch <= (1 << 20), "max_batch must be 1..2^20");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
        return mfail(NFX_ERR_NODEVICE, "no such CUDA device");
    MCUDA(cudaSetDevice(device));
    nfx_mlp* h = new nfx_mlp();
    h->device = device;
    h->n_in = n_in;
    h->n_out = n_out;
    h->width = width;
    h->depth = depth;
    h->nl = depth + 1;
    h->max_batch = (int)max_batch;
    h->mb = round_up((int)max_batch, 64);
    for (int l = 0; l < h->nl; l++) {
        h->kin[l] = l == 0 ? 16 : width;
        h->kl[l] = l == 0 ? n_in : width;
        h->nout[l] = l == h->nl - 1 ? n_out : width;
    }
    int rc = NFX_OK;
    auto fail_out = [&](int code) {
        nfx_mlp_destroy(h);
        return code;
    };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return fail_out(mfail(NFX_ERR_CUDA, "stream"));
    const size_t mb = (size_t)h->mb;
    for (int l = 0; l < h->nl; l++) {
        const size_t nk = (size_t)h->nout[l] * h->kin[l], n = (size_t)h->nout[l];
        if ((rc = malloc_dev(h, &h->w[l], nk)) || (rc = malloc_dev(h, &h->gw[l], nk)) || (rc = malloc_dev(h, &h->mw[l], nk)) ||
            (rc = malloc_dev(h, &h->vw[l], nk)) || (rc = malloc_dev(h, &h->b[l], n)) || (rc = malloc_dev(h, &h->gb[l], n)) ||
            (rc = malloc_dev(h, &h->mbias[l], n)) || (rc = malloc_dev(h, &h->vbias[l], n)) ||
            (rc = malloc_dev(h, &h->wb[l], nk)) || (rc = malloc_dev(h, &h->wbt[l], nk)) ||
            (rc = malloc_dev(h, &h->x[l], mb * h->kin[l])) || (rc = malloc_dev(h, &h->xt[l], mb * (h->kin[l] + 1))))
            return fail_out(rc);
        if (l < h->nl - 1 && (rc = malloc_dev(h, &h->z[l], mb * h->nout[l]))) return fail_out(rc);
        for (void* p : {(void*)h->w[l], (void*)h->gw[l], (void*)h->mw[l], (void*)h->vw[l], (void*)h->wb[l], (void*)h->wbt[l]})
            cudaMemsetAsync(p, 0, nk * (p == h->wb[l] || p == h->wbt[l] ? sizeof(bf16) : sizeof(float)), h->stream);
        for (void* p : {(void*)h->b[l], (void*)h->gb[l], (void*)h->mbias[l], (void*)h->vbias[l]})
            cudaMemsetAsync(p, 0, n * sizeof(float), h->stream);
        cudaMemsetAsync(h->x[l], 0, mb * h->kin[l] * sizeof(bf16), h->stream);
        cudaMemsetAsync(h->xt[l], 0, mb * h->kin[l] * sizeof(bf16), h->stream);
        // X^T carries a row of ones after its kin rows: the weight-gradient product then yields
        // the bias gradient as its last column
        k_fill_bf16<<<(unsigned)((mb + 255) / 256), 256, 0, h->stream>>>(h->xt[l] + mb * h->kin[l], (int)mb, 1.0f);
    }
    const size_t gw = (size_t)std::max(width, n_out);
    if ((rc = malloc_dev(h, &h->y, mb * n_out)) || (rc = malloc_dev(h, &h->dz, mb * gw)) || (rc = malloc_dev(h, &h->dzt, mb * gw)) ||
        (rc = malloc_dev(h, &h->dz2, mb * gw)) || (rc = malloc_dev(h, &h->dz2t, mb * gw)) || (rc = malloc_dev(h, &h->dx, mb * 16)) ||
        (rc = malloc_dev(h, &h->loss, mb)) || (rc = malloc_dev(h, &h->xin, mb * n_in)) || (rc = malloc_dev(h, &h->tgt, mb * n_out)) ||
        (rc = malloc_dev(h, &h->wts, mb)) || (rc = malloc_dev(h, &h->gdx, mb)))
        return fail_out(rc);
    // padding rows of the transposed buffers are read by the weight-gradient products: zero them
    for (void* p : {(void*)h->dz, (void*)h->dzt, (void*)h->dz2, (void*)h->dz2t})
        cudaMemsetAsync(p, 0, mb * gw * sizeof(bf16), h->stream);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail_out(mfail(NFX_ERR_CUDA, "initialisation failed"));
    *out = h;
    return NFX_OK;
}

int nfx_mlp_destroy(nfx_mlp* h) {
    if (!h) return NFX_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void* p : h->allocs) cudaFree(p);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return NFX_OK;
}

int nfx_mlp_set_output_gain(nfx_mlp* h, int input, float alpha) {
    MARG(h, "null handle");
    MARG(input >= -1 && input < h->n_in, "gain input index out of range");
    MARG(std::isfinite(alpha), "non-finite gain exponent");
    MCUDA(cudaSetDevice(h->device));
    MCUDA(cudaStreamSynchronize(h->stream));
    h->gain_k = input;
    h->gain_alpha = input >= 0 ? alpha : 0.f;
    return NFX_OK;
}

int nfx_mlp_num_params(nfx_mlp* h, int64_t* n) {
    MARG(h && n, "null argument");
    int64_t s = 0;
    for (int l = 0; l < h->nl; l++) s += (int64_t)h->nout[l] * h->kl[l] + h->nout[l];
    *n = s;
    return NFX_OK;
}

// Flat parameter layout (host, FP32): for each layer l, W_l [nout, kl] row-major then b_l [nout].
int nfx_mlp_set_params(nfx_mlp* h, const float* p) {
    MARG(h && p, "null argument");
    MCUDA(cudaSetDevice(h->device));
    MCUDA(cudaStreamSynchronize(h->stream));
    size_t off = 0;
    for (int l = 0; l < h->nl; l++) {
        const int N = h->nout[l], K = h->kin[l], kl = h->kl[l];
        std::vector<float> wpad((size_t)N * K, 0.f);
        for (int n = 0; n < N; n++)
            for (int k = 0; k < kl; k++) wpad[(size_t)n * K + k] = p[off + (size_t)n * kl + k];
        off += (size_t)N * kl;
        MCUDA(cudaMemcpy(h->w[l], wpad.data(), wpad.size() * sizeof(float), cudaMemcpyHostToDevice));
        MCUDA(cudaMemcpy(h->b[l], p + off, (size_t)N * sizeof(float), cudaMemcpyHostToDevice));
        off += N;
        k_refresh_bf16<<<(N * K + 255) / 256, 256, 0, h->stream>>>(N, K, h->w[l], h->wb[l], h->wbt[l]);
        MCUDA(cudaGetLastError());
        MCUDA(cudaMemsetAsync(h->mw[l], 0, (size_t)N * K * sizeof(float), h->stream));
        MCUDA(cudaMemsetAsync(h->vw[l], 0, (size_t)N * K * sizeof(float), h->stream));
        MCUDA(cudaMemsetAsync(h->mbias[l], 0, (size_t)N * sizeof(float), h->stream));
        MCUDA(cudaMemsetAsync(h->vbias[l], 0, (size_t)N * sizeof(float), h->stream));
    }
    h->adam_t = 0;
    MCUDA(cudaStreamSynchronize(h->stream));
    return NFX_OK;
}

static int copy_layers_out(nfx_mlp* h, float* const* wsrc, float* const* bsrc, float* p) {
    MCUDA(cudaSetDevice(h->device));
    MCUDA(cudaStreamSynchronize(h->stream));
    size_t off = 0;
    for (int l = 0; l < h->nl; l++) {
        const int N = h->nout[l], K = h->kin[l], kl = h->kl[l];
        std::vector<float> wpad((size_t)N * K);
        MCUDA(cudaMemcpy(wpad.data(), wsrc[l], wpad.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (int n = 0; n < N; n++)
            for (int k = 0; k < kl; k++) p[off + (size_t)n * kl + k] = wpad[(size_t)n * K + k];
        off += (size_t)N * kl;
        MCUDA(cudaMemcpy(p + off, bsrc[l], (size_t)N * sizeof(float), cudaMemcpyDeviceToHost));
        off += N;
    }
    return NFX_OK;
}

int nfx_mlp_get_params(nfx_mlp* h, float* p) {
    MARG(h && p, "null argument");
    return copy_layers_out(h, h->w, h->b, p);
}

int nfx_mlp_get_grads(nfx_mlp* h, float* p) {
    MARG(h && p, "null argument");
    return copy_layers_out(h, h->gw, h->gb, p);
}

int nfx_mlp_forward(nfx_mlp* h, const float* x, int64_t B, float* y) {
    MARG(h && x && y, "null argument");
    int rc;
    if ((rc = check_batch(h, B)) != NFX_OK) return rc;
    MCUDA(cudaSetDevice(h->device));
    MCUDA(cudaMemcpyAsync(h->xin, x, (size_t)B * h->n_in * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    if ((rc = pack_input(h, (int)B)) != NFX_OK || (rc = forward_dev(h, (int)B)) != NFX_OK) return rc;
    MCUDA(cudaMemcpyAsync(y, h->y, (size_t)B * h->n_out * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    MCUDA(cudaStreamSynchronize(h->stream));
    return NFX_OK;
}

int nfx_mlp_backward(nfx_mlp* h, const float* x, const float* target, const float* weight, int64_t B, float scale,
                     float* loss, float* dx) {
    MARG(h && x && target, "null argument");
    int rc;
    if ((rc = check_batch(h, B)) != NFX_OK) return rc;
    MCUDA(cudaSetDevice(h->device));
    const int M = (int)B;
    MCUDA(cudaMemcpyAsync(h->xin, x, (size_t)M * h->n_in * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    MCUDA(cudaMemcpyAsync(h->tgt, target, (size_t)M * h->n_out * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    if (weight) MCUDA(cudaMemcpyAsync(h->wts, weight, (size_t)M * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    if ((rc = pack_input(h, M)) || (rc = forward_dev(h, M)) || (rc = loss_grad(h, M, h->tgt, weight ? h->wts : nullptr, scale)) ||
        (rc = backward_dev(h, M, true, dx != nullptr)))
        return rc;
    if (loss) MCUDA(cudaMemcpyAsync(loss, h->loss, (size_t)M * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    if (dx) {
        std::vector<float> tmp((size_t)M * 16);
        MCUDA(cudaMemcpyAsync(tmp.data(), h->dx, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
        MCUDA(cudaStreamSynchronize(h->stream));
        for (int m = 0; m < M; m++)
            for (int k = 0; k < h->n_in; k++) dx[(size_t)m * h->n_in + k] = tmp[(size_t)m * 16 + k];
    }
    MCUDA(cudaStreamSynchronize(h->stream));
    return NFX_OK;
}

int nfx_mlp_adamw(nfx_mlp* h, float lr, float beta1, float beta2, float eps, float weight_decay) {
    MARG(h, "null handle");
    MCUDA(cudaSetDevice(h->device));
    int rc;
    if ((rc = adamw_dev(h, lr, beta1, beta2, eps, weight_decay)) != NFX_OK) return rc;
    MCUDA(cudaStreamSynchronize(h->stream));
    return NFX_OK;
}

// Minibatch training on a dataset uploaded once: each step draws `batch` rows (indices from a
// PCG32 stream seeded with `seed`, without replacement inside an epoch), runs forward, the
// weighted squared-error loss (mean over the batch), backward and AdamW with a cosine learning
// rate from hp[0] down to hp[5]. hp = {lr, beta1, beta2, eps, weight_decay, lr_min}. The mean
// loss of every step is written to losses[steps].
int nfx_mlp_train(nfx_mlp* h, const float* x_all, const float* t_all, const float* w_all, int64_t n, int64_t batch,
                  int64_t steps, const float* hp, uint64_t seed, float* losses) {
    const nfx::NvtxRange range("nfx_mlp_train");
    MARG(h && x_all && t_all && hp, "null argument");
    MARG(n >= 1 && steps >= 0, "bad sizes");
    int rc;
    if ((rc = check_batch(h, batch)) != NFX_OK) return rc;
    MARG(batch <= n, "batch larger than the dataset");
    MCUDA(cudaSetDevice(h->device));
    float *dx_all = nullptr, *dt_all = nullptr, *dw_all = nullptr, *loss_hist = nullptr;
    int* d_idx = nullptr;
    std::vector<void*> tmp;
    auto cleanup = [&]() {
        cudaStreamSynchronize(h->stream);
        for (void* p : tmp) cudaFree(p);
    };
    auto alloc = [&](auto** p, size_t bytes) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(bytes, 4)) != cudaSuccess) return false;
        tmp.push_back(q);
        *p = (std::remove_reference_t<decltype(*p)>)q;
        return true;
    };
    if (!alloc(&dx_all, (size_t)n * h->n_in * 4) || !alloc(&dt_all, (size_t)n * h->n_out * 4) ||
        !alloc(&dw_all, (size_t)n * 4) || !alloc(&d_idx, (size_t)steps * batch * 4 + 4) ||
        !alloc(&loss_hist, (size_t)std::max<int64_t>(steps, 1) * batch * 4)) {
        cleanup();
        return mfail(NFX_ERR_NOMEM, "cudaMalloc failed for the training set");
    }
    // index stream: epochs of a PCG32-driven Fisher-Yates shuffle
    std::vector<int> idx((size_t)steps * batch);
    {
        uint64_t state = seed * 6364136223846793005ull + 1442695040888963407ull;
        auto next = [&]() {
            const uint64_t old = state;
            state = old * 6364136223846793005ull + 1442695040888963407ull;
            const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u), rot = (uint32_t)(old >> 59u);
            return (xs >> rot) | (xs << ((32u - rot) & 31u));
        };
        std::vector<int> perm((size_t)n);
        for (int64_t i = 0; i < n; i++) perm[i] = (int)i;
        int64_t pos = n;
        for (size_t i = 0; i < idx.size(); i++) {
            if (pos >= n) {
                for (int64_t k = n - 1; k > 0; k--) std::swap(perm[k], perm[next() % (uint32_t)(k + 1)]);
                pos = 0;
            }
            idx[i] = perm[pos++];
        }
    }
    std::vector<float> wones;
    const float* wsrc = w_all;
    if (!wsrc) {
        wones.assign((size_t)n, 1.f);
        wsrc = wones.data();
    }
    cudaStream_t st = h->stream;
    if (cudaMemcpyAsync(dx_all, x_all, (size_t)n * h->n_in * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dt_all, t_all, (size_t)n * h->n_out * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dw_all, wsrc, (size_t)n * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (steps > 0 && cudaMemcpyAsync(d_idx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice, st) != cudaSuccess)) {
        cleanup();
        return mfail(NFX_ERR_CUDA, "upload of the training set failed");
    }
    const int M = (int)batch;
    const float scale = 1.0f / (float)M;
    long long* d_base = nullptr;
    if (!alloc(&d_base, sizeof(long long))) {
        cleanup();
        return mfail(NFX_ERR_NOMEM, "cudaMalloc failed for the step counter");
    }
    if (cudaMemsetAsync(d_base, 0, sizeof(long long), st) != cudaSuccess) {
        cleanup();
        return mfail(NFX_ERR_CUDA, "step counter reset failed");
    }
    const AdamTable tab = adam_table(h, hp[4]);
    AdamHyper ahp{};
    ahp.b1 = hp[1];
    ahp.b2 = hp[2];
    ahp.eps = hp[3];
    ahp.sched = 1;
    ahp.lr0 = hp[0];
    ahp.lr_min = hp[5];
    ahp.steps = steps;
    ahp.t0 = h->adam_t;
    ahp.base = d_base;
    // One training step k of a chunk: minibatch, forward, loss (into the history), backward,
    // AdamW; 14 launches, all reading the step index from the device counter.
    auto enqueue_step = [&](int k) -> int {
        const int cols = h->kin[0] + h->n_out + 1;
        k_gather_pack<<<(unsigned)((M * cols + 255) / 256), 256, 0, st>>>(M, h->n_in, h->kin[0], h->n_out, d_idx, d_base,
                                                                         k, dx_all, dt_all, dw_all, h->xin, h->tgt,
                                                                         h->wts, h->x[0], h->xt[0], h->mb);
        MCUDA(cudaGetLastError());
        int r;
        if ((r = forward_dev(h, M)) || (r = loss_grad(h, M, h->tgt, h->wts, scale, loss_hist, d_base, k)) ||
            (r = backward_dev(h, M, true, false)))
            return r;
        AdamHyper a = ahp;
        a.k = k;
        return adamw_launch(h, tab, a);
    };
    // chunks of TRAIN_GRAPH_STEPS steps replayed as one CUDA graph, the rest launched directly
    constexpr int TRAIN_GRAPH_STEPS = 16;
    cudaGraphExec_t gexec = nullptr;
    const int64_t chunks = steps / TRAIN_GRAPH_STEPS;
    if (chunks > 0) {
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cleanup();
            return mfail(NFX_ERR_CUDA, "training graph capture failed to start");
        }
        int r = NFX_OK;
        for (int k = 0; k < TRAIN_GRAPH_STEPS && r == NFX_OK; k++) r = enqueue_step(k);
        if (r == NFX_OK) k_advance_counter<<<1, 32, 0, st>>>(d_base, TRAIN_GRAPH_STEPS);
        const cudaError_t ec = cudaStreamEndCapture(st, &g);
        if (r != NFX_OK || ec != cudaSuccess || cudaGraphInstantiate(&gexec, g, 0) != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cleanup();
            return r != NFX_OK ? r : mfail(NFX_ERR_CUDA, "training graph capture failed");
        }
        cudaGraphDestroy(g);
    }
    for (int64_t c = 0; c < chunks; c++) {
        if (cudaGraphLaunch(gexec, st) != cudaSuccess) {
            cudaGraphExecDestroy(gexec);
            cleanup();
            return mfail(NFX_ERR_CUDA, "training graph launch failed");
        }
    }
    if (gexec) cudaGraphExecDestroy(gexec);
    for (int k = 0; k < (int)(steps - chunks * TRAIN_GRAPH_STEPS); k++) {
        if ((rc = enqueue_step(k)) != NFX_OK) {
            cleanup();
            return rc;
        }
    }
    h->adam_t += steps;
    if (losses && steps > 0) {
        std::vector<float> all((size_t)steps * M);
        if (cudaMemcpyAsync(all.data(), loss_hist, all.size() * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            cleanup();
            return mfail(NFX_ERR_CUDA, "loss readback failed");
        }
        for (int64_t s = 0; s < steps; s++) {
            double acc = 0.0;
            for (int m = 0; m < M; m++) acc += all[(size_t)s * M + m];
            losses[s] = (float)(acc / M);
        }
    }
    cleanup();
    MCUDA(cudaGetLastError());
    return NFX_OK;
}

// Inverse problem through the network: for each of the B rows, Adam on the inputs x (free
// entries only, clamped to [lo, hi]) to minimise w_b * ||f(x_b) - target_b||^2. x is updated in
// place; loss[B] receives the final per-row loss. hp = {lr, beta1, beta2, eps}.
int nfx_mlp_fit_inputs(nfx_mlp* h, float* x, const float* target, const float* weight, int64_t B,
                       const unsigned char* free_mask, const float* lo, const float* hi, int64_t steps, const float* hp,
                       float* loss) {
    MARG(h && x && target && free_mask && lo && hi && hp, "null argument");
    int rc;
    if ((rc = check_batch(h, B)) != NFX_OK) return rc;
    MCUDA(cudaSetDevice(h->device));
    const int M = (int)B, ni = h->n_in;
    float *m1 = nullptr, *m2 = nullptr, *dlo = nullptr, *dhi = nullptr;
    unsigned char* dmask = nullptr;
    std::vector<void*> tmp;
    auto cleanup = [&]() {
        cudaStreamSynchronize(h->stream);
        for (void* p : tmp) cudaFree(p);
    };
    auto alloc = [&](auto** p, size_t bytes) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(bytes, 4)) != cudaSuccess) return false;
        tmp.push_back(q);
        *p = (std::remove_reference_t<decltype(*p)>)q;
        return true;
    };
    if (!alloc(&m1, (size_t)M * ni * 4) || !alloc(&m2, (size_t)M * ni * 4) || !alloc(&dlo, ni * 4) || !alloc(&dhi, ni * 4) ||
        !alloc(&dmask, ni)) {
        cleanup();
        return mfail(NFX_ERR_NOMEM, "cudaMalloc failed for the fit state");
    }
    cudaStream_t st = h->stream;
    cudaMemsetAsync(m1, 0, (size_t)M * ni * 4, st);
    cudaMemsetAsync(m2, 0, (size_t)M * ni * 4, st);
    cudaMemcpyAsync(dlo, lo, ni * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dhi, hi, ni * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dmask, free_mask, ni, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(h->xin, x, (size_t)M * ni * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(h->tgt, target, (size_t)M * h->n_out * 4, cudaMemcpyHostToDevice, st);
    if (weight) cudaMemcpyAsync(h->wts, weight, (size_t)M * 4, cudaMemcpyHostToDevice, st);
    for (int64_t s = 0; s < steps; s++) {
        if ((rc = pack_input(h, M)) || (rc = forward_dev(h, M)) ||
            (rc = loss_grad(h, M, h->tgt, weight ? h->wts : nullptr, 1.0f)) || (rc = backward_dev(h, M, false, true))) {
            cleanup();
            return rc;
        }
        const float c1 = 1.f - std::pow(hp[1], (float)(s + 1)), c2 = 1.f - std::pow(hp[2], (float)(s + 1));
        k_input_adam<<<(M * ni + 255) / 256, 256, 0, st>>>(M, ni, h->xin, h->dx, 16, m1, m2, dmask, dlo, dhi, hp[0], hp[1],
                                                          hp[2], hp[3], c1, c2);
    }
    // final loss at the returned inputs
    if ((rc = pack_input(h, M)) || (rc = forward_dev(h, M)) ||
        (rc = loss_grad(h, M, h->tgt, weight ? h->wts : nullptr, 1.0f))) {
        cleanup();
        return rc;
    }
    cudaMemcpyAsync(x, h->xin, (size_t)M * ni * 4, cudaMemcpyDeviceToHost, st);
    if (loss) cudaMemcpyAsync(loss, h->loss, (size_t)M * 4, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cleanup();
    if (e != cudaSuccess) return mfail(NFX_ERR_CUDA, std::string("fit_inputs: ") + cudaGetErrorString(e));
    MCUDA(cudaGetLastError());
    return NFX_OK;
}

}  // extern "C"
