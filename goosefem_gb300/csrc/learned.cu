// Learned preconditioner for the matrix-free static solve: a 4-layer 3x3 convolutional network
// on the structured nodal grid (NHWC: the nodevec [nnode, 2] of a Regular Quad4 mesh is the
// [H, W, 2] image), channels 4 -> 32 -> 32 -> 32 -> 2 (input: the two residual components
// scaled by their RMS, plus the nodal bulk and shear moduli), dilations 1, 2, 4, 1, ReLU after
// the first three layers. Weights are BF16, biases and every accumulation FP32.
//
//  * training kernels (CUDA cores, FP32 accumulate): forward with stored activations, backward
//    for the inputs and the weights (per-block partial sums reduced in a fixed order:
//    deterministic), masked mean-squared error, Adam;
//  * inference: the 32 -> 32 layers on the tensor cores (mma.sync m16n8k16 BF16, FP32
//    accumulate) from a shared-memory halo tile, first and last layer on the CUDA cores;
//  * the flexible CG of Notay (FCG(1)) in FP64 that applies the network as preconditioner.
#include <cuda_bf16.h>

#include <cmath>

#include "common.cuh"

namespace gfgpu {
namespace nn {

__host__ __device__ constexpr int cin_of(int l) { return l == 0 ? 4 : 32; }
__host__ __device__ constexpr int cout_of(int l) { return l == 3 ? 2 : 32; }
__host__ __device__ constexpr int dil_of(int l) { return l == 0 ? 1 : (l == 1 ? 2 : (l == 2 ? 4 : 1)); }
// parameter layout: for each layer W [9][cin][cout] then b [cout]
__host__ __device__ constexpr int w_off(int l)
{
    return l == 0 ? 0 : w_off(l - 1) + 9 * cin_of(l - 1) * cout_of(l - 1) + cout_of(l - 1);
}
__host__ __device__ constexpr int b_off(int l) { return w_off(l) + 9 * cin_of(l) * cout_of(l); }
constexpr int kParams = b_off(3) + 2;
static_assert(kParams == 20258, "parameter count");

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
template <class T>
__device__ __forceinline__ T from_f(float v);
template <>
__device__ __forceinline__ float from_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// ------------------------------------------------------------------ CUDA-core convolutions

// y[p, co] = b[co] + sum_t sum_ci x[p + dil*off_t, ci] W[t, ci, co]   (zero padding)
template <int CI, int CO, bool RELU, class TI, class TO>
__global__ void __launch_bounds__(128)
k_conv_fwd(const TI* __restrict__ X, const __nv_bfloat16* __restrict__ W,
           const float* __restrict__ bias, int dil, int B, int H, int Wd, TO* __restrict__ Y)
{
    __shared__ float Ws[9 * CI * CO];
    __shared__ float bs[CO];
    for (int i = threadIdx.x; i < 9 * CI * CO; i += blockDim.x) Ws[i] = __bfloat162float(W[i]);
    for (int i = threadIdx.x; i < CO; i += blockDim.x) bs[i] = bias[i];
    __syncthreads();
    int64_t npix = static_cast<int64_t>(B) * H * Wd;
    GF_FOR(p, npix)
    {
        int x = static_cast<int>(p % Wd);
        int y = static_cast<int>((p / Wd) % H);
        int64_t img = p / (static_cast<int64_t>(H) * Wd);
        float acc[CO];
#pragma unroll
        for (int c = 0; c < CO; ++c) acc[c] = bs[c];
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            int yy = y + dil * (t / 3 - 1), xx = x + dil * (t % 3 - 1);
            if (yy < 0 || yy >= H || xx < 0 || xx >= Wd) continue;
            const TI* xp = X + ((img * H + yy) * Wd + xx) * CI;
#pragma unroll 4
            for (int ci = 0; ci < CI; ++ci) {
                float xv = to_f(xp[ci]);
                const float* w = Ws + (t * CI + ci) * CO;
#pragma unroll
                for (int c = 0; c < CO; ++c) acc[c] = fmaf(xv, w[c], acc[c]);
            }
        }
        TO* yp = Y + p * CO;
#pragma unroll
        for (int c = 0; c < CO; ++c) yp[c] = from_f<TO>(RELU ? fmaxf(acc[c], 0.0f) : acc[c]);
    }
}

// dX[p, ci] = (sum_t sum_co dY[p - dil*off_t, co] W[t, ci, co]) * (act[p, ci] > 0)
template <int CI, int CO>
__global__ void __launch_bounds__(128)
k_conv_bwd_data(const float* __restrict__ dY, const __nv_bfloat16* __restrict__ W, int dil, int B,
                int H, int Wd, const float* __restrict__ act, float* __restrict__ dX)
{
    __shared__ float Ws[9 * CI * CO];
    for (int i = threadIdx.x; i < 9 * CI * CO; i += blockDim.x) Ws[i] = __bfloat162float(W[i]);
    __syncthreads();
    int64_t npix = static_cast<int64_t>(B) * H * Wd;
    GF_FOR(p, npix)
    {
        int x = static_cast<int>(p % Wd);
        int y = static_cast<int>((p / Wd) % H);
        int64_t img = p / (static_cast<int64_t>(H) * Wd);
        float acc[CI];
#pragma unroll
        for (int c = 0; c < CI; ++c) acc[c] = 0.0f;
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            int yy = y - dil * (t / 3 - 1), xx = x - dil * (t % 3 - 1);
            if (yy < 0 || yy >= H || xx < 0 || xx >= Wd) continue;
            const float* gp = dY + ((img * H + yy) * Wd + xx) * CO;
#pragma unroll 4
            for (int co = 0; co < CO; ++co) {
                float g = gp[co];
#pragma unroll
                for (int ci = 0; ci < CI; ++ci) acc[ci] = fmaf(g, Ws[(t * CI + ci) * CO + co], acc[ci]);
            }
        }
        const float* ap = act + p * CI;
        float* o = dX + p * CI;
#pragma unroll
        for (int ci = 0; ci < CI; ++ci) o[ci] = ap[ci] > 0.0f ? acc[ci] : 0.0f;
    }
}

// Per-block partial sums of dW[t, ci, co] = sum_p x[p + dil*off_t, ci] dY[p, co] and
// db[co] = sum_p dY[p, co] over the block's contiguous pixel range. Thread (t, ci) owns the CO
// weights of its row; threads < CO also own one bias. partial: [gridDim.x][9*CI*CO + CO].
template <int CI, int CO>
__global__ void k_conv_bwd_weight(const float* __restrict__ X, const float* __restrict__ dY,
                                  int dil, int B, int H, int Wd, float* __restrict__ partial)
{
    constexpr int TILE = 32;
    __shared__ float gs[TILE][CO];
    int64_t npix = static_cast<int64_t>(B) * H * Wd;
    int64_t per = (npix + gridDim.x - 1) / gridDim.x;
    int64_t p0 = blockIdx.x * per;
    int64_t p1 = p0 + per < npix ? p0 + per : npix;
    int row = threadIdx.x; // (t, ci)
    int t = row / CI, ci = row % CI;
    bool owner = row < 9 * CI;
    int dy = dil * (t / 3 - 1), dx = dil * (t % 3 - 1);
    float acc[CO];
#pragma unroll
    for (int c = 0; c < CO; ++c) acc[c] = 0.0f;
    float bacc = 0.0f;
    for (int64_t base = p0; base < p1; base += TILE) {
        int n = p1 - base < TILE ? static_cast<int>(p1 - base) : TILE;
        __syncthreads();
        for (int i = threadIdx.x; i < n * CO; i += blockDim.x) gs[i / CO][i % CO] = dY[(base + i / CO) * CO + i % CO];
        __syncthreads();
        if (owner) {
            for (int k = 0; k < n; ++k) {
                int64_t p = base + k;
                int x = static_cast<int>(p % Wd);
                int y = static_cast<int>((p / Wd) % H);
                int yy = y + dy, xx = x + dx;
                if (yy < 0 || yy >= H || xx < 0 || xx >= Wd) continue;
                int64_t img = p / (static_cast<int64_t>(H) * Wd);
                float xv = X[((img * H + yy) * Wd + xx) * CI + ci];
#pragma unroll
                for (int c = 0; c < CO; ++c) acc[c] = fmaf(xv, gs[k][c], acc[c]);
            }
        }
        if (threadIdx.x < CO)
            for (int k = 0; k < n; ++k) bacc += gs[k][threadIdx.x];
    }
    float* out = partial + static_cast<int64_t>(blockIdx.x) * (9 * CI * CO + CO);
    if (owner)
#pragma unroll
        for (int c = 0; c < CO; ++c) out[row * CO + c] = acc[c];
    if (threadIdx.x < CO) out[9 * CI * CO + threadIdx.x] = bacc;
}

// out[i] = sum over blocks of partial[b][i], in block order (deterministic)
__global__ void k_sum_partials(const float* __restrict__ partial, int nblk, int n,
                               float* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int b = 0; b < nblk; ++b) s += partial[static_cast<int64_t>(b) * n + i];
    out[i] = s;
}

// masked MSE over the crop interior [m, S-m)^2: dY = 2 (y - t) / N, per-block loss partials
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, int B, int S,
                      int m, int C, float* __restrict__ dY, float* __restrict__ lpart)
{
    __shared__ float sh[256];
    int64_t n = static_cast<int64_t>(B) * S * S * C;
    float N = static_cast<float>(B) * (S - 2 * m) * (S - 2 * m) * C;
    float acc = 0.0f;
    GF_FOR(i, n)
    {
        int64_t p = i / C;
        int x = static_cast<int>(p % S), y = static_cast<int>((p / S) % S);
        bool in = x >= m && x < S - m && y >= m && y < S - m;
        float d = in ? Y[i] - T[i] : 0.0f;
        dY[i] = 2.0f * d / N;
        acc += d * d / N;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) lpart[blockIdx.x] = sh[0];
}

// Adam on the FP32 master parameters; the BF16 copy feeds the convolutions.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2, __nv_bfloat16* __restrict__ pb)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float mi = b1 * m[i] + (1.0f - b1) * g[i];
    float vi = b2 * v[i] + (1.0f - b2) * g[i] * g[i];
    m[i] = mi;
    v[i] = vi;
    float w = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = w;
    pb[i] = __float2bfloat16_rn(w);
}

// crops [B, S, S, 4] (scaled residual + material) and targets [B, S, S, 2] from the stored pairs
__global__ void k_gather_crops(const float* __restrict__ R, const float* __restrict__ Tg,
                               const float* __restrict__ mat, const int* __restrict__ pos, int B,
                               int S, int H, int Wd, float* __restrict__ X, float* __restrict__ T)
{
    int64_t n = static_cast<int64_t>(B) * S * S;
    GF_FOR(i, n)
    {
        int b = static_cast<int>(i / (static_cast<int64_t>(S) * S));
        int y = static_cast<int>((i / S) % S), x = static_cast<int>(i % S);
        int pair = pos[3 * b], yy = pos[3 * b + 1] + y, xx = pos[3 * b + 2] + x;
        bool in = yy >= 0 && yy < H && xx >= 0 && xx < Wd;
        int64_t q = (static_cast<int64_t>(pair) * H + yy) * Wd + xx;
        int64_t g = static_cast<int64_t>(yy) * Wd + xx;
        X[i * 4 + 0] = in ? R[q * 2 + 0] : 0.0f;
        X[i * 4 + 1] = in ? R[q * 2 + 1] : 0.0f;
        X[i * 4 + 2] = in ? mat[g * 2 + 0] : 0.0f;
        X[i * 4 + 3] = in ? mat[g * 2 + 1] : 0.0f;
        T[i * 2 + 0] = in ? Tg[q * 2 + 0] : 0.0f;
        T[i * 2 + 1] = in ? Tg[q * 2 + 1] : 0.0f;
    }
}

// ------------------------------------------------------------------ tensor-core 32 -> 32 layer

// Weights in shared memory as [t][co][ci] with the ci row padded to 40 BF16 (80 B): the 32-bit
// fragment loads of 8 rows x 4 column pairs then hit 32 different banks.
constexpr int kPadC = 40;
constexpr int kTileY = 8, kTileX = 16;

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Y = relu(conv(X, W) + b) for 32 -> 32 channels, X and Y BF16 [H, W, 32]. CTA: 128 threads,
// output tile 8 rows x 16 columns; warp w computes rows 2w, 2w+1 (one m16 tile of 16 pixels
// each) for the 4 n8 tiles of output channels, K = 9 taps x 32 input channels.
__global__ void __launch_bounds__(128)
k_conv32_mma(const __nv_bfloat16* __restrict__ X, const __nv_bfloat16* __restrict__ W,
             const float* __restrict__ bias, int dil, int H, int Wd, __nv_bfloat16* __restrict__ Y)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int hh = kTileY + 2 * dil, hw = kTileX + 2 * dil;
    __nv_bfloat16* halo = reinterpret_cast<__nv_bfloat16*>(smem);          // [hh][hw][40]
    __nv_bfloat16* ws = halo + hh * hw * kPadC;                             // [9][32][40]
    const int y0 = blockIdx.y * kTileY, x0 = blockIdx.x * kTileX;
    // weights: W [t][ci][co] -> ws [t][co][ci]
    for (int i = threadIdx.x; i < 9 * 32 * 32; i += blockDim.x) {
        int t = i / 1024, ci = (i / 32) % 32, co = i % 32;
        ws[(t * 32 + co) * kPadC + ci] = W[i];
    }
    // halo: 16-byte chunks (8 channels)
    for (int i = threadIdx.x; i < hh * hw * 4; i += blockDim.x) {
        int pix = i >> 2, ch = (i & 3) * 8;
        int yy = y0 - dil + pix / hw, xx = x0 - dil + pix % hw;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (yy >= 0 && yy < H && xx >= 0 && xx < Wd)
            v = *reinterpret_cast<const uint4*>(X + (static_cast<int64_t>(yy) * Wd + xx) * 32 + ch);
        *reinterpret_cast<uint4*>(halo + pix * kPadC + ch) = v;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    float c[2][4][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int k = 0; k < 4; ++k) c[mt][nt][k] = 0.0f;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int dy = dil * (t / 3 - 1), dx = dil * (t % 3 - 1);
#pragma unroll
        for (int kc = 0; kc < 2; ++kc) {
            uint32_t b[4][2];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const __nv_bfloat16* wp = ws + (t * 32 + nt * 8 + gid) * kPadC + kc * 16 + tig * 2;
                b[nt][0] = *reinterpret_cast<const uint32_t*>(wp);
                b[nt][1] = *reinterpret_cast<const uint32_t*>(wp + 8);
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int hr = 2 * warp + mt + dil + dy;
                const __nv_bfloat16* ap0 = halo + (hr * hw + gid + dil + dx) * kPadC + kc * 16 + tig * 2;
                const __nv_bfloat16* ap1 = ap0 + 8 * kPadC;
                uint32_t a0 = *reinterpret_cast<const uint32_t*>(ap0);
                uint32_t a1 = *reinterpret_cast<const uint32_t*>(ap1);
                uint32_t a2 = *reinterpret_cast<const uint32_t*>(ap0 + 8);
                uint32_t a3 = *reinterpret_cast<const uint32_t*>(ap1 + 8);
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) mma_bf16(c[mt][nt], a0, a1, a2, a3, b[nt][0], b[nt][1]);
            }
        }
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int yy = y0 + 2 * warp + mt;
        if (yy >= H) continue;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int xx = x0 + gid + 8 * half;
            if (xx >= Wd) continue;
            __nv_bfloat16* yp = Y + (static_cast<int64_t>(yy) * Wd + xx) * 32;
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int co = nt * 8 + tig * 2;
                float v0 = fmaxf(c[mt][nt][2 * half + 0] + bias[co], 0.0f);
                float v1 = fmaxf(c[mt][nt][2 * half + 1] + bias[co + 1], 0.0f);
                *reinterpret_cast<__nv_bfloat162*>(yp + co) = __floats2bfloat162_rn(v0, v1);
            }
        }
    }
}

inline size_t mma_smem_bytes(int dil)
{
    return static_cast<size_t>((kTileY + 2 * dil) * (kTileX + 2 * dil) + 9 * 32) * kPadC * 2;
}

// ------------------------------------------------------------------ preconditioner glue (FP64)

// network input from the FP64 residual nodevec: (r / sigma, K_node, G_node), sigma = sqrt(rr/n)
__global__ void k_nn_input(const double* __restrict__ r, const float* __restrict__ mat,
                           const double* __restrict__ sc, int rr_slot, double nfree, int64_t nnode,
                           float* __restrict__ X0)
{
    double sigma = sqrt(sc[rr_slot] / nfree);
    double inv = sigma > 0.0 ? 1.0 / sigma : 0.0;
    GF_FOR(p, nnode)
    {
        X0[p * 4 + 0] = static_cast<float>(r[2 * p] * inv);
        X0[p * 4 + 1] = static_cast<float>(r[2 * p + 1] * inv);
        X0[p * 4 + 2] = mat[2 * p];
        X0[p * 4 + 3] = mat[2 * p + 1];
    }
}

// z = sigma * y on the free dofs, 0 on the prescribed dofs
__global__ void k_nn_output(const float* __restrict__ y, const double* __restrict__ sc, int rr_slot,
                            double nfree, const int32_t* __restrict__ part, int64_t nnu, int64_t n,
                            double* __restrict__ z)
{
    double sigma = sqrt(sc[rr_slot] / nfree);
    GF_FOR(t, n) z[t] = part[t] < nnu ? sigma * static_cast<double>(y[t]) : 0.0;
}

} // namespace nn
} // namespace gfgpu

// ====================================================================== host side

using namespace gfgpu;
using namespace gfgpu::nn;

// element-kernel launch shared with the explicit step (dynamics.cu)
int gfgpu_internal_element_forces(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                  cudaStream_t s);

namespace gfgpu {
namespace nn {

constexpr int kWgtBlocks = 256; // fixed partition of the weight-gradient reduction
constexpr int kRed = 1024;      // fixed grid of the FCG reductions

inline int64_t a256(int64_t b)
{
    return (b + 255) / 256 * 256;
}

inline unsigned pix_grid(int64_t npix)
{
    int64_t g = (npix + 127) / 128;
    return static_cast<unsigned>(g < 1 ? 1 : (g > 65535 * 4 ? 65535 * 4 : g));
}

struct TrainWs {
    float *a1, *a2, *a3, *y, *g3, *g2, *g1, *partial, *lpart;
};

inline TrainWs carve_train(void* ws, int64_t npix)
{
    char* c = static_cast<char*>(ws);
    TrainWs w;
    float** bufs[] = {&w.a1, &w.a2, &w.a3, &w.g2, &w.g1};
    for (auto b : bufs) {
        *b = reinterpret_cast<float*>(c);
        c += a256(npix * 32 * 4);
    }
    w.y = reinterpret_cast<float*>(c);
    c += a256(npix * 2 * 4);
    w.g3 = reinterpret_cast<float*>(c);
    c += a256(npix * 2 * 4);
    w.partial = reinterpret_cast<float*>(c);
    c += a256(int64_t(kWgtBlocks) * (9 * 32 * 32 + 32) * 4);
    w.lpart = reinterpret_cast<float*>(c);
    return w;
}

inline int64_t train_bytes(int64_t npix)
{
    return 5 * a256(npix * 32 * 4) + 2 * a256(npix * 2 * 4) +
           a256(int64_t(kWgtBlocks) * (9 * 32 * 32 + 32) * 4) + a256(1024 * 4 + 16);
}

inline const __nv_bfloat16* wb(const void* p, int l)
{
    return static_cast<const __nv_bfloat16*>(p) + w_off(l);
}

// forward of the four layers in FP32 on B images of H x W, activations kept for the backward
inline void forward_f32(const void* wbf, const float* pf, const float* X, int B, int H, int W,
                        TrainWs& w, cudaStream_t s)
{
    int64_t npix = int64_t(B) * H * W;
    unsigned g = pix_grid(npix);
    k_conv_fwd<4, 32, true, float, float><<<g, 128, 0, s>>>(X, wb(wbf, 0), pf + b_off(0), dil_of(0), B, H, W, w.a1);
    k_conv_fwd<32, 32, true, float, float><<<g, 128, 0, s>>>(w.a1, wb(wbf, 1), pf + b_off(1), dil_of(1), B, H, W, w.a2);
    k_conv_fwd<32, 32, true, float, float><<<g, 128, 0, s>>>(w.a2, wb(wbf, 2), pf + b_off(2), dil_of(2), B, H, W, w.a3);
    k_conv_fwd<32, 2, false, float, float><<<g, 128, 0, s>>>(w.a3, wb(wbf, 3), pf + b_off(3), dil_of(3), B, H, W, w.y);
}

template <int CI, int CO>
inline void weight_grad(const float* X, const float* dY, int dil, int B, int H, int W, float* partial,
                        float* grad, cudaStream_t s)
{
    int threads = (9 * CI + 31) / 32 * 32;
    if (threads < CO) threads = 32;
    k_conv_bwd_weight<CI, CO><<<kWgtBlocks, threads, 0, s>>>(X, dY, dil, B, H, W, partial);
    int n = 9 * CI * CO + CO;
    k_sum_partials<<<(n + 255) / 256, 256, 0, s>>>(partial, kWgtBlocks, n, grad);
}

// ---------------------------------------------------------------- FCG kernels

enum { F_RP = 0, F_PQ, F_ZQ, F_RR, F_BB, F_ALPHA, F_BETA, F_COUNT };

__device__ __forceinline__ double bsum(double v, double* sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    if (lane == 0) sh[wi] = v;
    __syncthreads();
    double r = 0.0;
    if (wi == 0) {
        r = lane < (blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;
}

__global__ void k_fred(const double* __restrict__ partial, int nparts, double* __restrict__ sc, int slot0)
{
    __shared__ double sh[32];
    for (int p = 0; p < nparts; ++p) {
        double v = 0.0;
        for (int i = threadIdx.x; i < kRed; i += blockDim.x) v += partial[p * kRed + i];
        double s = bsum(v, sh);
        if (threadIdx.x == 0) sc[slot0 + p] = s;
        __syncthreads();
    }
}

__global__ void k_finv(const int32_t* __restrict__ part, int64_t nnu, const double* __restrict__ diag,
                       int64_t n, double* __restrict__ minv)
{
    GF_FOR(t, n) minv[t] = part[t] < nnu ? 1.0 / diag[t] : 0.0;
}

__global__ void k_fkeep(const int32_t* __restrict__ part, int64_t nnu, const double* __restrict__ x,
                        int64_t n, double* __restrict__ o)
{
    GF_FOR(t, n) o[t] = part[t] < nnu ? 0.0 : x[t];
}

// r = rhs_u - (A x)_u (0 on prescribed); partial r.r
__global__ void __launch_bounds__(256)
k_fres(const int32_t* __restrict__ dofs, const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
       const int32_t* __restrict__ part, int64_t nnu, const double* __restrict__ fe,
       const double* __restrict__ rhs, int64_t n, double* __restrict__ r, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double rr = 0.0;
    GF_FOR(t, n)
    {
        double rv = 0.0;
        if (part[t] < nnu) {
            int32_t d = dofs[t];
            double f = 0.0;
            for (int32_t j = ptr[d]; j < ptr[d + 1]; ++j) f += fe[idx[j]];
            rv = (rhs ? rhs[t] : 0.0) - f;
            rr = fma(rv, rv, rr);
        }
        r[t] = rv;
    }
    double s = bsum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// q = (A p)_u; partials p.q (row 0) and r.p (row 1)
__global__ void __launch_bounds__(256)
k_fgather(const int32_t* __restrict__ dofs, const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
          const int32_t* __restrict__ part, int64_t nnu, const double* __restrict__ fe,
          const double* __restrict__ p, const double* __restrict__ r, int64_t n, double* __restrict__ q,
          double* __restrict__ partial)
{
    __shared__ double sh[32];
    double pq = 0.0, rp = 0.0;
    GF_FOR(t, n)
    {
        double f = 0.0;
        if (part[t] < nnu) {
            int32_t d = dofs[t];
            for (int32_t j = ptr[d]; j < ptr[d + 1]; ++j) f += fe[idx[j]];
            pq = fma(p[t], f, pq);
            rp = fma(r[t], p[t], rp);
        }
        q[t] = f;
    }
    double s1 = bsum(pq, sh);
    double s2 = bsum(rp, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = s1;
        partial[kRed + blockIdx.x] = s2;
    }
}

__global__ void k_falpha(double* sc)
{
    if (threadIdx.x == 0) sc[F_ALPHA] = sc[F_RP] / sc[F_PQ];
}

// x += alpha p, r -= alpha q; partial r.r
__global__ void __launch_bounds__(256)
k_fupdate(const int32_t* __restrict__ part, int64_t nnu, const double* __restrict__ p,
          const double* __restrict__ q, int64_t n, const double* __restrict__ sc, double* __restrict__ x,
          double* __restrict__ r, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double alpha = sc[F_ALPHA];
    double rr = 0.0;
    GF_FOR(t, n)
    {
        if (part[t] < nnu) {
            x[t] = fma(alpha, p[t], x[t]);
            double rv = fma(-alpha, q[t], r[t]);
            r[t] = rv;
            rr = fma(rv, rv, rr);
        }
    }
    double s = bsum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void k_fjacobi(const double* __restrict__ minv, const double* __restrict__ r, int64_t n,
                          double* __restrict__ z)
{
    GF_FOR(t, n) z[t] = minv[t] * r[t];
}

// partial z.q
__global__ void __launch_bounds__(256)
k_fdot(const double* __restrict__ a, const double* __restrict__ b, int64_t n, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double acc = 0.0;
    GF_FOR(t, n) acc = fma(a[t], b[t], acc);
    double s = bsum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void k_fbeta(double* sc)
{
    if (threadIdx.x == 0) sc[F_BETA] = sc[F_ZQ] / sc[F_PQ];
}

// p = z - beta p
__global__ void k_fdir(const double* __restrict__ z, const double* __restrict__ sc, int64_t n,
                       double* __restrict__ p)
{
    double beta = sc[F_BETA];
    GF_FOR(t, n) p[t] = fma(-beta, p[t], z[t]);
}

struct FcgWs {
    double *fe, *p, *r, *z, *q, *minv, *partial, *sc;
    float *x0, *y;
    __nv_bfloat16 *a1, *a2, *a3;
};

inline FcgWs carve_fcg(const gfgpu_verlet_desc* d, int64_t hw, void* ws)
{
    char* c = static_cast<char*>(ws);
    int64_t n = d->nnode * d->ndim;
    FcgWs w;
    w.fe = reinterpret_cast<double*>(c);
    c += a256(d->nelem * d->nne * d->ndim * 8);
    double** v[] = {&w.p, &w.r, &w.z, &w.q, &w.minv};
    for (auto b : v) {
        *b = reinterpret_cast<double*>(c);
        c += a256(n * 8);
    }
    w.partial = reinterpret_cast<double*>(c);
    c += a256(2 * kRed * 8);
    w.sc = reinterpret_cast<double*>(c);
    c += a256(F_COUNT * 8);
    w.x0 = reinterpret_cast<float*>(c);
    c += a256(hw * 4 * 4);
    w.y = reinterpret_cast<float*>(c);
    c += a256(hw * 2 * 4);
    __nv_bfloat16** a[] = {&w.a1, &w.a2, &w.a3};
    for (auto b : a) {
        *b = reinterpret_cast<__nv_bfloat16*>(c);
        c += a256(hw * 32 * 2);
    }
    return w;
}

inline int64_t fcg_bytes(const gfgpu_verlet_desc* d, int64_t hw)
{
    int64_t n = d->nnode * d->ndim;
    return a256(d->nelem * d->nne * d->ndim * 8) + 5 * a256(n * 8) + a256(2 * kRed * 8) +
           a256(F_COUNT * 8) + a256(hw * 16) + a256(hw * 8) + 3 * a256(hw * 64);
}

// z = network(r) on the nodal grid, with the tensor-core middle layers
inline int nn_apply(const gfgpu_nn_desc* nn, const double* r, const double* sc, int rr_slot,
                    double nfree, const int32_t* part, int64_t nnu, FcgWs& w, double* z, cudaStream_t s)
{
    int H = nn->H, W = nn->W;
    int64_t hw = int64_t(H) * W;
    k_nn_input<<<grid_for(hw), kBlock, 0, s>>>(r, nn->material, sc, rr_slot, nfree, hw, w.x0);
    unsigned g = pix_grid(hw);
    k_conv_fwd<4, 32, true, float, __nv_bfloat16><<<g, 128, 0, s>>>(
        w.x0, wb(nn->weights_bf16, 0), nn->params_f32 + b_off(0), dil_of(0), 1, H, W, w.a1);
    dim3 grid((W + kTileX - 1) / kTileX, (H + kTileY - 1) / kTileY);
    k_conv32_mma<<<grid, 128, mma_smem_bytes(dil_of(1)), s>>>(
        w.a1, wb(nn->weights_bf16, 1), nn->params_f32 + b_off(1), dil_of(1), H, W, w.a2);
    k_conv32_mma<<<grid, 128, mma_smem_bytes(dil_of(2)), s>>>(
        w.a2, wb(nn->weights_bf16, 2), nn->params_f32 + b_off(2), dil_of(2), H, W, w.a3);
    k_conv_fwd<32, 2, false, __nv_bfloat16, float><<<g, 128, 0, s>>>(
        w.a3, wb(nn->weights_bf16, 3), nn->params_f32 + b_off(3), dil_of(3), 1, H, W, w.y);
    k_nn_output<<<grid_for(hw * 2), kBlock, 0, s>>>(w.y, sc, rr_slot, nfree, part, nnu, hw * 2, z);
    return check_launch("nn_apply");
}

inline int prepare_mma(cudaStream_t)
{
    static bool done = false;
    if (done) return GFGPU_OK;
    GF_TRY(check_cuda(cudaFuncSetAttribute(k_conv32_mma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(mma_smem_bytes(4))),
                      "cudaFuncSetAttribute"));
    done = true;
    return GFGPU_OK;
}

} // namespace nn
} // namespace gfgpu

extern "C" {

int32_t gfgpu_nn_param_count(void)
{
    return kParams;
}

int32_t gfgpu_nn_param_offset(int32_t layer, int32_t bias)
{
    if (layer < 0 || layer > 3) return -1;
    return bias ? b_off(layer) : w_off(layer);
}

int64_t gfgpu_nn_train_workspace_bytes(int32_t B, int32_t H, int32_t W)
{
    return train_bytes(int64_t(B) * H * W);
}

int gfgpu_nn_forward(const void* weights_bf16, const float* params_f32, const float* X, int32_t B,
                     int32_t H, int32_t W, float* Y, void* workspace, gfgpu_stream_t stream)
{
    GF_REQUIRE(weights_bf16 && params_f32 && X && Y && workspace && B > 0 && H > 0 && W > 0,
               "bad argument");
    TrainWs w = carve_train(workspace, int64_t(B) * H * W);
    forward_f32(weights_bf16, params_f32, X, B, H, W, w, S(stream));
    GF_TRY(check_cuda(cudaMemcpyAsync(Y, w.y, int64_t(B) * H * W * 2 * 4, cudaMemcpyDeviceToDevice,
                                      S(stream)),
                      "cudaMemcpyAsync"));
    return check_launch("nn_forward");
}

int gfgpu_nn_train_step(const void* weights_bf16, const float* params_f32, const float* X,
                        const float* T, int32_t B, int32_t S_, int32_t margin, float* grads,
                        float* loss, void* workspace, gfgpu_stream_t stream)
{
    GF_REQUIRE(weights_bf16 && params_f32 && X && T && grads && loss && workspace, "bad argument");
    GF_REQUIRE(B > 0 && S_ > 2 * margin && margin >= 0, "bad crop size");
    cudaStream_t s = S(stream);
    int64_t npix = int64_t(B) * S_ * S_;
    TrainWs w = carve_train(workspace, npix);
    forward_f32(weights_bf16, params_f32, X, B, S_, S_, w, s);
    k_mse<<<1024, 256, 0, s>>>(w.y, T, B, S_, margin, 2, w.g3, w.lpart);
    k_sum_partials<<<1, 32, 0, s>>>(w.lpart, 1024, 1, loss);
    // layer 4 (32 -> 2)
    weight_grad<32, 2>(w.a3, w.g3, dil_of(3), B, S_, S_, w.partial, grads + w_off(3), s);
    unsigned g = pix_grid(npix);
    k_conv_bwd_data<32, 2><<<g, 128, 0, s>>>(w.g3, wb(weights_bf16, 3), dil_of(3), B, S_, S_, w.a3, w.g2);
    // layer 3 (32 -> 32)
    weight_grad<32, 32>(w.a2, w.g2, dil_of(2), B, S_, S_, w.partial, grads + w_off(2), s);
    k_conv_bwd_data<32, 32><<<g, 128, 0, s>>>(w.g2, wb(weights_bf16, 2), dil_of(2), B, S_, S_, w.a2, w.g1);
    // layer 2 (32 -> 32): the gradient of its input goes back into g2
    weight_grad<32, 32>(w.a1, w.g1, dil_of(1), B, S_, S_, w.partial, grads + w_off(1), s);
    k_conv_bwd_data<32, 32><<<g, 128, 0, s>>>(w.g1, wb(weights_bf16, 1), dil_of(1), B, S_, S_, w.a1, w.g2);
    // layer 1 (4 -> 32)
    weight_grad<4, 32>(X, w.g2, dil_of(0), B, S_, S_, w.partial, grads + w_off(0), s);
    return check_launch("nn_train_step");
}

int gfgpu_nn_adam(float* params, const float* grads, float* m, float* v, int32_t n, float lr,
                  float beta1, float beta2, float eps, int32_t step, void* weights_bf16,
                  gfgpu_stream_t stream)
{
    GF_REQUIRE(params && grads && m && v && weights_bf16 && n > 0 && step >= 1, "bad argument");
    float c1 = 1.0f - std::pow(beta1, static_cast<float>(step));
    float c2 = 1.0f - std::pow(beta2, static_cast<float>(step));
    k_adam<<<(n + 255) / 256, 256, 0, S(stream)>>>(params, grads, m, v, n, lr, beta1, beta2, eps, c1,
                                                   c2, static_cast<__nv_bfloat16*>(weights_bf16));
    return check_launch("nn_adam");
}

int gfgpu_nn_gather_crops(const float* R, const float* T, const float* material, const int32_t* pos,
                          int32_t B, int32_t S_, int32_t H, int32_t W, float* X, float* Tc,
                          gfgpu_stream_t stream)
{
    GF_REQUIRE(R && T && material && pos && X && Tc && B > 0 && S_ > 0, "bad argument");
    k_gather_crops<<<grid_for(int64_t(B) * S_ * S_), kBlock, 0, S(stream)>>>(R, T, material, pos, B, S_,
                                                                           H, W, X, Tc);
    return check_launch("nn_gather_crops");
}

int64_t gfgpu_fcg_workspace_bytes(const gfgpu_verlet_desc* d, int32_t H, int32_t W)
{
    return d ? fcg_bytes(d, int64_t(H) * W) : 0;
}

int gfgpu_nn_infer(const gfgpu_nn_desc* nn, const float* X0, float* Y, void* workspace,
                   gfgpu_stream_t stream)
{
    GF_REQUIRE(nn && X0 && Y && workspace && nn->H > 0 && nn->W > 0, "bad argument");
    GF_TRY(prepare_mma(S(stream)));
    cudaStream_t s = S(stream);
    int H = nn->H, W = nn->W;
    int64_t hw = int64_t(H) * W;
    char* c = static_cast<char*>(workspace);
    __nv_bfloat16* a1 = reinterpret_cast<__nv_bfloat16*>(c);
    __nv_bfloat16* a2 = reinterpret_cast<__nv_bfloat16*>(c + a256(hw * 64));
    __nv_bfloat16* a3 = reinterpret_cast<__nv_bfloat16*>(c + 2 * a256(hw * 64));
    unsigned g = pix_grid(hw);
    k_conv_fwd<4, 32, true, float, __nv_bfloat16><<<g, 128, 0, s>>>(
        X0, wb(nn->weights_bf16, 0), nn->params_f32 + b_off(0), dil_of(0), 1, H, W, a1);
    dim3 grid((W + kTileX - 1) / kTileX, (H + kTileY - 1) / kTileY);
    k_conv32_mma<<<grid, 128, mma_smem_bytes(dil_of(1)), s>>>(a1, wb(nn->weights_bf16, 1),
                                                             nn->params_f32 + b_off(1), dil_of(1), H, W, a2);
    k_conv32_mma<<<grid, 128, mma_smem_bytes(dil_of(2)), s>>>(a2, wb(nn->weights_bf16, 2),
                                                             nn->params_f32 + b_off(2), dil_of(2), H, W, a3);
    k_conv_fwd<32, 2, false, __nv_bfloat16, float><<<g, 128, 0, s>>>(
        a3, wb(nn->weights_bf16, 3), nn->params_f32 + b_off(3), dil_of(3), 1, H, W, Y);
    return check_launch("nn_infer");
}

int gfgpu_fcg_solve(const gfgpu_verlet_desc* d, const double* diag, const gfgpu_nn_desc* nn,
                    double* x, double tol, int64_t maxiter, int32_t check_every, void* workspace,
                    gfgpu_stream_t stream, int64_t* iters, double* relres)
{
    GF_REQUIRE(d && diag && x && workspace && iters && relres && tol > 0.0 && maxiter >= 0,
               "bad argument");
    GF_REQUIRE(!nn || (d->nne == 4 && d->ndim == 2 && int64_t(nn->H) * nn->W == d->nnode &&
                       nn->weights_bf16 && nn->params_f32 && nn->material),
               "the network preconditioner needs a Quad4 Regular grid of H x W nodes");
    if (check_every < 1) check_every = 1;
    cudaStream_t s = S(stream);
    if (nn) GF_TRY(prepare_mma(s));
    int64_t hw = nn ? int64_t(nn->H) * nn->W : 0;
    FcgWs w = carve_fcg(d, hw, workspace);
    int64_t n = d->nnode * d->ndim;
    double nfree = static_cast<double>(d->nnu);
    const unsigned gb = kRed;
    auto precond = [&]() -> int {
        if (nn) return nn_apply(nn, w.r, w.sc, F_RR, nfree, d->part, d->nnu, w, w.z, s);
        k_fjacobi<<<grid_for(n), kBlock, 0, s>>>(w.minv, w.r, n, w.z);
        return check_launch("jacobi");
    };
    auto read_sc = [&](double* h) -> int {
        GF_TRY(check_cuda(cudaMemcpyAsync(h, w.sc, F_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s),
                          "cudaMemcpyAsync"));
        return check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    };
    double h[F_COUNT];
    k_finv<<<grid_for(n), kBlock, 0, s>>>(d->part, d->nnu, diag, n, w.minv);
    // ||b||, b = -(A x_p)_u
    k_fkeep<<<grid_for(n), kBlock, 0, s>>>(d->part, d->nnu, x, n, w.p);
    GF_TRY(gfgpu_internal_element_forces(d, w.p, w.fe, s));
    k_fres<<<gb, 256, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe, nullptr, n, w.z,
                              w.partial);
    k_fred<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, F_BB);
    // r = -(A x)_u, z = M(r), p = z
    GF_TRY(gfgpu_internal_element_forces(d, x, w.fe, s));
    k_fres<<<gb, 256, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe, nullptr, n, w.r,
                              w.partial);
    k_fred<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, F_RR);
    GF_TRY(precond());
    GF_TRY(check_cuda(cudaMemcpyAsync(w.p, w.z, n * 8, cudaMemcpyDeviceToDevice, s), "copy"));
    GF_TRY(read_sc(h));
    double bnorm = std::sqrt(h[F_BB]);
    if (bnorm == 0.0) bnorm = 1.0;
    double rel = std::sqrt(h[F_RR]) / bnorm;
    int64_t it = 0;
    while (rel > tol && it < maxiter) {
        int64_t nb = std::min<int64_t>(check_every, maxiter - it);
        for (int64_t k = 0; k < nb; ++k) {
            GF_TRY(gfgpu_internal_element_forces(d, w.p, w.fe, s));
            k_fgather<<<gb, 256, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe, w.p, w.r,
                                         n, w.q, w.partial);
            k_fred<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, F_PQ);
            k_fred<<<1, 1024, 0, s>>>(w.partial + kRed, 1, w.sc, F_RP);
            k_falpha<<<1, 32, 0, s>>>(w.sc);
            k_fupdate<<<gb, 256, 0, s>>>(d->part, d->nnu, w.p, w.q, n, w.sc, x, w.r, w.partial);
            k_fred<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, F_RR);
            GF_TRY(precond());
            k_fdot<<<gb, 256, 0, s>>>(w.z, w.q, n, w.partial);
            k_fred<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, F_ZQ);
            k_fbeta<<<1, 32, 0, s>>>(w.sc);
            k_fdir<<<grid_for(n), kBlock, 0, s>>>(w.z, w.sc, n, w.p);
        }
        it += nb;
        GF_TRY(check_launch("fcg iteration"));
        GF_TRY(read_sc(h));
        if (!std::isfinite(h[F_RR])) {
            *iters = it;
            *relres = h[F_RR];
            return fail(GFGPU_ERR_NAN, "gfgpu_fcg_solve: non-finite residual");
        }
        rel = std::sqrt(h[F_RR]) / bnorm;
    }
    // true residual -(A x)_u
    GF_TRY(gfgpu_internal_element_forces(d, x, w.fe, s));
    k_fres<<<gb, 256, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe, nullptr, n, w.r,
                              w.partial);
    k_fred<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, F_RR);
    GF_TRY(read_sc(h));
    *iters = it;
    *relres = std::sqrt(h[F_RR]) / bnorm;
    if (*relres > tol) return fail(GFGPU_ERR_DIVERGED, "gfgpu_fcg_solve: tolerance not reached");
    return GFGPU_OK;
}

} // extern "C"
