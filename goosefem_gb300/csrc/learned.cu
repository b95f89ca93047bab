// Learned preconditioner for the matrix-free static solve: a 4-layer 3x3 convolutional network
// on the structured nodal grid (NHWC: the nodevec [nnode, 2] of a Regular Quad4 mesh is the
// [H, W, 2] image), channels 4 -> 32 -> 32 -> 32 -> 2 (input: the two residual components
// scaled by their RMS, plus the nodal bulk and shear moduli), dilations 1, 2, 4, 1, ReLU after
// the first three layers. Weights are BF16, biases and every accumulation FP32.
//
//  * training kernels (CUDA cores, FP32 accumulate): forward with stored activations, backward
//    for the inputs and the weights (per-block partial sums reduced in a fixed order:
//    deterministic), masked mean-squared error or energy-norm loss, Adam;
//  * inference: the 32 -> 32 layers on the tensor cores (mma.sync m16n8k16 BF16, FP32
//    accumulate) from a shared-memory halo tile, first and last layer on the CUDA cores;
//  * energy-norm training loss: for each crop, e^T A e / t^T A t with A the crop's stiffness
//    (unit square Quad4 elements with the crop's moduli) and e the masked output error;
//  * a flexible CG in FP64 (Notay's truncated FCG with two search directions per iteration, the
//    Jacobi-preconditioned residual and the network's correction, each A-orthogonalised against
//    a ring of earlier directions), replayed as a CUDA graph.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <numeric>

#include "common.cuh"
#include "ffpair.cuh"

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

// Stiffness of the unit square Quad4 element (2x2 Gauss, plane strain) split by modulus:
// Ke = K * c_ke[0] + G * c_ke[1], rows / columns a*2+i (local node a, component i).
__constant__ float c_ke[2][64];
constexpr int kEnergyBlocks = 64; // fixed blocks per crop of the energy reduction

// Energy-norm loss of the crops (sum over the crops of e^T A e over the sum of t'^T A t': a
// ratio of sums, so a crop with a near-zero target cannot blow up the gradient), first pass. For node (b, y, x) of a crop, with
// e = M F (y - t) and t' = M F t (M: crop interior, F: free dofs), sums over the <= 4 elements
// around the node the element forces (Ke e) and (Ke t') at this node; writes the unscaled
// gradient 2 M F (A e) and per-block partials of e.(A e) and t'.(A t').
__global__ void __launch_bounds__(256)
k_crop_energy(const float* __restrict__ Y, const float* __restrict__ T, const float* __restrict__ E,
              const float* __restrict__ F, int B, int S, int m, float* __restrict__ dY,
              float* __restrict__ part)
{
    __shared__ float sh[2][8];
    int b = blockIdx.y;
    int64_t nn = static_cast<int64_t>(S) * S;
    const float* Yb = Y + b * nn * 2;
    const float* Tb = T + b * nn * 2;
    const float* Fb = F + b * nn * 2;
    const float* Eb = E + static_cast<int64_t>(b) * (S - 1) * (S - 1) * 2;
    float num = 0.0f, den = 0.0f;
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < nn;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int y = static_cast<int>(p / S), x = static_cast<int>(p % S);
        float ae[2] = {0.0f, 0.0f}, at[2] = {0.0f, 0.0f};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            // element (ey, ex) around the node, in which the node is local node a
            int ey = y - (k >= 2 ? 1 : 0), ex = x - ((k == 1 || k == 2) ? 1 : 0);
            int a = k == 0 ? 0 : (k == 1 ? 1 : (k == 2 ? 2 : 3));
            if (ey < 0 || ex < 0 || ey >= S - 1 || ex >= S - 1) continue;
            float Km = Eb[(static_cast<int64_t>(ey) * (S - 1) + ex) * 2];
            float Gm = Eb[(static_cast<int64_t>(ey) * (S - 1) + ex) * 2 + 1];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                int ny = ey + (c >= 2 ? 1 : 0), nx = ex + ((c == 1 || c == 2) ? 1 : 0);
                bool in = ny >= m && ny < S - m && nx >= m && nx < S - m;
                int64_t q = (static_cast<int64_t>(ny) * S + nx) * 2;
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    float f = in ? Fb[q + j] : 0.0f;
                    float ev = f * (Yb[q + j] - Tb[q + j]);
                    float tv = f * Tb[q + j];
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                        float kk = Km * c_ke[0][(a * 2 + i) * 8 + c * 2 + j] +
                                   Gm * c_ke[1][(a * 2 + i) * 8 + c * 2 + j];
                        ae[i] = fmaf(kk, ev, ae[i]);
                        at[i] = fmaf(kk, tv, at[i]);
                    }
                }
            }
        }
        bool in = y >= m && y < S - m && x >= m && x < S - m;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            float f = in ? Fb[p * 2 + i] : 0.0f;
            float ev = f * (Yb[p * 2 + i] - Tb[p * 2 + i]);
            float tv = f * Tb[p * 2 + i];
            num = fmaf(ev, ae[i], num);
            den = fmaf(tv, at[i], den);
            dY[(b * nn + p) * 2 + i] = 2.0f * f * ae[i];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        num += __shfl_down_sync(0xffffffffu, num, o);
        den += __shfl_down_sync(0xffffffffu, den, o);
    }
    int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wi] = num;
        sh[1][wi] = den;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float sn = 0.0f, sd = 0.0f;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
            sn += sh[0][w];
            sd += sh[1][w];
        }
        part[(static_cast<int64_t>(b) * gridDim.x + blockIdx.x) * 2] = sn;
        part[(static_cast<int64_t>(b) * gridDim.x + blockIdx.x) * 2 + 1] = sd;
    }
}

// loss = sum_b num_b / sum_b den_b (block, then crop order); scale = 1 / sum_b den_b
__global__ void k_energy_reduce(const float* __restrict__ part, int B, int nblk,
                                float* __restrict__ scale, float* __restrict__ loss)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float sn = 0.0f, sd = 0.0f;
    for (int b = 0; b < B; ++b) {
        float cn = 0.0f, cd = 0.0f;
        for (int k = 0; k < nblk; ++k) {
            cn += part[(static_cast<int64_t>(b) * nblk + k) * 2];
            cd += part[(static_cast<int64_t>(b) * nblk + k) * 2 + 1];
        }
        sn += cn;
        sd += cd;
    }
    bool ok = sd > 0.0f;
    *scale = ok ? 1.0f / sd : 0.0f;
    *loss = ok ? sn / sd : 0.0f;
}

__global__ void k_scale_grad(const float* __restrict__ scale, int64_t n, float* __restrict__ dY)
{
    float f = *scale;
    GF_FOR(i, n) dY[i] *= f;
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

// crops [B, S, S, 4] (scaled residual + material) and targets [B, S, S, 2] from the stored
// pairs; optionally the crops' element moduli E [B, S-1, S-1, 2] and free-dof mask F [B, S, S, 2]
// (0 outside the mesh)
__global__ void k_gather_crops(const float* __restrict__ R, const float* __restrict__ Tg,
                               const float* __restrict__ mat, const float* __restrict__ ekg,
                               const float* __restrict__ freem, const int* __restrict__ pos, int B,
                               int S, int H, int Wd, float* __restrict__ X, float* __restrict__ T,
                               float* __restrict__ E, float* __restrict__ F)
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
        if (F) {
            F[i * 2 + 0] = in ? freem[g * 2 + 0] : 0.0f;
            F[i * 2 + 1] = in ? freem[g * 2 + 1] : 0.0f;
        }
        if (E && y < S - 1 && x < S - 1) {
            bool ein = yy >= 0 && yy < H - 1 && xx >= 0 && xx < Wd - 1;
            int64_t e = static_cast<int64_t>(yy) * (Wd - 1) + xx;
            int64_t o = (static_cast<int64_t>(b) * (S - 1) + y) * (S - 1) + x;
            E[o * 2 + 0] = ein ? ekg[e * 2 + 0] : 0.0f;
            E[o * 2 + 1] = ein ? ekg[e * 2 + 1] : 0.0f;
        }
    }
}

// ------------------------------------------------------------------ tensor-core 32 -> 32 layer

// Weights in shared memory as [t][co][ci] with the ci row padded to 40 BF16 (80 B): the 32-bit
// fragment loads of 8 rows x 4 column pairs then hit 32 different banks.
constexpr int kPadC = 40;
constexpr int kTileY = 16, kTileX = 16;
constexpr int kMmaThreads = 256; // 8 warps, warp w computes tile rows 2w and 2w + 1

// 16-byte asynchronous global -> shared copy (zero fill when !valid; src must still be a valid
// address); completion: cp_async_wait_all() then __syncthreads()
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc, bool valid)
{
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(sdst));
    const int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gsrc), "r"(n) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// W [t][ci][co] (BF16) -> WT [t][co][kPadC] with zero padding: the shared-memory layout of
// the tensor-core layer, prepared once per set of weights
__global__ void k_nn_wprep(const __nv_bfloat16* __restrict__ W, __nv_bfloat16* __restrict__ WT)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * 32 * kPadC) return;
    int t = i / (32 * kPadC), co = (i / kPadC) % 32, ci = i % kPadC;
    WT[i] = ci < 32 ? W[(t * 32 + ci) * 32 + co] : __float2bfloat16_rn(0.0f);
}

// W [t][ci][co=2] (layer 4) -> WL [t][8][kPadC]: output channels padded to one n8 tile
__global__ void k_nn_wprep_last(const __nv_bfloat16* __restrict__ W, __nv_bfloat16* __restrict__ WL)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * 8 * kPadC) return;
    int t = i / (8 * kPadC), co = (i / kPadC) % 8, ci = i % kPadC;
    WL[i] = (ci < 32 && co < 2) ? W[(t * 32 + ci) * 2 + co] : __float2bfloat16_rn(0.0f);
}

// First layer as three k16 steps of 4 taps x 4 input channels (taps 9..11 zero):
// W [t][ci=4][co] -> WF [kk][co][kPadF], k = 4 tl + ci for tap 4 kk + tl. Row padding 24 BF16
// (48 B) keeps the 32-bit fragment loads of 8 rows x 4 pairs on distinct banks.
constexpr int kPadF = 24;
__global__ void k_nn_wprep_first(const __nv_bfloat16* __restrict__ W, __nv_bfloat16* __restrict__ WF)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * 32 * kPadF) return;
    int kk = i / (32 * kPadF), co = (i / kPadF) % 32, k = i % kPadF;
    int t = kk * 4 + k / 4, ci = k % 4;
    WF[i] = (k < 16 && t < 9) ? W[(t * 4 + ci) * 32 + co] : __float2bfloat16_rn(0.0f);
}

// 3x3 convolution from BF16 [H, W, 32] on the tensor cores (mma.sync m16n8k16, FP32 accumulate),
// NT n8 tiles of output channels. CTA: 256 threads, output tile 16 rows x 16 columns; warp w
// computes rows 2w, 2w+1 (one m16 tile of 16 pixels each), K = 9 taps x 32 input channels.
// LAST = false: Y = relu(conv + b), BF16 [H, W, 32] (NT = 4). LAST = true (NT = 1, the 32 -> 2
// output layer): z = sigma (conv + b) on the free dofs, 0 on prescribed (FP64 nodevec; sigma =
// RMS of the residual, sqrt(sc[rr_slot] / nfree)), or Yf [H, W, 2] FP32 when z is null.
// Programmatic dependent launch between the network's layers: a layer lets the next one launch
// as soon as all of its CTAs are resident (the next one's launch, TMEM allocation, barrier set-up
// and weight load then overlap this layer's tail) and waits for the previous layer's grid to
// complete before it touches the previous layer's output or writes anything. Both are no-ops for
// a kernel launched without the attribute.
__device__ __forceinline__ void pdl_launch_dependents()
{
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

__device__ __forceinline__ void pdl_wait()
{
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

// Channel-planar activations of the tcgen05 layers: [4][H][Wp][8] BF16, pixel (y, x) stored at
// row position x + kPlanarPad, Wp = planar_row(W) (a multiple of 8 pixels); the pad pixels are
// zero. Rows of 128-byte groups of 8 pixels make a halo tile one TMA box per plane with
// 128-byte inner lines.
constexpr int kPlanarPad = 4;

__host__ __device__ constexpr int planar_row(int W)
{
    return (W + kPlanarPad + 7) / 8 * 8;
}

template <int NT, bool LAST, bool PLANAR_IN = false>
__global__ void __launch_bounds__(kMmaThreads)
k_conv_mma(const __nv_bfloat16* __restrict__ X, const __nv_bfloat16* __restrict__ WT,
           const float* __restrict__ bias, int dil, int H, int Wd, __nv_bfloat16* __restrict__ Y,
           const double* __restrict__ sc, int rr_slot, double nfree, const int32_t* __restrict__ part,
           int64_t nnu, double* __restrict__ z, float* __restrict__ Yf)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_sigma;
    if (PLANAR_IN) pdl_wait(); // launched as a dependent of the tcgen05 layer
    const int hh = kTileY + 2 * dil, hw = kTileX + 2 * dil;
    __nv_bfloat16* halo = reinterpret_cast<__nv_bfloat16*>(smem);          // [hh][hw][40]
    __nv_bfloat16* ws = halo + hh * hw * kPadC;                             // [9][8 NT][40]
    const int y0 = blockIdx.y * kTileY, x0 = blockIdx.x * kTileX;
    // weights and halo (16-byte chunks of 8 channels, zero outside the grid) staged with
    // asynchronous copies, all in flight at once
    for (int i = threadIdx.x; i < 9 * 8 * NT * kPadC / 8; i += blockDim.x)
        cp_async16(ws + i * 8, WT + i * 8, true);
    for (int i = threadIdx.x; i < hh * hw * 4; i += blockDim.x) {
        int pix = i >> 2, ch = (i & 3) * 8;
        int yy = y0 - dil + pix / hw, xx = x0 - dil + pix % hw;
        const bool in = yy >= 0 && yy < H && xx >= 0 && xx < Wd;
        const int64_t gp = static_cast<int64_t>(yy) * Wd + xx;
        const __nv_bfloat16* src =
            !in ? X
                : (PLANAR_IN ? X + (ch / 8) * (static_cast<int64_t>(H) * planar_row(Wd) * 8) +
                                   (static_cast<int64_t>(yy) * planar_row(Wd) + xx + kPlanarPad) * 8
                             : X + gp * 32 + ch);
        cp_async16(halo + pix * kPadC + ch, src, in);
    }
    if (LAST && threadIdx.x == 0) s_sigma = z ? sqrt(sc[rr_slot] / nfree) : 1.0;
    cp_async_wait_all();
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    float c[2][NT][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt)
#pragma unroll
            for (int k = 0; k < 4; ++k) c[mt][nt][k] = 0.0f;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int dy = dil * (t / 3 - 1), dx = dil * (t % 3 - 1);
#pragma unroll
        for (int kc = 0; kc < 2; ++kc) {
            uint32_t b[NT][2];
#pragma unroll
            for (int nt = 0; nt < NT; ++nt) {
                const __nv_bfloat16* wp = ws + (t * 8 * NT + nt * 8 + gid) * kPadC + kc * 16 + tig * 2;
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
                for (int nt = 0; nt < NT; ++nt) mma_bf16(c[mt][nt], a0, a1, a2, a3, b[nt][0], b[nt][1]);
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
            const int64_t p = static_cast<int64_t>(yy) * Wd + xx;
            if constexpr (LAST) {
                if (tig != 0) continue; // output channels 0, 1 live in the lanes with tig = 0
                const float v0 = c[mt][0][2 * half + 0] + bias[0];
                const float v1 = c[mt][0][2 * half + 1] + bias[1];
                if (z) {
                    const double sg = s_sigma;
                    // exact float -> double on the integer pipe (ffpair.cuh)
                    z[2 * p] = part[2 * p] < nnu ? sg * ff_f32_to_f64(v0) : 0.0;
                    z[2 * p + 1] = part[2 * p + 1] < nnu ? sg * ff_f32_to_f64(v1) : 0.0;
                }
                else {
                    *reinterpret_cast<float2*>(Yf + 2 * p) = make_float2(v0, v1);
                }
            }
            else {
                __nv_bfloat16* yp = Y + p * 32;
#pragma unroll
                for (int nt = 0; nt < NT; ++nt) {
                    const int co = nt * 8 + tig * 2;
                    float v0 = fmaxf(c[mt][nt][2 * half + 0] + bias[co], 0.0f);
                    float v1 = fmaxf(c[mt][nt][2 * half + 1] + bias[co + 1], 0.0f);
                    *reinterpret_cast<__nv_bfloat162*>(yp + co) = __floats2bfloat162_rn(v0, v1);
                }
            }
        }
    }
}

// First layer (4 -> 32, dilation 1, ReLU) on the tensor cores: the input channels (the FP64
// residual scaled by 1 / sigma and the two material channels, or X0 [H, W, 4]) are rounded to
// BF16 into a shared halo tile [18][18][4]; K = 3 steps of 4 taps x 4 channels. Output BF16
// [H, W, 32]. Same tile and warp layout as k_conv_mma.
template <bool PLANAR_OUT = false>
__global__ void __launch_bounds__(kMmaThreads, 4)
k_first_mma(const double* __restrict__ r, const double* __restrict__ sc, int rr_slot, double nfree,
            const float* __restrict__ mat, const float* __restrict__ X0,
            const __nv_bfloat16* __restrict__ WF, const float* __restrict__ bias, int H, int Wd,
            __nv_bfloat16* __restrict__ Y)
{
    constexpr int hh = kTileY + 2, hw = kTileX + 2;
    __shared__ __align__(16) __nv_bfloat16 halo[hh * hw * 4];
    __shared__ __align__(16) __nv_bfloat16 wf[3 * 32 * kPadF];
    __shared__ float s_inv;
    if (PLANAR_OUT) pdl_launch_dependents(); // the tcgen05 layer that follows may launch
    const int y0 = blockIdx.y * kTileY, x0 = blockIdx.x * kTileX;
    for (int i = threadIdx.x; i < 3 * 32 * kPadF / 8; i += blockDim.x) cp_async16(wf + i * 8, WF + i * 8, true);
    if (threadIdx.x == 0) {
        double sigma = r ? sqrt(sc[rr_slot] / nfree) : 1.0;
        s_inv = sigma > 0.0 ? static_cast<float>(1.0 / sigma) : 0.0f;
    }
    __syncthreads();
    const float inv = s_inv;
    for (int pix = threadIdx.x; pix < hh * hw; pix += blockDim.x) {
        int yy = y0 - 1 + pix / hw, xx = x0 - 1 + pix % hw;
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (yy >= 0 && yy < H && xx >= 0 && xx < Wd) {
            int64_t q = static_cast<int64_t>(yy) * Wd + xx;
            if (r) {
                double2 rv = *reinterpret_cast<const double2*>(r + 2 * q);
                float2 mv = *reinterpret_cast<const float2*>(mat + 2 * q);
                // rn_f32 of the FP64 residual on the integer pipe (ffpair.cuh; the conversion
                // instruction issues at the FP64 rate)
                v[0] = ff_from_double(rv.x).h * inv;
                v[1] = ff_from_double(rv.y).h * inv;
                v[2] = mv.x;
                v[3] = mv.y;
            }
            else {
                float4 xv = *reinterpret_cast<const float4*>(X0 + 4 * q);
                v[0] = xv.x;
                v[1] = xv.y;
                v[2] = xv.z;
                v[3] = xv.w;
            }
        }
        __nv_bfloat162 h[2] = {__floats2bfloat162_rn(v[0], v[1]), __floats2bfloat162_rn(v[2], v[3])};
        *reinterpret_cast<uint2*>(halo + pix * 4) = *reinterpret_cast<uint2*>(h);
    }
    cp_async_wait_all();
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    const int ch = (tig & 1) * 2;
    float c[2][4][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int k = 0; k < 4; ++k) c[mt][nt][k] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 3; ++kk) {
        uint32_t b[4][2];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const __nv_bfloat16* wp = wf + (kk * 32 + nt * 8 + gid) * kPadF + tig * 2;
            b[nt][0] = *reinterpret_cast<const uint32_t*>(wp);
            b[nt][1] = *reinterpret_cast<const uint32_t*>(wp + 8);
        }
        // taps of the fragment's k pairs: k = tig * 2 (tap 4 kk + tig / 2) and k + 8 (2 taps on);
        // taps past 8 have zero weights and read the tile centre
        const int ta = kk * 4 + (tig >> 1), tb = ta + 2;
        const int dya = ta < 9 ? ta / 3 - 1 : 0, dxa = ta < 9 ? ta % 3 - 1 : 0;
        const int dyb = tb < 9 ? tb / 3 - 1 : 0, dxb = tb < 9 ? tb % 3 - 1 : 0;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int hr = 2 * warp + mt + 1;
            const __nv_bfloat16* pa = halo + ((hr + dya) * hw + gid + 1 + dxa) * 4 + ch;
            const __nv_bfloat16* pb = halo + ((hr + dyb) * hw + gid + 1 + dxb) * 4 + ch;
            uint32_t a0 = *reinterpret_cast<const uint32_t*>(pa);
            uint32_t a1 = *reinterpret_cast<const uint32_t*>(pa + 8 * 4);
            uint32_t a2 = *reinterpret_cast<const uint32_t*>(pb);
            uint32_t a3 = *reinterpret_cast<const uint32_t*>(pb + 8 * 4);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) mma_bf16(c[mt][nt], a0, a1, a2, a3, b[nt][0], b[nt][1]);
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
            const int64_t gp = static_cast<int64_t>(yy) * Wd + xx;
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int co = nt * 8 + tig * 2;
                float v0 = fmaxf(c[mt][nt][2 * half + 0] + bias[co], 0.0f);
                float v1 = fmaxf(c[mt][nt][2 * half + 1] + bias[co + 1], 0.0f);
                if (PLANAR_OUT) {
                    const int Wp = planar_row(Wd);
                    __nv_bfloat16* row = Y + nt * (static_cast<int64_t>(H) * Wp * 8) + static_cast<int64_t>(yy) * Wp * 8;
                    *reinterpret_cast<__nv_bfloat162*>(row + (xx + kPlanarPad) * 8 + tig * 2) =
                        __floats2bfloat162_rn(v0, v1);
                    // the row's pad pixels (left of x = 0, right of x = W - 1) stay zero
                    const __nv_bfloat162 z2 = __floats2bfloat162_rn(0.0f, 0.0f);
                    if (xx == 0)
                        for (int pp = 0; pp < kPlanarPad; ++pp)
                            *reinterpret_cast<__nv_bfloat162*>(row + pp * 8 + tig * 2) = z2;
                    if (xx == Wd - 1)
                        for (int pp = Wd + kPlanarPad; pp < Wp; ++pp)
                            *reinterpret_cast<__nv_bfloat162*>(row + pp * 8 + tig * 2) = z2;
                }
                else {
                    *reinterpret_cast<__nv_bfloat162*>(Y + gp * 32 + co) = __floats2bfloat162_rn(v0, v1);
                }
            }
        }
    }
}

// ------------------------------------------------------------------ tcgen05 32 -> 32 layer
//
// Implicit GEMM on the 5th-generation tensor cores: M = 128 output pixels of one grid row,
// N = 32 output channels, K = 9 taps x 32 input channels = 18 MMAs of K = 16, FP32 accumulators
// in tensor memory (TMEM), one CTA of 4 warps per RPC consecutive output rows. The input halo
// tile, (RPC + 2 dil) rows x (128 + 2 dil) pixels, is staged (cp.async, zero outside the grid)
// as 4 channel planes of 16 bytes per pixel: in that layout the A operand of every tap and
// K half is the same canonical no-swizzle K-major matrix (core matrices of 8 pixels x 16 B,
// 128 B apart along M, one plane apart along K) at a shifted start address, so the taps need
// no data movement. Weights: [tap][k half][8-channel half][co][8 ci], core matrices 128 B apart
// along N and 512 B apart along K. Thread 0 issues the MMAs and commits them to an mbarrier;
// every wait is bounded (flag gfgpu_nn_tc_status on time-out), TMEM is always freed.

__device__ int g_tc_timeout = 0;

constexpr int kTcThreads = 128;
constexpr int kTcM = 128;
constexpr int kTcWBytes = 9 * 2 * 2 * 32 * 16; // 18432
constexpr long kTcSpin = 1L << 22;

// W [t][ci][co] -> WB [t][kc][h][co][8]: ci = 16 kc + 8 h + e
__global__ void k_nn_wprep_tc(const __nv_bfloat16* __restrict__ W, __nv_bfloat16* __restrict__ WB)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * 1024) return;
    int t = i / 1024, kc = (i / 512) % 2, h = (i / 256) % 2, co = (i / 8) % 32, e = i % 8;
    WB[i] = W[(t * 32 + kc * 16 + h * 8 + e) * 32 + co];
}

__host__ __device__ constexpr int tc_rows(int rpc, int dil)
{
    return rpc + 2 * dil;
}

__host__ __device__ constexpr int tc_cols(int dil)
{
    return kTcM + 2 * dil;
}

// shared memory: weights, 4 planes, mbarrier + TMEM address slot
inline size_t tc_smem_bytes(int rpc, int dil)
{
    return static_cast<size_t>(kTcWBytes) + 4 * static_cast<size_t>(tc_rows(rpc, dil)) * tc_cols(dil) * 16 + 64;
}

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    // no-swizzle K-major matrix descriptor: start, leading (K) and stride (M/N) byte offsets in
    // 16-byte units, version 1 (bits 46-47), layout type 0 (no swizzle)
    return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9,
// 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t phase)
{
    for (long it = 0; it < kTcSpin; ++it) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(mbar), "r"(phase)
                     : "memory");
        if (done) return true;
    }
    return false;
}

template <int RPC>
__global__ void __launch_bounds__(kTcThreads)
k_conv32_tc(const __nv_bfloat16* __restrict__ X, const __nv_bfloat16* __restrict__ WB,
            const float* __restrict__ bias, int dil, int H, int Wd, __nv_bfloat16* __restrict__ Y)
{
    constexpr uint32_t kCols = 32 * RPC; // TMEM columns: one 32-column accumulator per row
    extern __shared__ __align__(128) unsigned char tsmem[];
    const int R = tc_rows(RPC, dil), C = tc_cols(dil);
    const uint32_t PL = static_cast<uint32_t>(R * C * 16);
    unsigned char* wsm = tsmem;
    unsigned char* planes = tsmem + kTcWBytes;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(planes + 4 * PL);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    const uint32_t s_w = static_cast<uint32_t>(__cvta_generic_to_shared(wsm));
    const uint32_t s_a = static_cast<uint32_t>(__cvta_generic_to_shared(planes));
    const uint32_t s_mbar = static_cast<uint32_t>(__cvta_generic_to_shared(mbar));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y0 = blockIdx.y * RPC, x0 = blockIdx.x * kTcM;

    if (warp == 0) {
        const uint32_t s_slot = static_cast<uint32_t>(__cvta_generic_to_shared(tslot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_slot), "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    for (int i = threadIdx.x; i < kTcWBytes / 16; i += blockDim.x) cp_async16(wsm + i * 16, WB + i * 8, true);
    for (int i = threadIdx.x; i < R * C * 4; i += blockDim.x) {
        const int q = i & 3, pix = i >> 2;
        const int yy = y0 - dil + pix / C, xx = x0 - dil + pix % C;
        const bool in = yy >= 0 && yy < H && xx >= 0 && xx < Wd;
        const __nv_bfloat16* src = in ? X + (static_cast<int64_t>(yy) * Wd + xx) * 32 + q * 8 : X;
        cp_async16(planes + q * PL + pix * 16, src, in);
    }
    cp_async_wait_all();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = *tslot;

    if (threadIdx.x == 0) {
#pragma unroll 1
        for (int m = 0; m < RPC; ++m) {
#pragma unroll 1
            for (int t = 0; t < 9; ++t) {
                const int dy = dil * (t / 3 - 1), dx = dil * (t % 3 - 1);
                const uint32_t pix0 = static_cast<uint32_t>((m + dil + dy) * C + dil + dx);
#pragma unroll
                for (int kc = 0; kc < 2; ++kc) {
                    const uint64_t da = tc_desc(s_a + 2 * kc * PL + pix0 * 16, PL, 128);
                    const uint64_t db = tc_desc(s_w + (t * 2 + kc) * 1024, 512, 128);
                    const uint32_t acc = (t | kc) ? 1u : 0u;
                    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr + m * 32),
                                 "l"(da), "l"(db), "r"(kTcIdesc), "r"(acc)
                                 : "memory");
                }
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(s_mbar)
                     : "memory");
    }
    bool ok = __all_sync(0xffffffffu, tc_wait(s_mbar, 0)); // warp-uniform: tcgen05.ld is .sync.aligned
    if (!ok) {
        atomicExch(&g_tc_timeout, 1);
        tc_wait(s_mbar, 0); // give the tensor cores a second bounded chance before TMEM is freed
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (ok) {
#pragma unroll 1
        for (int m = 0; m < RPC; ++m) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr + (static_cast<uint32_t>(warp * 32) << 16) + m * 32));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            const int yy = y0 + m, xx = x0 + warp * 32 + lane;
            if (yy < H && xx < Wd) {
                uint4* yp = reinterpret_cast<uint4*>(Y + (static_cast<int64_t>(yy) * Wd + xx) * 32);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    __nv_bfloat162 h[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int co = k * 8 + 2 * j;
                        h[j] = __floats2bfloat162_rn(fmaxf(__uint_as_float(v[co]) + bias[co], 0.0f),
                                                     fmaxf(__uint_as_float(v[co + 1]) + bias[co + 1], 0.0f));
                    }
                    yp[k] = *reinterpret_cast<uint4*>(h);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(kCols) : "memory");
    }
}

// ------------------------------------------------------- tcgen05 + TMA, persistent pipeline
//
// The same implicit GEMM as k_conv32_tc, as a persistent kernel (one CTA per SM) that overlaps
// the three stages of consecutive tiles of RPC rows x 128 pixels. Activations in and out are
// channel-planar with padded rows (planar_row), so that the halo tile of a plane is one TMA box
// (cp.async.bulk.tensor, 4-d view [4][H][Wp/8][16] of 8-byte elements, box R x 17 groups of 128
// bytes, zero fill outside the grid) into one of the 2-4 shared-memory stages that fit; warp 0
// (one lane) issues the 4 boxes of a tile. (A TMA instruction costs about the same whatever its
// size, and 128-byte inner lines are the fast case: 16-byte-wide boxes or one box per row were
// 1.2-1.3x slower per application.) Warp 1 (one lane) issues the 18 RPC MMAs of a tile into one of two TMEM accumulators
// and commits them to the stage's "empty" and the accumulator's "full" mbarrier; warps 2-5 drain
// an accumulator (tcgen05.ld, bias, ReLU, BF16) while the next tile is multiplied. Every wait is
// bounded; a role that gives up sets the time-out flag and leaves its loop.

constexpr int kTcpThreads = 192;
constexpr int kTcpMaxStages = 4;
constexpr size_t kTcpSmemBudget = 232448; // maximum dynamic shared memory of a CTA
constexpr int kTcpRPC = 4;

// pixels per shared-memory row of the halo tile: 17 groups of 8 (2176 bytes), the planar
// positions x0 .. x0 + 135 = image pixels x0 - 4 .. x0 + 131, which hold the 128 + 2 dil pixels of
// any dilation <= kPlanarPad
constexpr int kTcpGroups = 17;

__host__ __device__ constexpr int tcp_row_pixels(int)
{
    return kTcpGroups * 8;
}

__host__ __device__ constexpr uint32_t tcp_plane_bytes(int dil)
{
    return static_cast<uint32_t>(tc_rows(kTcpRPC, dil) * tcp_row_pixels(dil) * 16);
}

// halo-tile stages that fit beside the weights (2 .. kTcpMaxStages)
__host__ __device__ constexpr int tcp_stages(int dil)
{
    return static_cast<int>((kTcpSmemBudget - 1024 - kTcWBytes - 128) / (4 * tcp_plane_bytes(dil))) < kTcpMaxStages
               ? static_cast<int>((kTcpSmemBudget - 1024 - kTcWBytes - 128) / (4 * tcp_plane_bytes(dil)))
               : kTcpMaxStages;
}

inline size_t tcp_smem_bytes(int dil)
{
    return 1024 + kTcWBytes + static_cast<size_t>(tcp_stages(dil)) * 4 * tcp_plane_bytes(dil) + 128;
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t a)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(a) : "memory");
}

// MMA and commit issued by one elected lane of a converged warp (the descriptors stay
// warp-uniform, so the whole warp runs the issue loop)
__device__ __forceinline__ void tc_mma_elect(uint32_t tmem, uint64_t da, uint64_t db, uint32_t acc)
{
    asm volatile("{\n .reg .pred p, e;\n setp.ne.b32 p, %4, 0;\n elect.sync _|e, 0xffffffff;\n"
                 " @e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                 "l"(da), "l"(db), "r"(kTcIdesc), "r"(acc)
                 : "memory");
}

__device__ __forceinline__ void tc_commit_elect(uint32_t a)
{
    asm volatile("{\n .reg .pred e;\n elect.sync _|e, 0xffffffff;\n"
                 " @e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}\n" ::"r"(a)
                 : "memory");
}

template <int RPC>
__global__ void __launch_bounds__(kTcpThreads, 1)
k_conv32_tcp(const __grid_constant__ CUtensorMap tmap, const __nv_bfloat16* __restrict__ WB,
             const float* __restrict__ bias, int dil, int H, int Wd, __nv_bfloat16* __restrict__ Y)
{
    constexpr uint32_t kCols = 2 * 32 * RPC; // two accumulators of RPC x 32 columns
    extern __shared__ unsigned char tpsm[];
    unsigned char* wsm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tpsm) + 1023) & ~uintptr_t(1023));
    unsigned char* stages = wsm + kTcWBytes;
    const int R = tc_rows(RPC, dil), CP = tcp_row_pixels(dil);
    const uint32_t PL = tcp_plane_bytes(dil), SB = 4 * PL;
    const int NS = tcp_stages(dil);
    // full[4] empty[4] tfull[2] tempty[2], then the TMEM address slot
    uint64_t* bars = reinterpret_cast<uint64_t*>(stages + NS * SB);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * kTcpMaxStages + 4);
    const uint32_t s_w = static_cast<uint32_t>(__cvta_generic_to_shared(wsm));
    const uint32_t s_st = static_cast<uint32_t>(__cvta_generic_to_shared(stages));
    const uint32_t s_bar = static_cast<uint32_t>(__cvta_generic_to_shared(bars));
    auto full = [&](int i) { return s_bar + 8u * i; };
    auto empty = [&](int i) { return s_bar + 8u * (kTcpMaxStages + i); };
    auto tfull = [&](int i) { return s_bar + 8u * (2 * kTcpMaxStages + i); };
    auto tempty = [&](int i) { return s_bar + 8u * (2 * kTcpMaxStages + 2 + i); };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_x = (Wd + kTcM - 1) / kTcM, ntiles = tiles_x * ((H + RPC - 1) / RPC);
    pdl_launch_dependents();

    if (warp == 1) {
        const uint32_t s_slot = static_cast<uint32_t>(__cvta_generic_to_shared(tslot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_slot), "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; ++i) {
            mbar_init(full(i), 1);
            mbar_init(empty(i), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(tfull(i), 1);
            mbar_init(tempty(i), 128);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
    }
    for (int i = threadIdx.x; i < kTcWBytes / 16; i += blockDim.x) cp_async16(wsm + i * 16, WB + i * 8, true);
    cp_async_wait_all();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = *tslot;
    pdl_wait(); // the previous layer's output is complete from here on

    if (warp == 0) { // TMA producer: the whole warp waits, one lane loads the 4 planes of a tile
        // box: R rows x 17 groups of 8 pixels (128-byte lines) from planar position x0, i.e. image
        // pixels x0 - 4 .. x0 + 131; rows and groups outside the grid read as zeros
        const uint32_t bytes = 4u * static_cast<uint32_t>(R) * kTcpGroups * 128u;
        for (int k = 0, tile = blockIdx.x; tile < ntiles; ++k, tile += gridDim.x) {
            const int st = k % NS;
            if (k >= NS && !__all_sync(0xffffffffu, tc_wait(empty(st), ((k / NS) - 1) & 1))) {
                if (lane == 0) atomicExch(&g_tc_timeout, 1);
                break;
            }
            const int y0 = (tile / tiles_x) * RPC, x0 = (tile % tiles_x) * kTcM;
            if (lane == 0) {
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(full(st)), "r"(bytes)
                             : "memory");
                for (int q = 0; q < 4; ++q)
                    asm volatile(
                        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(s_st + st * SB + q * PL),
                        "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(0), "r"(x0 / 8), "r"(y0 - dil), "r"(q),
                        "r"(full(st))
                        : "memory");
            }
            __syncwarp();
        }
    }
    else if (warp == 1) { // MMA issuer: the whole warp, one elected lane issues
        {
            for (int k = 0, tile = blockIdx.x; tile < ntiles; ++k, tile += gridDim.x) {
                const int st = k % NS, b = k & 1;
                const bool ok = __all_sync(0xffffffffu, tc_wait(full(st), (k / NS) & 1)) &&
                                (k < 2 || __all_sync(0xffffffffu, tc_wait(tempty(b), ((k >> 1) - 1) & 1)));
                if (!ok) {
                    if (lane == 0) atomicExch(&g_tc_timeout, 1);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                // descriptors differ only in the start-address field (16-byte units, no carry:
                // shared addresses < 256 KB): one base each, offsets added
                const uint64_t da0 = tc_desc(s_st + st * SB, PL, 128), db0 = tc_desc(s_w, 512, 128);
#pragma unroll 1
                for (int m = 0; m < RPC; ++m) {
#pragma unroll
                    for (int t = 0; t < 9; ++t) {
                        const int dy = dil * (t / 3 - 1), dx = dil * (t % 3 - 1);
                        const uint32_t pix0 = static_cast<uint32_t>((m + dil + dy) * CP + kPlanarPad + dx);
#pragma unroll
                        for (int kc = 0; kc < 2; ++kc) {
                            const uint64_t da = da0 + pix0 + kc * (2 * PL >> 4);
                            const uint64_t db = db0 + (t * 2 + kc) * 64;
                            tc_mma_elect(taddr + b * 32 * RPC + m * 32, da, db, (t | kc) ? 1u : 0u);
                        }
                    }
                }
                tc_commit_elect(empty(st));
                tc_commit_elect(tfull(b));
            }
        }
    }
    else { // epilogue, warps 2-5: TMEM lane quarter warp % 4
        const int q4 = warp & 3;
        float bs[32];
#pragma unroll
        for (int co = 0; co < 32; ++co) bs[co] = bias[co];
        for (int k = 0, tile = blockIdx.x; tile < ntiles; ++k, tile += gridDim.x) {
            const int b = k & 1;
            if (!__all_sync(0xffffffffu, tc_wait(tfull(b), (k >> 1) & 1))) {
                atomicExch(&g_tc_timeout, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int y0 = (tile / tiles_x) * RPC, x0 = (tile % tiles_x) * kTcM;
#pragma unroll 1
            for (int m = 0; m < RPC; ++m) {
                uint32_t v[32];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                      "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                      "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(taddr + (static_cast<uint32_t>(q4 * 32) << 16) + b * 32 * RPC + m * 32));
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                const int yy = y0 + m, xx = x0 + q4 * 32 + lane;
                if (yy < H && xx < Wd) {
                    // planar output: the lanes of a warp write 32 consecutive 16-byte pixels of a plane
                    const int Wp = planar_row(Wd);
                    __nv_bfloat16* yrow = Y + static_cast<int64_t>(yy) * Wp * 8;
                    __nv_bfloat16* yp = yrow + (xx + kPlanarPad) * 8;
                    const int64_t plane = static_cast<int64_t>(H) * Wp * 8;
                    // the row's pad pixels stay zero
                    for (int kk = 0; kk < 4 && xx == 0; ++kk)
                        for (int pp = 0; pp < kPlanarPad; ++pp)
                            *reinterpret_cast<uint4*>(yrow + kk * plane + pp * 8) = make_uint4(0u, 0u, 0u, 0u);
                    for (int kk = 0; kk < 4 && xx == Wd - 1; ++kk)
                        for (int pp = Wd + kPlanarPad; pp < Wp; ++pp)
                            *reinterpret_cast<uint4*>(yrow + kk * plane + pp * 8) = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        __nv_bfloat162 h[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int co = kk * 8 + 2 * j;
                            h[j] = __floats2bfloat162_rn(fmaxf(__uint_as_float(v[co]) + bs[co], 0.0f),
                                                         fmaxf(__uint_as_float(v[co + 1]) + bs[co + 1], 0.0f));
                        }
                        *reinterpret_cast<uint4*>(yp + kk * plane) = *reinterpret_cast<uint4*>(h);
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            mbar_arrive(tempty(b));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(kCols) : "memory");
    }
}

// The 32 -> 32 layer with row reuse: each persistent CTA takes a contiguous range of tiles
// (RPC rows x 128 pixels) in column-strip order, so consecutive tiles of a strip share all but
// RPC of their R = RPC + 2 dil halo rows. Halo rows live in a ring of row slots (4 planes x CP
// pixels x 16 bytes each); a row is loaded once per run of tiles by TMA (the same two boxes per
// plane as k_conv32_tcp), each slot with its own "full" (TMA landed) and "empty" (the last MMA
// reading it completed) mbarrier. Warp 0 streams rows into slots, warp 1 (one lane) waits for a
// tile's R rows and issues its 18 RPC MMAs (the A operand of output row m and tap (dy, dx) is
// 128 pixels of the slot of halo row m + dil + dy) into one of two TMEM accumulators, then
// releases the rows the next tile no longer reads (all of them at the end of a run); warps 2-5
// drain the accumulators. A slot is reloaded only after its release, and NSLOT >= R keeps the
// producer from waiting on a tile that needs the row it is about to load. Every wait is bounded.
constexpr int kTcrThreads = 192;
constexpr int kTcrMaxSlots = 24;

__host__ __device__ constexpr uint32_t tcr_slot_bytes(int dil)
{
    return static_cast<uint32_t>(4 * tcp_row_pixels(dil) * 16);
}

__host__ __device__ constexpr int tcr_slots(int dil)
{
    return static_cast<int>((kTcpSmemBudget - 1024 - kTcWBytes - 512) / tcr_slot_bytes(dil)) < kTcrMaxSlots
               ? static_cast<int>((kTcpSmemBudget - 1024 - kTcWBytes - 512) / tcr_slot_bytes(dil))
               : kTcrMaxSlots;
}

inline size_t tcr_smem_bytes(int dil)
{
    return 1024 + kTcWBytes + static_cast<size_t>(tcr_slots(dil)) * tcr_slot_bytes(dil) + 512;
}

template <int RPC>
__global__ void __launch_bounds__(kTcrThreads, 1)
k_conv32_tcr(const __grid_constant__ CUtensorMap tmap, const __nv_bfloat16* __restrict__ WB, const float* __restrict__ bias, int dil, int H, int Wd,
             __nv_bfloat16* __restrict__ Y)
{
    constexpr uint32_t kCols = 2 * 32 * RPC;
    extern __shared__ unsigned char trsm[];
    unsigned char* wsm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(trsm) + 1023) & ~uintptr_t(1023));
    unsigned char* ring = wsm + kTcWBytes;
    const int R = tc_rows(RPC, dil), C = tc_cols(dil), CP = tcp_row_pixels(dil);
    const int NSLOT = tcr_slots(dil);
    const uint32_t SL = tcr_slot_bytes(dil), PLR = static_cast<uint32_t>(CP * 16); // slot, plane row
    // full[NSLOT] empty[NSLOT] tfull[2] tempty[2], then the TMEM address slot
    uint64_t* bars = reinterpret_cast<uint64_t*>(ring + NSLOT * SL);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * kTcrMaxSlots + 4);
    const uint32_t s_w = static_cast<uint32_t>(__cvta_generic_to_shared(wsm));
    const uint32_t s_ring = static_cast<uint32_t>(__cvta_generic_to_shared(ring));
    const uint32_t s_bar = static_cast<uint32_t>(__cvta_generic_to_shared(bars));
    auto full = [&](int i) { return s_bar + 8u * i; };
    auto empty = [&](int i) { return s_bar + 8u * (kTcrMaxSlots + i); };
    auto tfull = [&](int i) { return s_bar + 8u * (2 * kTcrMaxSlots + i); };
    auto tempty = [&](int i) { return s_bar + 8u * (2 * kTcrMaxSlots + 2 + i); };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_x = (Wd + kTcM - 1) / kTcM, tiles_y = (H + RPC - 1) / RPC;
    const int ntiles = tiles_x * tiles_y;
    // this CTA's tiles [t0, t1) in strip order: strip t / tiles_y, row tile t % tiles_y
    const int t0 = static_cast<int>(static_cast<int64_t>(ntiles) * blockIdx.x / gridDim.x);
    const int t1 = static_cast<int>(static_cast<int64_t>(ntiles) * (blockIdx.x + 1) / gridDim.x);
    // a tile continues the previous one's run when it is the next row tile of the same strip
    auto continues = [&](int t) { return t > t0 && (t % tiles_y) != 0; };

    if (warp == 1) {
        const uint32_t s_slot = static_cast<uint32_t>(__cvta_generic_to_shared(tslot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_slot), "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < NSLOT; ++i) {
            mbar_init(full(i), 1);
            mbar_init(empty(i), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(tfull(i), 1);
            mbar_init(tempty(i), 128);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
    }
    for (int i = threadIdx.x; i < kTcWBytes / 16; i += blockDim.x) cp_async16(wsm + i * 16, WB + i * 8, true);
    cp_async_wait_all();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = *tslot;

    if (warp == 0) { // row producer
        const uint32_t bytes = 4u * kTcpGroups * 128u; // a row of the 4 planes
        int row = 0; // stream index of the next row to load
        bool ok = true;
        for (int t = t0; t < t1 && ok; ++t) {
            const int x0 = (t / tiles_y) * kTcM, y0 = (t % tiles_y) * RPC;
            // rows of this tile not yet loaded: all R at the start of a run, else the last RPC
            const int first = continues(t) ? RPC + 2 * dil - RPC : 0;
            for (int r = first; r < R; ++r, ++row) {
                const int sl = row % NSLOT;
                if (row >= NSLOT && !__all_sync(0xffffffffu, tc_wait(empty(sl), ((row / NSLOT) - 1) & 1))) {
                    if (lane == 0) atomicExch(&g_tc_timeout, 1);
                    ok = false;
                    break;
                }
                if (lane == 0)
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(full(sl)),
                                 "r"(bytes)
                                 : "memory");
                __syncwarp();
                if (lane < 4) { // plane lane: one row of 17 groups from planar position x0
                    const uint32_t dst = s_ring + sl * SL + lane * PLR;
                    asm volatile(
                        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(dst),
                        "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(0), "r"(x0 / 8), "r"(y0 - dil + r), "r"(lane),
                        "r"(full(sl))
                        : "memory");
                }
            }
        }
    }
    else if (warp == 1) { // MMA issuer: the whole warp, one elected lane issues
        {
            int base = 0; // stream index of the current tile's first halo row
            int next = 0; // stream index after the rows loaded so far
            for (int t = t0, k = 0; t < t1; ++t, ++k) {
                const int b = k & 1;
                if (continues(t))
                    base += RPC;
                else
                    base = next;
                next = base + R;
                bool ok = k < 2 || __all_sync(0xffffffffu, tc_wait(tempty(b), ((k >> 1) - 1) & 1));
                for (int r = 0; r < R && ok; ++r)
                    ok = __all_sync(0xffffffffu, tc_wait(full((base + r) % NSLOT), ((base + r) / NSLOT) & 1));
                if (!ok) {
                    if (lane == 0) atomicExch(&g_tc_timeout, 1);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const int b0 = base % NSLOT; // slot of the tile's first halo row
                const uint64_t db0 = tc_desc(s_w, 512, 128);
#pragma unroll
                for (int m = 0; m < RPC; ++m) {
#pragma unroll
                    for (int ry = 0; ry < 3; ++ry) { // halo row m + ry dil
                        int sl = b0 + m + ry * dil;
                        sl -= sl >= NSLOT ? NSLOT : 0;
                        const uint64_t dr = tc_desc(s_ring + sl * SL, PLR, 128);
#pragma unroll
                        for (int rx = 0; rx < 3; ++rx) { // image pixels from x0 + (rx - 1) dil
                            const int tp = ry * 3 + rx;
                            const uint64_t da0 = dr + static_cast<uint64_t>(kPlanarPad + (rx - 1) * dil);
#pragma unroll
                            for (int kc = 0; kc < 2; ++kc)
                                tc_mma_elect(taddr + b * 32 * RPC + m * 32, da0 + kc * (2 * PLR >> 4),
                                             db0 + (tp * 2 + kc) * 64, (tp | kc) ? 1u : 0u);
                        }
                    }
                }
                tc_commit_elect(tfull(b));
                // release the rows no later tile of this run reads
                const int nrel = (t + 1 < t1 && continues(t + 1)) ? RPC : R;
                for (int r = 0; r < nrel; ++r) tc_commit_elect(empty((base + r) % NSLOT));
            }
        }
    }
    else { // epilogue, warps 2-5: TMEM lane quarter warp % 4
        const int q4 = warp & 3;
        float bs[32];
#pragma unroll
        for (int co = 0; co < 32; ++co) bs[co] = bias[co];
        for (int t = t0, k = 0; t < t1; ++t, ++k) {
            const int b = k & 1;
            if (!__all_sync(0xffffffffu, tc_wait(tfull(b), (k >> 1) & 1))) {
                atomicExch(&g_tc_timeout, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int x0 = (t / tiles_y) * kTcM, y0 = (t % tiles_y) * RPC;
#pragma unroll 1
            for (int m = 0; m < RPC; ++m) {
                uint32_t v[32];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                      "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                      "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(taddr + (static_cast<uint32_t>(q4 * 32) << 16) + b * 32 * RPC + m * 32));
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                const int yy = y0 + m, xx = x0 + q4 * 32 + lane;
                if (yy < H && xx < Wd) {
                    // planar output: the lanes of a warp write 32 consecutive 16-byte pixels of a plane
                    const int Wp = planar_row(Wd);
                    __nv_bfloat16* yrow = Y + static_cast<int64_t>(yy) * Wp * 8;
                    __nv_bfloat16* yp = yrow + (xx + kPlanarPad) * 8;
                    const int64_t plane = static_cast<int64_t>(H) * Wp * 8;
                    // the row's pad pixels stay zero
                    for (int kk = 0; kk < 4 && xx == 0; ++kk)
                        for (int pp = 0; pp < kPlanarPad; ++pp)
                            *reinterpret_cast<uint4*>(yrow + kk * plane + pp * 8) = make_uint4(0u, 0u, 0u, 0u);
                    for (int kk = 0; kk < 4 && xx == Wd - 1; ++kk)
                        for (int pp = Wd + kPlanarPad; pp < Wp; ++pp)
                            *reinterpret_cast<uint4*>(yrow + kk * plane + pp * 8) = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        __nv_bfloat162 h[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int co = kk * 8 + 2 * j;
                            h[j] = __floats2bfloat162_rn(fmaxf(__uint_as_float(v[co]) + bs[co], 0.0f),
                                                         fmaxf(__uint_as_float(v[co + 1]) + bs[co + 1], 0.0f));
                        }
                        *reinterpret_cast<uint4*>(yp + kk * plane) = *reinterpret_cast<uint4*>(h);
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            mbar_arrive(tempty(b));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(kCols) : "memory");
    }
}

inline size_t mma_smem_bytes(int dil, int nt = 4)
{
    return static_cast<size_t>((kTileY + 2 * dil) * (kTileX + 2 * dil) + 9 * 8 * nt) * kPadC * 2;
}

// ------------------------------------------------------------------ preconditioner glue (FP64)

} // namespace nn
} // namespace gfgpu

// ====================================================================== host side

using namespace gfgpu;
using namespace gfgpu::nn;

// element-kernel launch shared with the explicit step (dynamics.cu)
int gfgpu_internal_element_forces(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                  cudaStream_t s);
int gfgpu_internal_iteration_element_forces(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                            cudaStream_t s);
// two-level correction z = P ainv P^T r + minv r (coarse.cu)
int gfgpu_internal_coarse_apply(const gfgpu_coarse_desc* g, const int32_t* part, int64_t nnu,
                                const double* minv, const double* r, double* vc, double* yc,
                                double* z, cudaStream_t s);

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
    float *a1, *a2, *a3, *y, *g3, *g2, *g1, *partial, *lpart, *epart, *escale;
};

inline TrainWs carve_train(void* ws, int64_t B, int64_t npix)
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
    c += a256(1024 * 4 + 16);
    w.epart = reinterpret_cast<float*>(c);
    c += a256(int64_t(B) * kEnergyBlocks * 2 * 4);
    w.escale = reinterpret_cast<float*>(c);
    return w;
}

inline int64_t loss_bytes(int64_t B)
{
    return a256(1024 * 4 + 16) + a256(B * kEnergyBlocks * 2 * 4) + a256(B * 4);
}

inline int64_t train_bytes(int64_t B, int64_t npix)
{
    return 5 * a256(npix * 32 * 4) + 2 * a256(npix * 2 * 4) +
           a256(int64_t(kWgtBlocks) * (9 * 32 * 32 + 32) * 4) + loss_bytes(B);
}

// Element stiffness of the unit square (2x2 Gauss, plane strain) per unit K and per unit G.
// Local nodes (0,0), (1,0), (1,1), (0,1); x = (1 + xi) / 2; rows / columns a*2+i.
inline void unit_square_ke(double (&ke)[2][8][8])
{
    const double xa[4] = {-1, 1, 1, -1}, ya[4] = {-1, -1, 1, 1};
    const double g = 1.0 / std::sqrt(3.0);
    for (int m = 0; m < 2; ++m)
        for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) ke[m][r][c] = 0.0;
    for (int qy = 0; qy < 2; ++qy)
        for (int qx = 0; qx < 2; ++qx) {
            double xi = qx ? g : -g, eta = qy ? g : -g;
            double dN[4][2];
            for (int a = 0; a < 4; ++a) {
                dN[a][0] = 2.0 * 0.25 * xa[a] * (1.0 + eta * ya[a]); // d/dx = 2 d/dxi
                dN[a][1] = 2.0 * 0.25 * ya[a] * (1.0 + xi * xa[a]);
            }
            for (int a = 0; a < 4; ++a)
                for (int i = 0; i < 2; ++i)
                    for (int b = 0; b < 4; ++b)
                        for (int k = 0; k < 2; ++k)
                            for (int j = 0; j < 2; ++j)
                                for (int l = 0; l < 2; ++l) {
                                    double dij = i == j, dkl = k == l, dik = i == k, djl = j == l,
                                           dil = i == l, djk = j == k;
                                    double cK = dij * dkl;
                                    double cG = dik * djl + dil * djk - 2.0 / 3.0 * dij * dkl;
                                    double w = 0.25 * dN[a][j] * dN[b][l]; // weight x det(J)
                                    ke[0][a * 2 + i][b * 2 + k] += w * cK;
                                    ke[1][a * 2 + i][b * 2 + k] += w * cG;
                                }
        }
}

// c_ke, uploaded once per device
inline int upload_ke()
{
    static bool done[64] = {};
    int dev = 0;
    GF_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
    if (dev < 0 || dev >= 64) return fail(GFGPU_ERR_ARG, "upload_ke: device index");
    if (done[dev]) return GFGPU_OK;
    double ke[2][8][8];
    unit_square_ke(ke);
    float h[2][64];
    for (int m = 0; m < 2; ++m)
        for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) h[m][r * 8 + c] = static_cast<float>(ke[m][r][c]);
    GF_TRY(check_cuda(cudaMemcpyToSymbol(c_ke, h, sizeof(h)), "cudaMemcpyToSymbol"));
    done[dev] = true;
    return GFGPU_OK;
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

// Ring of search directions of the flexible CG: slot j holds P_j, Q_j = (A P_j)_u.
constexpr int kMaxSlots = 20;
struct SlotList {
    int n;
    int s[kMaxSlots];
};
// device scalars: r.r, b.b, step length per new direction, P.Q per slot, orthogonalisation
// coefficient per basis entry
enum { F_RR = 0, F_BB, F_A0, F_A1, F_PQ, F_C = F_PQ + kMaxSlots, F_R1 = F_C + kMaxSlots, F_COUNT };

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

// Last-block reductions: every block of a 1024-block (kRed) partial-sum kernel writes its partial,
// fences and counts itself in; the last block to arrive reduces the partials (fixed order, so the
// result does not depend on which block is last) and resets the counter for the next launch. This
// replaces a separate one-block reduction launch.
__device__ __forceinline__ bool last_block(unsigned int* counter)
{
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int prev = atomicAdd(counter, 1u);
        is_last = prev == gridDim.x - 1;
        if (is_last) *counter = 0u;
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// sum of partial[0 .. kRed) by the whole block in a fixed order
__device__ __forceinline__ double block_sum_partials(const double* partial, double* sh)
{
    double v = 0.0;
    for (int i = threadIdx.x; i < kRed; i += blockDim.x) v += __ldcg(partial + i);
    return bsum(v, sh);
}

// coefficient c_k = (z.Q_j) / (P_j.Q_j) of basis entry k (slot j = L.s[k]) from partial row k,
// computed by the last block (warp k -> rows k, k + nwarps, ...; lane-strided sums, then the
// shuffle tree); 0 for a degenerate or non-finite direction, which the combination then skips
__device__ __forceinline__ void coef_rows(const double* partial, const SlotList& L, double* sc)
{
    const int nw = blockDim.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x >> 5; k < L.n; k += nw) {
        double v = 0.0;
        for (int i = lane; i < kRed; i += 32) v += __ldcg(partial + k * kRed + i);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) {
            double pq = sc[F_PQ + L.s[k]];
            double c = (pq > 0.0 && isfinite(pq)) ? v / pq : 0.0;
            sc[F_C + k] = isfinite(c) ? c : 0.0;
        }
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
       const double* __restrict__ rhs, int64_t n, double* __restrict__ r, double* __restrict__ partial,
       RegGrid reg)
{
    __shared__ double sh[32];
    double rr = 0.0;
    GF_FOR(t, n)
    {
        double rv = 0.0;
        if (part[t] < nnu) {
            const double f = gather_dof(t, dofs, ptr, idx, fe, reg);
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
          double* __restrict__ partial, double* __restrict__ sc, int slot, int dd,
          unsigned int* __restrict__ counter, RegGrid reg)
{
    __shared__ double sh[32];
    double pq = 0.0, rp = 0.0;
    GF_FOR(t, n)
    {
        double f = 0.0;
        if (part[t] < nnu) {
            f = gather_dof(t, dofs, ptr, idx, fe, reg);
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
    if (last_block(counter)) { // P.Q and the step length alpha_dd = r.P / P.Q (0 if degenerate)
        const double tpq = block_sum_partials(partial, sh);
        const double trp = block_sum_partials(partial + kRed, sh);
        if (threadIdx.x == 0) {
            sc[F_PQ + slot] = tpq;
            double a = (tpq > 0.0 && isfinite(tpq)) ? trp / tpq : 0.0;
            sc[F_A0 + dd] = isfinite(a) ? a : 0.0;
        }
    }
}

// r1 = r - alpha_0 q0 (the residual after the step along the first direction of the iteration);
// partial r1.r1
__global__ void __launch_bounds__(256)
k_resid1(const double* __restrict__ r, const double* __restrict__ q0, double* __restrict__ sc,
         int64_t n, double* __restrict__ r1, double* __restrict__ partial, unsigned int* __restrict__ counter)
{
    __shared__ double sh[32];
    const double a0 = sc[F_A0];
    double rr = 0.0;
    GF_FOR(t, n)
    {
        double v = fma(-a0, q0[t], r[t]);
        r1[t] = v;
        rr = fma(v, v, rr);
    }
    double s = bsum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
    if (last_block(counter)) {
        const double t = block_sum_partials(partial, sh);
        if (threadIdx.x == 0) sc[F_R1] = t;
    }
}

// sc[dst.s[k]] = sum of partial row k (fixed order)
__global__ void k_fredv(const double* __restrict__ partial, SlotList dst, double* __restrict__ sc)
{
    __shared__ double sh[32];
    for (int p = 0; p < dst.n; ++p) {
        double v = 0.0;
        for (int i = threadIdx.x; i < kRed; i += blockDim.x) v += partial[p * kRed + i];
        double t = bsum(v, sh);
        if (threadIdx.x == 0) sc[dst.s[p]] = t;
        __syncthreads();
    }
}

// partial dots z.Q_j for the basis slots (z = minv * r when zin is null); NS >= L.n. Vectors
// are read as double2 (n even, slots 256-byte aligned).
template <int NS>
__global__ void __launch_bounds__(256)
k_mdot(const double* __restrict__ zin, const double* __restrict__ minv, const double* __restrict__ r,
       const double* __restrict__ Q, int64_t ld, SlotList L, int64_t n, double* __restrict__ partial,
       double* __restrict__ sc, unsigned int* __restrict__ counter)
{
    __shared__ double sh[32];
    double acc[NS];
    const double2* q[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
        acc[j] = 0.0;
        q[j] = reinterpret_cast<const double2*>(Q + (j < L.n ? L.s[j] : 0) * ld);
    }
    const int64_t n2 = n / 2;
    GF_FOR(t, n2)
    {
        double2 z;
        if (zin) {
            z = reinterpret_cast<const double2*>(zin)[t];
        }
        else {
            double2 m = reinterpret_cast<const double2*>(minv)[t];
            double2 rv = reinterpret_cast<const double2*>(r)[t];
            z = make_double2(m.x * rv.x, m.y * rv.y);
        }
#pragma unroll
        for (int j = 0; j < NS; ++j)
            if (j < L.n) {
                double2 qv = q[j][t];
                acc[j] = fma(z.x, qv.x, acc[j]);
                acc[j] = fma(z.y, qv.y, acc[j]);
            }
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) { // odd length: the last entry
        const int64_t t = n - 1;
        double z = zin ? zin[t] : minv[t] * r[t];
#pragma unroll
        for (int j = 0; j < NS; ++j)
            if (j < L.n) acc[j] = fma(z, Q[(j < L.n ? L.s[j] : 0) * ld + t], acc[j]);
    }
#pragma unroll
    for (int j = 0; j < NS; ++j) {
        if (j < L.n) {
            double v = bsum(acc[j], sh);
            if (threadIdx.x == 0) partial[j * kRed + blockIdx.x] = v;
        }
    }
    if (last_block(counter)) coef_rows(partial, L, sc);
}

// P_new = z - sum_k c_k P_{L.s[k]} (A-orthogonalisation with the precomputed coefficients),
// double2 access as in k_mdot
template <int NS>
__global__ void __launch_bounds__(256)
k_mcombine(const double* __restrict__ zin, const double* __restrict__ minv,
           const double* __restrict__ r, const double* __restrict__ sc, double* P, int64_t ld,
           SlotList L, int snew, int64_t n)
{
    double c[NS];
    const double2* p[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
        c[j] = j < L.n ? sc[F_C + j] : 0.0;
        p[j] = reinterpret_cast<const double2*>(P + (j < L.n ? L.s[j] : 0) * ld);
    }
    double2* out = reinterpret_cast<double2*>(P + snew * ld);
    const int64_t n2 = n / 2;
    GF_FOR(t, n2)
    {
        double2 v;
        if (zin) {
            v = reinterpret_cast<const double2*>(zin)[t];
        }
        else {
            double2 m = reinterpret_cast<const double2*>(minv)[t];
            double2 rv = reinterpret_cast<const double2*>(r)[t];
            v = make_double2(m.x * rv.x, m.y * rv.y);
        }
#pragma unroll
        for (int j = 0; j < NS; ++j)
            if (c[j] != 0.0) {
                double2 pv = p[j][t];
                v.x = fma(-c[j], pv.x, v.x);
                v.y = fma(-c[j], pv.y, v.y);
            }
        out[t] = v;
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) { // odd length: the last entry
        const int64_t t = n - 1;
        double v = zin ? zin[t] : minv[t] * r[t];
#pragma unroll
        for (int j = 0; j < NS; ++j)
            if (c[j] != 0.0) v = fma(-c[j], P[(j < L.n ? L.s[j] : 0) * ld + t], v);
        P[snew * ld + t] = v;
    }
}

// x += sum_d alpha_d P_d, r -= sum_d alpha_d Q_d (the new directions are mutually
// A-orthogonal, so every alpha is taken with the same r); partial r.r
__global__ void __launch_bounds__(256)
k_mupdate(const int32_t* __restrict__ part, int64_t nnu, const double* __restrict__ P,
          const double* __restrict__ Q, int64_t ld, int s0, int s1, int ndir,
          double* __restrict__ sc, int64_t n, double* __restrict__ x, double* __restrict__ r,
          double* __restrict__ partial, unsigned int* __restrict__ counter)
{
    __shared__ double sh[32];
    double a0 = sc[F_A0], a1 = ndir > 1 ? sc[F_A1] : 0.0;
    const double* P0 = P + s0 * ld;
    const double* Q0 = Q + s0 * ld;
    const double* P1 = P + s1 * ld;
    const double* Q1 = Q + s1 * ld;
    double rr = 0.0;
    GF_FOR(t, n)
    {
        if (part[t] < nnu) {
            double xv = x[t], rv = r[t];
            if (a0 != 0.0) {
                xv = fma(a0, P0[t], xv);
                rv = fma(-a0, Q0[t], rv);
            }
            if (a1 != 0.0) {
                xv = fma(a1, P1[t], xv);
                rv = fma(-a1, Q1[t], rv);
            }
            x[t] = xv;
            r[t] = rv;
            rr = fma(rv, rv, rr);
        }
    }
    double v = bsum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
    if (last_block(counter)) {
        const double t = block_sum_partials(partial, sh);
        if (threadIdx.x == 0) sc[F_RR] = t;
    }
}

// launch k_mdot / k_mcombine with the smallest slot-count instantiation that holds L.n
template <template <int> class F, class... A>
inline void with_ns(int n, A&&... a)
{
    if (n <= 1) F<1>::go(a...);
    else if (n <= 2) F<2>::go(a...);
    else if (n <= 4) F<4>::go(a...);
    else if (n <= 8) F<8>::go(a...);
    else if (n <= 12) F<12>::go(a...);
    else if (n <= 16) F<16>::go(a...);
    else F<kMaxSlots>::go(a...);
}

template <int NS>
struct MdotL {
    static void go(unsigned g, cudaStream_t st, const double* zin, const double* minv, const double* r,
                   const double* Q, int64_t ld, const SlotList& L, int64_t n, double* partial, double* sc,
                   unsigned int* counter)
    {
        k_mdot<NS><<<g, 256, 0, st>>>(zin, minv, r, Q, ld, L, n, partial, sc, counter);
    }
};

template <int NS>
struct McombineL {
    static void go(unsigned g, cudaStream_t st, const double* zin, const double* minv, const double* r,
                   const double* sc, double* P, int64_t ld, const SlotList& L, int snew, int64_t n)
    {
        k_mcombine<NS><<<g, 256, 0, st>>>(zin, minv, r, sc, P, ld, L, snew, n);
    }
};

struct FcgWs {
    unsigned int* cnt; // last-block counters: [0] dots, [1] gather, [2] update, [3] resid1
    double *fe, *r, *z, *minv, *P, *Q, *partial, *sc;
    int64_t ld;
    __nv_bfloat16 *a1, *a2, *a3, *wt1, *wt2, *wt0, *wt3;
};

constexpr int64_t kWtBytes = 9 * 32 * kPadC * 2; // prepared weights of one tensor-core layer

// pixels of an activation buffer: H rows of planar_row(W) (the padded planar rows of the tcgen05
// layers; the other layouts use H x W of them)
inline int64_t act_pixels(int H, int W)
{
    return int64_t(H) * planar_row(W);
}

// network buffers: three activations [hw][32] BF16 and the four prepared weight sets (layers
// 2, 3 in kWtBytes each; the first and last layer's smaller sets in the same room)
inline char* carve_nn(char* c, int64_t hw, __nv_bfloat16** a1, __nv_bfloat16** a2,
                      __nv_bfloat16** a3, __nv_bfloat16** wt1, __nv_bfloat16** wt2,
                      __nv_bfloat16** wt0, __nv_bfloat16** wt3)
{
    __nv_bfloat16** a[] = {a1, a2, a3};
    for (auto b : a) {
        *b = reinterpret_cast<__nv_bfloat16*>(c);
        c += a256(hw * 32 * 2);
    }
    __nv_bfloat16** wts[] = {wt1, wt2, wt0, wt3};
    for (auto b : wts) {
        *b = reinterpret_cast<__nv_bfloat16*>(c);
        c += a256(kWtBytes);
    }
    return c;
}

inline int64_t nn_bytes(int64_t hw)
{
    return 3 * a256(hw * 32 * 2) + 4 * a256(kWtBytes);
}

inline FcgWs carve_fcg(const gfgpu_verlet_desc* d, int64_t hw, int nslots, void* ws)
{
    char* c = static_cast<char*>(ws);
    int64_t n = d->nnode * d->ndim;
    FcgWs w;
    w.ld = a256(n * 8) / 8;
    w.fe = reinterpret_cast<double*>(c);
    c += a256(d->nelem * d->nne * d->ndim * 8);
    double** v[] = {&w.r, &w.z, &w.minv};
    for (auto b : v) {
        *b = reinterpret_cast<double*>(c);
        c += a256(n * 8);
    }
    w.P = reinterpret_cast<double*>(c);
    c += nslots * w.ld * 8;
    w.Q = reinterpret_cast<double*>(c);
    c += nslots * w.ld * 8;
    w.partial = reinterpret_cast<double*>(c);
    c += a256(int64_t(kMaxSlots) * kRed * 8);
    w.sc = reinterpret_cast<double*>(c);
    c += a256(F_COUNT * 8);
    w.cnt = reinterpret_cast<unsigned int*>(c);
    c += 256;
    carve_nn(c, hw, &w.a1, &w.a2, &w.a3, &w.wt1, &w.wt2, &w.wt0, &w.wt3);
    return w;
}

inline int64_t fcg_bytes(const gfgpu_verlet_desc* d, int64_t hw, int nslots)
{
    int64_t n = d->nnode * d->ndim;
    return a256(d->nelem * d->nne * d->ndim * 8) + (3 + 2 * int64_t(nslots)) * a256(n * 8) +
           a256(int64_t(kMaxSlots) * kRed * 8) + a256(F_COUNT * 8) + 256 + nn_bytes(hw);
}

// the tensor-core layers' weights in their shared-memory layouts
inline void nn_prepare_weights(const gfgpu_nn_desc* nn, __nv_bfloat16* wt1, __nv_bfloat16* wt2,
                               __nv_bfloat16* wt0, __nv_bfloat16* wt3, cudaStream_t s)
{
    static_assert(kTcWBytes <= kWtBytes, "tcgen05 weights fit the prepared-weight buffers");
    if (nn_tensor_path() >= 1) {
        k_nn_wprep_tc<<<(9 * 1024 + 255) / 256, 256, 0, s>>>(wb(nn->weights_bf16, 1), wt1);
        k_nn_wprep_tc<<<(9 * 1024 + 255) / 256, 256, 0, s>>>(wb(nn->weights_bf16, 2), wt2);
    }
    else {
        const unsigned g = (9 * 32 * kPadC + 255) / 256;
        k_nn_wprep<<<g, 256, 0, s>>>(wb(nn->weights_bf16, 1), wt1);
        k_nn_wprep<<<g, 256, 0, s>>>(wb(nn->weights_bf16, 2), wt2);
    }
    k_nn_wprep_first<<<(3 * 32 * kPadF + 255) / 256, 256, 0, s>>>(wb(nn->weights_bf16, 0), wt0);
    k_nn_wprep_last<<<(9 * 8 * kPadC + 255) / 256, 256, 0, s>>>(wb(nn->weights_bf16, 3), wt3);
}

// TMA view of a channel-planar BF16 activation with padded rows ([4][H][Wp][8], Wp =
// planar_row(W)) as [4][H][Wp/8][16] 8-byte elements; box: box_rows rows x 17 groups of 8
// pixels (128-byte inner lines) of one plane, zero fill outside the grid
inline int tcp_tensor_map(CUtensorMap* map, const __nv_bfloat16* X, int H, int W, int box_rows)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        GF_TRY(check_cuda(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q),
                          "cudaGetDriverEntryPointByVersion"));
        if (q != cudaDriverEntryPointSuccess || !fn) return fail(GFGPU_ERR_CUDA, "cuTensorMapEncodeTiled not found");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    GF_REQUIRE((reinterpret_cast<uintptr_t>(X) & 15u) == 0, "activation not 16-byte aligned");
    GF_REQUIRE(box_rows >= 1 && box_rows <= 256, "box rows");
    const cuuint64_t Wp = static_cast<cuuint64_t>(planar_row(W));
    const cuuint64_t dims[4] = {16, Wp / 8, static_cast<cuuint64_t>(H), 4};
    const cuuint64_t strides[3] = {128, Wp * 16, static_cast<cuuint64_t>(H) * Wp * 16};
    const cuuint32_t box[4] = {16, kTcpGroups, static_cast<cuuint32_t>(box_rows), 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult rc = encode(map, CU_TENSOR_MAP_DATA_TYPE_INT64, 4, const_cast<__nv_bfloat16*>(X), dims, strides, box,
                         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (rc != CUDA_SUCCESS) return fail(GFGPU_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(rc)) + ")");
    return GFGPU_OK;
}

// Dependent launches between the network's layers (gfgpu_set_nn_pdl): on by default.
int g_nn_pdl = 1;

// launch with programmatic stream serialisation (the kernel's pdl_wait orders it after the
// previous kernel of the stream); an ordinary stream-ordered launch when dependent launches are
// switched off (griddepcontrol.wait / launch_dependents are then no-ops)
template <typename... KArgs, typename... Args>
inline int launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                      Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = g_nn_pdl ? 1 : 0;
    return check_cuda(cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...), "cudaLaunchKernelEx");
}

// the four layers on one H x W grid: input from the FP64 residual (r != null) or from X0,
// output to the FP64 correction z (z != null) or to Y
inline int nn_forward(const gfgpu_nn_desc* nn, const double* r, const float* X0, const double* sc,
                      int rr_slot, double nfree, const int32_t* part, int64_t nnu,
                      __nv_bfloat16* a1, __nv_bfloat16* a2, __nv_bfloat16* a3,
                      const __nv_bfloat16* wt1, const __nv_bfloat16* wt2, const __nv_bfloat16* wt0,
                      const __nv_bfloat16* wt3, double* z, float* Y, cudaStream_t s)
{
    const int H = nn->H, W = nn->W;
    dim3 grid((W + kTileX - 1) / kTileX, (H + kTileY - 1) / kTileY);
    const bool planar = nn_tensor_path() >= 2; // paths 2, 3: channel-planar activations
    if (planar)
        k_first_mma<true><<<grid, kMmaThreads, 0, s>>>(r, sc, rr_slot, nfree, nn->material, X0, wt0,
                                                       nn->params_f32 + b_off(0), H, W, a1);
    else
        k_first_mma<false><<<grid, kMmaThreads, 0, s>>>(r, sc, rr_slot, nfree, nn->material, X0, wt0,
                                                        nn->params_f32 + b_off(0), H, W, a1);
    if (nn_tensor_path() >= 2) {
        static_assert(kPlanarPad >= 4, "dilations up to 4 fit the 17-group box");
        // path 2: one box per plane of a whole halo tile; path 3: one box per plane row
        CUtensorMap m1, m2;
        const bool ring = nn_tensor_path() == 3;
        GF_TRY(tcp_tensor_map(&m1, a1, H, W, ring ? 1 : tc_rows(kTcpRPC, dil_of(1))));
        GF_TRY(tcp_tensor_map(&m2, a2, H, W, ring ? 1 : tc_rows(kTcpRPC, dil_of(2))));
        const int ntiles = ((W + kTcM - 1) / kTcM) * ((H + kTcpRPC - 1) / kTcpRPC);
        int sms = 0, dev = 0;
        GF_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
        GF_TRY(check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
        const unsigned g = static_cast<unsigned>(std::max(1, std::min(ntiles, sms)));
        GF_REQUIRE(((reinterpret_cast<uintptr_t>(a1) | reinterpret_cast<uintptr_t>(a2)) & 15u) == 0,
                   "activations not 16-byte aligned");
        if (nn_tensor_path() == 3) {
            k_conv32_tcr<kTcpRPC><<<g, kTcrThreads, tcr_smem_bytes(dil_of(1)), s>>>(
                m1, wt1, nn->params_f32 + b_off(1), dil_of(1), H, W, a2);
            k_conv32_tcr<kTcpRPC><<<g, kTcrThreads, tcr_smem_bytes(dil_of(2)), s>>>(
                m2, wt2, nn->params_f32 + b_off(2), dil_of(2), H, W, a3);
        }
        else {
            GF_TRY(launch_pdl(k_conv32_tcp<kTcpRPC>, dim3(g), dim3(kTcpThreads), tcp_smem_bytes(dil_of(1)), s,
                              m1, wt1, nn->params_f32 + b_off(1), dil_of(1), H, W, a2));
            GF_TRY(launch_pdl(k_conv32_tcp<kTcpRPC>, dim3(g), dim3(kTcpThreads), tcp_smem_bytes(dil_of(2)), s,
                              m2, wt2, nn->params_f32 + b_off(2), dil_of(2), H, W, a3));
        }
    }
    else if (nn_tensor_path() == 1) {
        // layer 2 (dilation 2): 4 rows per CTA; layer 3 (dilation 4): 2 rows, so that two CTAs
        // share an SM (shared memory 87 / 105 KB)
        dim3 g4((W + kTcM - 1) / kTcM, (H + 3) / 4), g2((W + kTcM - 1) / kTcM, (H + 1) / 2);
        k_conv32_tc<4><<<g4, kTcThreads, tc_smem_bytes(4, dil_of(1)), s>>>(a1, wt1, nn->params_f32 + b_off(1),
                                                                          dil_of(1), H, W, a2);
        k_conv32_tc<2><<<g2, kTcThreads, tc_smem_bytes(2, dil_of(2)), s>>>(a2, wt2, nn->params_f32 + b_off(2),
                                                                          dil_of(2), H, W, a3);
    }
    else {
        k_conv_mma<4, false><<<grid, kMmaThreads, mma_smem_bytes(dil_of(1)), s>>>(
            a1, wt1, nn->params_f32 + b_off(1), dil_of(1), H, W, a2, nullptr, 0, 0.0, nullptr, 0, nullptr,
            nullptr);
        k_conv_mma<4, false><<<grid, kMmaThreads, mma_smem_bytes(dil_of(2)), s>>>(
            a2, wt2, nn->params_f32 + b_off(2), dil_of(2), H, W, a3, nullptr, 0, 0.0, nullptr, 0, nullptr,
            nullptr);
    }
    if (planar && nn_tensor_path() == 2)
        GF_TRY(launch_pdl(k_conv_mma<1, true, true>, grid, dim3(kMmaThreads), mma_smem_bytes(dil_of(3), 1), s, a3,
                          static_cast<const __nv_bfloat16*>(wt3), static_cast<const float*>(nn->params_f32 + b_off(3)),
                          dil_of(3), H, W, static_cast<__nv_bfloat16*>(nullptr), sc, rr_slot, nfree, part, nnu, z, Y));
    else if (planar)
        k_conv_mma<1, true, true><<<grid, kMmaThreads, mma_smem_bytes(dil_of(3), 1), s>>>(
            a3, wt3, nn->params_f32 + b_off(3), dil_of(3), H, W, nullptr, sc, rr_slot, nfree, part, nnu, z,
            Y);
    else
        k_conv_mma<1, true><<<grid, kMmaThreads, mma_smem_bytes(dil_of(3), 1), s>>>(
            a3, wt3, nn->params_f32 + b_off(3), dil_of(3), H, W, nullptr, sc, rr_slot, nfree, part, nnu, z,
            Y);
    return check_launch("nn_forward");
}

// z = RMS(r) * net(r / RMS(r)) on the nodal grid (0 on prescribed dofs)
inline int nn_apply(const gfgpu_nn_desc* nn, const double* r, const double* sc, int rr_slot,
                    double nfree, const int32_t* part, int64_t nnu, FcgWs& w, double* z, cudaStream_t s)
{
    return nn_forward(nn, r, nullptr, sc, rr_slot, nfree, part, nnu, w.a1, w.a2, w.a3, w.wt1, w.wt2,
                      w.wt0, w.wt3, z, nullptr, s);
}

inline int prepare_mma(cudaStream_t)
{
    static bool done = false;
    if (done) return GFGPU_OK;
    GF_TRY(check_cuda(cudaFuncSetAttribute(k_conv_mma<4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(mma_smem_bytes(4))),
                      "cudaFuncSetAttribute"));
    GF_TRY(check_cuda(cudaFuncSetAttribute(k_conv_mma<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(mma_smem_bytes(dil_of(3), 1))),
                      "cudaFuncSetAttribute"));
    GF_TRY(check_cuda(cudaFuncSetAttribute(k_conv_mma<1, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(mma_smem_bytes(dil_of(3), 1))),
                      "cudaFuncSetAttribute"));
    GF_TRY(check_cuda(cudaFuncSetAttribute(k_conv32_tcp<kTcpRPC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(std::max(tcp_smem_bytes(dil_of(1)),
                                                                     tcp_smem_bytes(dil_of(2))))),
                      "cudaFuncSetAttribute"));
    GF_TRY(check_cuda(cudaFuncSetAttribute(k_conv32_tcr<kTcpRPC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(std::max(tcr_smem_bytes(dil_of(1)),
                                                                     tcr_smem_bytes(dil_of(2))))),
                      "cudaFuncSetAttribute"));
    GF_TRY(check_cuda(cudaFuncSetAttribute(k_conv32_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(tc_smem_bytes(4, dil_of(1)))),
                      "cudaFuncSetAttribute"));
    GF_TRY(check_cuda(cudaFuncSetAttribute(k_conv32_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(tc_smem_bytes(2, dil_of(2)))),
                      "cudaFuncSetAttribute"));
    done = true;
    return GFGPU_OK;
}

} // namespace nn
} // namespace gfgpu

extern "C" {

int gfgpu_set_nn_pdl(int on)
{
    gfgpu::nn::g_nn_pdl = on ? 1 : 0;
    return GFGPU_OK;
}

int gfgpu_nn_tc_status(void)
{
    int flag = 0, zero = 0;
    GF_TRY(check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize"));
    GF_TRY(check_cuda(cudaMemcpyFromSymbol(&flag, g_tc_timeout, sizeof(int)), "cudaMemcpyFromSymbol"));
    if (flag) {
        GF_TRY(check_cuda(cudaMemcpyToSymbol(g_tc_timeout, &zero, sizeof(int)), "cudaMemcpyToSymbol"));
        return fail(GFGPU_ERR_TIMEOUT, "gfgpu_nn_tc_status: a tcgen05 layer's wait for the tensor cores gave up");
    }
    return GFGPU_OK;
}

int gfgpu_nn_unit_element_stiffness(double* out)
{
    GF_REQUIRE(out, "bad argument");
    double ke[2][8][8];
    unit_square_ke(ke);
    for (int m = 0; m < 2; ++m)
        for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) out[(m * 8 + r) * 8 + c] = ke[m][r][c];
    return GFGPU_OK;
}

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
    return train_bytes(B, int64_t(B) * H * W);
}

int gfgpu_nn_forward(const void* weights_bf16, const float* params_f32, const float* X, int32_t B,
                     int32_t H, int32_t W, float* Y, void* workspace, gfgpu_stream_t stream)
{
    GF_REQUIRE(weights_bf16 && params_f32 && X && Y && workspace && B > 0 && H > 0 && W > 0,
               "bad argument");
    TrainWs w = carve_train(workspace, B, int64_t(B) * H * W);
    forward_f32(weights_bf16, params_f32, X, B, H, W, w, S(stream));
    GF_TRY(check_cuda(cudaMemcpyAsync(Y, w.y, int64_t(B) * H * W * 2 * 4, cudaMemcpyDeviceToDevice,
                                      S(stream)),
                      "cudaMemcpyAsync"));
    return check_launch("nn_forward");
}

int gfgpu_nn_train_step(const void* weights_bf16, const float* params_f32, const float* X,
                        const float* T, const float* E, const float* F, int32_t B, int32_t S_,
                        int32_t margin, float* grads, float* loss, void* workspace,
                        gfgpu_stream_t stream)
{
    GF_REQUIRE(weights_bf16 && params_f32 && X && T && grads && loss && workspace, "bad argument");
    GF_REQUIRE(B > 0 && B <= 1024 && S_ > 2 * margin && margin >= 0, "bad crop size");
    GF_REQUIRE((E == nullptr) == (F == nullptr), "E and F are given together");
    cudaStream_t s = S(stream);
    int64_t npix = int64_t(B) * S_ * S_;
    TrainWs w = carve_train(workspace, B, npix);
    forward_f32(weights_bf16, params_f32, X, B, S_, S_, w, s);
    if (E) {
        GF_TRY(upload_ke());
        k_crop_energy<<<dim3(kEnergyBlocks, B), 256, 0, s>>>(w.y, T, E, F, B, S_, margin, w.g3, w.epart);
        k_energy_reduce<<<1, 32, 0, s>>>(w.epart, B, kEnergyBlocks, w.escale, loss);
        k_scale_grad<<<grid_for(npix * 2), kBlock, 0, s>>>(w.escale, npix * 2, w.g3);
    } else {
        k_mse<<<1024, 256, 0, s>>>(w.y, T, B, S_, margin, 2, w.g3, w.lpart);
        k_sum_partials<<<1, 32, 0, s>>>(w.lpart, 1024, 1, loss);
    }
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

int gfgpu_nn_gather_crops(const float* R, const float* T, const float* material,
                          const float* elem_kg, const float* free_mask, const int32_t* pos,
                          int32_t B, int32_t S_, int32_t H, int32_t W, float* X, float* Tc,
                          float* Ec, float* Fc, gfgpu_stream_t stream)
{
    GF_REQUIRE(R && T && material && pos && X && Tc && B > 0 && S_ > 1 && H > 1 && W > 1,
               "bad argument");
    GF_REQUIRE((!Ec || elem_kg) && (!Fc || free_mask), "Ec needs elem_kg and Fc needs free_mask");
    k_gather_crops<<<grid_for(int64_t(B) * S_ * S_), kBlock, 0, S(stream)>>>(
        R, T, material, elem_kg, free_mask, pos, B, S_, H, W, X, Tc, Ec, Fc);
    return check_launch("nn_gather_crops");
}

int64_t gfgpu_fcg_workspace_bytes(const gfgpu_verlet_desc* d, int32_t H, int32_t W, int32_t nkeep,
                                  int32_t ndir)
{
    if (!d || nkeep < 1 || ndir < 1 || ndir > 2 || nkeep + ndir > kMaxSlots) return 0;
    return fcg_bytes(d, act_pixels(H, W), nkeep + ndir);
}

int64_t gfgpu_nn_infer_workspace_bytes(int32_t H, int32_t W)
{
    return H > 0 && W > 0 ? nn_bytes(act_pixels(H, W)) : 0;
}

int gfgpu_nn_infer(const gfgpu_nn_desc* nn, const float* X0, float* Y, void* workspace,
                   gfgpu_stream_t stream)
{
    GF_REQUIRE(nn && X0 && Y && workspace && nn->H > 0 && nn->W > 0, "bad argument");
    GF_REQUIRE(nn->weights_bf16 && nn->params_f32, "bad network descriptor");
    GF_REQUIRE((reinterpret_cast<uintptr_t>(X0) & 15u) == 0 && (reinterpret_cast<uintptr_t>(Y) & 7u) == 0 &&
                   (reinterpret_cast<uintptr_t>(workspace) & 255u) == 0,
               "X0 must be 16-byte, Y 8-byte and the workspace 256-byte aligned");
    GF_TRY(prepare_mma(S(stream)));
    cudaStream_t s = S(stream);
    __nv_bfloat16 *a1, *a2, *a3, *wt1, *wt2, *wt0, *wt3;
    carve_nn(static_cast<char*>(workspace), act_pixels(nn->H, nn->W), &a1, &a2, &a3, &wt1, &wt2, &wt0, &wt3);
    nn_prepare_weights(nn, wt1, wt2, wt0, wt3, s);
    return nn_forward(nn, nullptr, X0, nullptr, 0, 1.0, nullptr, 0, a1, a2, a3, wt1, wt2, wt0, wt3,
                      nullptr, Y, s);
}

} // extern "C"

// the flexible CG of gfgpu_fcg_solve; with g != NULL the first direction of every iteration is
// the two-level correction D^-1 r + P ainv P^T r (buffers after the ring workspace)
static int fcg_core(const gfgpu_verlet_desc* d, const double* diag, const gfgpu_nn_desc* nn,
                    const gfgpu_coarse_desc* g, bool post, const double* rhs, double* x, double tol,
                    int64_t maxiter,
                    int32_t nkeep, int32_t check_every, void* workspace, gfgpu_stream_t stream,
                    int64_t* iters, double* relres)
{
    GF_REQUIRE(d && diag && x && workspace && iters && relres && tol > 0.0 && maxiter >= 0,
               "bad argument");
    GF_REQUIRE(!nn || (d->nne == 4 && d->ndim == 2 && int64_t(nn->H) * nn->W == d->nnode &&
                       nn->weights_bf16 && nn->params_f32 && nn->material),
               "the network preconditioner needs a Quad4 Regular grid of H x W nodes");
    const int ndir = nn ? 2 : 1;
    GF_REQUIRE(nkeep >= 1 && nkeep + ndir <= kMaxSlots, "nkeep out of range");
    if (check_every < 1) check_every = 1;
    cudaStream_t s = S(stream);
    if (nn) GF_TRY(prepare_mma(s));
    const int nslots = nkeep + ndir;
    int64_t hw = nn ? act_pixels(nn->H, nn->W) : 0;
    FcgWs w = carve_fcg(d, hw, nslots, workspace);
    const int64_t n = d->nnode * d->ndim;
    double *zc = nullptr, *vc = nullptr, *yc = nullptr;
    if (g) {
        char* c = static_cast<char*>(workspace) + fcg_bytes(d, hw, nslots);
        const int64_t nc = int64_t(g->ncx) * g->ncy * 2;
        zc = reinterpret_cast<double*>(c);
        vc = reinterpret_cast<double*>(c + a256(n * 8));
        yc = reinterpret_cast<double*>(c + a256(n * 8) + a256(nc * 8));
    }
    const double nfree = static_cast<double>(d->nnu);
    const unsigned gb = kRed;
    double h[F_COUNT];
    auto read_sc = [&]() -> int {
        GF_TRY(check_cuda(cudaMemcpyAsync(h, w.sc, F_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s),
                          "cudaMemcpyAsync"));
        return check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    };
    auto one = [](int slot) {
        SlotList l{};
        l.n = 1;
        l.s[0] = slot;
        return l;
    };

    // One iteration, direction counter `c0` on entry (slot of direction k: k mod nslots). New
    // direction d is A-orthogonalised against the last nkeep directions of earlier iterations
    // and the earlier directions of this iteration.
    auto iteration = [&](int64_t c0, cudaStream_t st) -> int {
        for (int dd = 0; dd < ndir; ++dd) {
            int64_t cur = c0 + dd;
            int snew = static_cast<int>(cur % nslots);
            SlotList L{};
            for (int64_t k = std::max<int64_t>(0, c0 - nkeep); k < cur; ++k)
                L.s[L.n++] = static_cast<int>(k % nslots);
            const double* zin = nullptr;
            if (dd == 0 && g) {
                GF_TRY(gfgpu_internal_coarse_apply(g, d->part, d->nnu, w.minv, w.r, vc, yc, zc, st));
                zin = zc;
            }
            if (dd == 1 && post) {
                // the network sees the residual left after the step along the two-level direction
                // (zc is free again: its direction is stored in slot c0 % nslots)
                const double* q0 = w.Q + static_cast<int>(c0 % nslots) * w.ld;
                k_resid1<<<gb, 256, 0, st>>>(w.r, q0, w.sc, n, zc, w.partial, w.cnt + 3);
                GF_TRY(nn_apply(nn, zc, w.sc, F_R1, nfree, d->part, d->nnu, w, w.z, st));
                zin = w.z;
            }
            else if (dd == 1) {
                GF_TRY(nn_apply(nn, w.r, w.sc, F_RR, nfree, d->part, d->nnu, w, w.z, st));
                zin = w.z;
            }
            if (L.n > 0) {
                with_ns<MdotL>(L.n, gb, st, zin, w.minv, w.r, w.Q, w.ld, L, n, w.partial, w.sc, w.cnt);
            }
            with_ns<McombineL>(L.n, grid_for(n / 2), st, zin, w.minv, w.r, w.sc, w.P, w.ld, L, snew, n);
            double* Pn = w.P + snew * w.ld;
            double* Qn = w.Q + snew * w.ld;
            GF_TRY(gfgpu_internal_iteration_element_forces(d, Pn, w.fe, st));
            k_fgather<<<gb, 256, 0, st>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe, Pn,
                                          w.r, n, Qn, w.partial, w.sc, snew, dd, w.cnt + 1, reg_grid(d));
        }
        k_mupdate<<<gb, 256, 0, st>>>(d->part, d->nnu, w.P, w.Q, w.ld, static_cast<int>(c0 % nslots),
                                      static_cast<int>((c0 + 1) % nslots), ndir, w.sc, n, x, w.r,
                                      w.partial, w.cnt + 2);
        return check_launch("fcg iteration");
    };

    if (nn) nn_prepare_weights(nn, w.wt1, w.wt2, w.wt0, w.wt3, s);
    GF_TRY(check_cuda(cudaMemsetAsync(w.cnt, 0, 256, s), "cudaMemsetAsync"));
    k_finv<<<grid_for(n), kBlock, 0, s>>>(d->part, d->nnu, diag, n, w.minv);
    // ||b||, b = -(A x_p)_u (P slot 0 as scratch)
    k_fkeep<<<grid_for(n), kBlock, 0, s>>>(d->part, d->nnu, x, n, w.P);
    GF_TRY(gfgpu_internal_element_forces(d, w.P, w.fe, s));
    k_fres<<<gb, 256, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe, rhs, n, w.z,
                              w.partial, reg_grid(d));
    k_fredv<<<1, 1024, 0, s>>>(w.partial, one(F_BB), w.sc);
    // r = -(A x)_u
    GF_TRY(gfgpu_internal_element_forces(d, x, w.fe, s));
    k_fres<<<gb, 256, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe, rhs, n, w.r,
                              w.partial, reg_grid(d));
    k_fredv<<<1, 1024, 0, s>>>(w.partial, one(F_RR), w.sc);
    GF_TRY(read_sc());
    double bnorm = std::sqrt(h[F_BB]);
    if (bnorm == 0.0) bnorm = 1.0;
    double rel = std::sqrt(h[F_RR]) / bnorm;

    // Warm-up iterations run one by one until the ring is full and aligned (direction counter a
    // multiple of nslots); from there `chunk` iterations repeat the same slot pattern and replay
    // as one CUDA graph.
    int64_t it = 0, c = 0;
    const int64_t period = nslots / std::gcd(nslots, ndir); // iterations per ring turn
    const int64_t chunk = period * ((check_every + period - 1) / period);
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    int rc = GFGPU_OK;
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (cs) cudaStreamDestroy(cs);
    };
    while (rel > tol && it < maxiter) {
        bool steady = c >= int64_t(nkeep) + ndir && c % nslots == 0;
        if (steady && !exec && maxiter - it >= chunk) {
            rc = check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate");
            if (rc != GFGPU_OK) break;
            cudaGraph_t graph = nullptr;
            rc = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
            if (rc != GFGPU_OK) break;
            int crc = GFGPU_OK;
            for (int64_t k = 0; k < chunk && crc == GFGPU_OK; ++k) crc = iteration(c + k * ndir, cs);
            cudaError_t e = cudaStreamEndCapture(cs, &graph);
            if (crc != GFGPU_OK) {
                if (graph) cudaGraphDestroy(graph);
                rc = crc;
                break;
            }
            rc = check_cuda(e, "cudaStreamEndCapture");
            if (rc == GFGPU_OK) rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
            if (graph) cudaGraphDestroy(graph);
            if (rc != GFGPU_OK) break;
        }
        if (exec && maxiter - it >= chunk) {
            rc = check_cuda(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
            if (rc != GFGPU_OK) break;
            it += chunk;
            c += chunk * ndir;
        }
        else {
            int64_t nb = exec ? maxiter - it : std::min<int64_t>(check_every, maxiter - it);
            for (int64_t k = 0; k < nb && rc == GFGPU_OK; ++k) {
                rc = iteration(c, s);
                ++it;
                c += ndir;
                if (!exec && c >= int64_t(nkeep) + ndir && c % nslots == 0 && maxiter - it >= chunk) break;
            }
            if (rc != GFGPU_OK) break;
        }
        rc = read_sc();
        if (rc != GFGPU_OK) break;
        if (!std::isfinite(h[F_RR])) {
            cleanup();
            *iters = it;
            *relres = h[F_RR];
            return fail(GFGPU_ERR_NAN, "gfgpu_fcg_solve: non-finite residual");
        }
        rel = std::sqrt(h[F_RR]) / bnorm;
    }
    cleanup();
    GF_TRY(rc);
    // true residual -(A x)_u
    GF_TRY(gfgpu_internal_element_forces(d, x, w.fe, s));
    k_fres<<<gb, 256, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe, rhs, n, w.r,
                              w.partial, reg_grid(d));
    k_fredv<<<1, 1024, 0, s>>>(w.partial, one(F_RR), w.sc);
    GF_TRY(read_sc());
    *iters = it;
    *relres = std::sqrt(h[F_RR]) / bnorm;
    if (*relres > tol) return fail(GFGPU_ERR_DIVERGED, "gfgpu_fcg_solve: tolerance not reached");
    return GFGPU_OK;
}

extern "C" {

int gfgpu_fcg_solve(const gfgpu_verlet_desc* d, const double* diag, const gfgpu_nn_desc* nn,
                    double* x, double tol, int64_t maxiter, int32_t nkeep, int32_t check_every,
                    void* workspace, gfgpu_stream_t stream, int64_t* iters, double* relres)
{
    return fcg_core(d, diag, nn, nullptr, false, nullptr, x, tol, maxiter, nkeep, check_every,
                    workspace, stream, iters, relres);
}

int64_t gfgpu_fcg_coarse_workspace_bytes(const gfgpu_verlet_desc* d, int32_t H, int32_t W,
                                         int32_t nkeep, int32_t ndir, const gfgpu_coarse_desc* g)
{
    int64_t base = gfgpu_fcg_workspace_bytes(d, H, W, nkeep, ndir);
    if (base == 0 || !g) return 0;
    const int64_t nc = int64_t(g->ncx) * g->ncy * 2;
    return base + a256(d->nnode * d->ndim * 8) + 2 * a256(nc * 8);
}

int gfgpu_fcg_solve_coarse(const gfgpu_verlet_desc* d, const double* diag, const gfgpu_nn_desc* nn,
                           const gfgpu_coarse_desc* g, int32_t post, const double* rhs, double* x,
                           double tol, int64_t maxiter,
                           int32_t nkeep, int32_t check_every, void* workspace,
                           gfgpu_stream_t stream, int64_t* iters, double* relres)
{
    GF_REQUIRE(g && g->ainv && d && d->nne == 4 && d->ndim == 2 &&
                   int64_t(g->nx + 1) * (g->ny + 1) == d->nnode &&
                   g->ncx == (g->nx + g->hc - 1) / g->hc + 1 && g->ncy == (g->ny + g->hc - 1) / g->hc + 1 &&
                   int64_t(g->ncx) * g->ncy * 2 <= 8192 && g->ld % 32 == 0 && g->ld >= 2 * g->ncx * g->ncy,
               "bad coarse grid");
    return fcg_core(d, diag, nn, g, post != 0, rhs, x, tol, maxiter, nkeep, check_every, workspace,
                    stream, iters, relres);
}

} // extern "C"
