// Explicit velocity-Verlet increments of a Regular square-element Quad4 mesh in float-float
// ("pair") arithmetic, one fused tile kernel per increment.
//
// The FP64 kernels of dynamics.cu (element kernel + node kernel) sit at the FP64 issue rate of
// GB300 (about 1.7 FP64 operations per SM and clock): 34 + 2 x 10 FP64 instructions per node and
// increment take ~0.43 ms at 2048^2, five times the HBM time of the increment. Here the same
// closed form (uniform square elements, Walsh combinations of the nodal values, lumped-mass
// classes; see k_elem_force_quad4_square and k_verlet_node_cls_regular) runs on the FP32 pipes
// in pair arithmetic (ffpair.cuh, ~48-bit significands), and the element and node phases are one
// kernel: a CTA loads the displacement of its node tile plus a one-node halo into shared memory,
// computes the element terms of the (TX+1) x (TY+1) elements touching the tile (the halo
// elements are computed by both neighbouring CTAs instead of being exchanged), gathers each
// node's four element contributions in a fixed order and takes the three velocity estimates of
// docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:129-157 and the predictor of the next
// increment (main.cpp:119). The element forces never go to global memory.
//
// State between the increments of one call: pair nodevecs [nnode] of float4 {x.h, x.l, y.h,
// y.l} (16 bytes per node, like a double2) in the workspace, the displacement double-buffered
// (the halo of one CTA is the tile of another: the increment reads one buffer and writes the
// other). The caller's FP64 u, v, a are converted in at the start of a call (after the FP64
// predictor) and out at its end.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "ffpair.cuh"
#include "ffpair2.cuh"

namespace gfgpu {

constexpr int kPairTX = 32;  // nodes per tile in x (= threads per tile row)
constexpr int kPairTY = 8;   // nodes per tile in y
constexpr int kPairThreads = kPairTX * kPairTY;

// pair coefficients of the closed-form velocity estimates per lumped-mass class
// (v' = c1 v + c2 a + c3 mR, a' = mR - be v', mR = mi (fext - f)); see MassClassTab
struct PairClassTab {
    float2 mi[GFGPU_MASS_CLASSES], be[GFGPU_MASS_CLASSES], c1[GFGPU_MASS_CLASSES],
        c2[GFGPU_MASS_CLASSES], c3[GFGPU_MASS_CLASSES];
};

struct PairStep {
    const float4* uin;   // [nnode] displacement of this increment (predicted)
    float4* uout;        // [nnode] predicted displacement of the next increment
    float4* v;           // [nnode] velocity (in/out)
    float4* a;           // [nnode] acceleration (in/out)
    const float4* fext;  // [nnode] external force or null
    const float4* cLN;   // [nelem] {L.h, L.l, N.h, N.l}
    const float2* cH;    // [ny][nxp] {kH.h, kH.l}
    const uchar2* mcls;  // [nnode] lumped-mass class per component
    int nx, ny, nxp;
    int advance;         // write uout
    float2 dt, cc;       // dt and dt^2 / 2 as pairs
};

// Two pair values in a float4. Interleaved {x.h, x.l, y.h, y.l} (lo2, hi2, pack): the element
// forces and the state of pair paths 2 and 3. Packed {x.h, y.h, x.l, y.l} (px_, py_, ppack): the
// state and the {L, N} coefficients of pair path 1, so that a float4 is directly the two
// FP32x2 registers {h, l} of an ff2 (ffpair2.cuh).
__device__ __forceinline__ ffv lo2(float4 q) { return ff_make(q.x, q.y); }
__device__ __forceinline__ ffv hi2(float4 q) { return ff_make(q.z, q.w); }
__device__ __forceinline__ ffv pf(float2 q) { return ff_make(q.x, q.y); }
__device__ __forceinline__ float4 pack(ffv x, ffv y) { return make_float4(x.h, x.l, y.h, y.l); }
__device__ __forceinline__ ffv px_(float4 q) { return ff_make(q.x, q.z); }
__device__ __forceinline__ ffv py_(float4 q) { return ff_make(q.y, q.w); }
__device__ __forceinline__ float4 ppack(ffv x, ffv y) { return make_float4(x.h, y.h, x.l, y.l); }

// pair sum of a nodevec entry's element forces through the gather table (the CSR's entries and
// order; -1 pads): the first term assigned, the others added, as the CSR loop does
__device__ __forceinline__ ffv gather_ell_pair(const int4* __restrict__ ell, const float2* __restrict__ fe,
                                               int64_t t)
{
    const int4 q = __ldg(ell + t);
    ffv f = q.x >= 0 ? pf(__ldg(fe + q.x)) : ff_make(0.f, 0.f);
    if (q.y >= 0) f = ff_add(f, pf(__ldg(fe + q.y)));
    if (q.z >= 0) f = ff_add(f, pf(__ldg(fe + q.z)));
    if (q.w >= 0) f = ff_add(f, pf(__ldg(fe + q.w)));
    return f;
}

// element (ex, ey) of a square-element Regular mesh with per-element L = lam/4, N = G/4 (M = 2N)
// and kH = g^2 (lam + 3G)/4: the sums S = P0 + P1, D = P0 - P1 (x) and P1 + Q1, P1 - Q1 (y) and
// the hourglass terms H, from which the element forces are (H - S, D - H, S + H, -(D + H)) at
// nodes 0..3 (k_elem_force_quad4_square's formulas, every sum and product on pairs)
__device__ __forceinline__ void pair_element(ffv u0x, ffv u0y, ffv u1x, ffv u1y, ffv u2x, ffv u2y, ffv u3x,
                                             ffv u3y, ffv L, ffv N, ffv kH, float4& S, float4& D, float4& H)
{
    const ffv px = ff_sub(u2x, u0x), qx = ff_sub(u1x, u3x);
    const ffv py = ff_sub(u2y, u0y), qy = ff_sub(u1y, u3y);
    const ffv A1x = ff_add(px, qx), A2x = ff_sub(px, qx);
    const ffv A1y = ff_add(py, qy), A2y = ff_sub(py, qy);
    const ffv A3x = ff_sub(ff_add(u0x, u2x), ff_add(u1x, u3x));
    const ffv A3y = ff_sub(ff_add(u0y, u2y), ff_add(u1y, u3y));
    const ffv Lt = ff_mul(L, ff_add(A1x, A2y));
    const ffv P0 = ff_add(ff_twice(ff_mul(N, A1x)), Lt);
    const ffv Q1 = ff_add(ff_twice(ff_mul(N, A2y)), Lt);
    const ffv P1 = ff_mul(N, ff_add(A1y, A2x));
    const ffv H0 = ff_mul(kH, A3x), H1 = ff_mul(kH, A3y);
    S = pack(ff_norm(ff_add(P0, P1)), ff_norm(ff_add(P1, Q1)));
    D = pack(ff_norm(ff_sub(P0, P1)), ff_norm(ff_sub(P1, Q1)));
    H = pack(ff_norm(H0), ff_norm(H1));
}

// The same closed form from the element's node differences P = u2 - u0, Q = u1 - u3 and
// D = u0 - u1, E = u2 - u3 (A1 = P + Q, A2 = P - Q, A3 = D + E), given as pairs: a caller that
// forms them in FP64 from an FP64 displacement keeps the pair rounding at the scale of the
// differences, not of the displacement (an applied affine field cancels exactly as in FP64).
__device__ __forceinline__ void pair_element_diff(ffv Px, ffv Py, ffv Qx, ffv Qy, ffv Dx, ffv Dy, ffv Ex,
                                                  ffv Ey, ffv L, ffv N, ffv kH, float4& S, float4& D, float4& H)
{
    const ffv A1x = ff_add(Px, Qx), A2x = ff_sub(Px, Qx);
    const ffv A1y = ff_add(Py, Qy), A2y = ff_sub(Py, Qy);
    const ffv A3x = ff_add(Dx, Ex), A3y = ff_add(Dy, Ey);
    const ffv Lt = ff_mul(L, ff_add(A1x, A2y));
    const ffv P0 = ff_add(ff_twice(ff_mul(N, A1x)), Lt);
    const ffv Q1 = ff_add(ff_twice(ff_mul(N, A2y)), Lt);
    const ffv P1 = ff_mul(N, ff_add(A1y, A2x));
    const ffv H0 = ff_mul(kH, A3x), H1 = ff_mul(kH, A3y);
    S = pack(ff_norm(ff_add(P0, P1)), ff_norm(ff_add(P1, Q1)));
    D = pack(ff_norm(ff_sub(P0, P1)), ff_norm(ff_sub(P1, Q1)));
    H = pack(ff_norm(H0), ff_norm(H1));
}

// One velocity-Verlet component update (closed form per mass class, or a prescribed dof).
__device__ __forceinline__ void pair_update(int c, ffv f, ffv fx, bool has_fext, ffv vn, ffv an,
                                            const float2* smi, const float2* sbe, const float2* sc1,
                                            const float2* sc2, const float2* sc3, ffv dt, ffv& vv,
                                            ffv& aa)
{
    if (c < GFGPU_MASS_CLASSES) {
        const ffv R = has_fext ? ff_sub(fx, f) : ff_neg(f);
        const ffv mR = ff_mul(pf(smi[c]), R);
        vv = ff_norm(ff_add(ff_add(ff_mul(pf(sc1[c]), vn), ff_mul(pf(sc2[c]), an)), ff_mul(pf(sc3[c]), mR)));
        aa = ff_norm(ff_sub(mR, ff_mul(pf(sbe[c]), vv)));
    }
    else {
        // prescribed dof: the solve leaves a untouched; v follows the three estimates (v + dt a)
        aa = an;
        vv = ff_norm(ff_add(vn, ff_mul(dt, an)));
    }
}

__global__ void __launch_bounds__(kPairThreads)
k_verlet_pair_quad4(const PairStep p, const __grid_constant__ PairClassTab tab)
{
    constexpr int UW = kPairTX + 2, UH = kPairTY + 2;  // displacement tile with a one-node halo
    constexpr int EW = kPairTX + 1, EH = kPairTY + 1;  // elements touching the node tile
    __shared__ float4 su[UH * UW];
    __shared__ float4 sS[EH * EW], sD[EH * EW], sH[EH * EW];
    __shared__ float2 smi[GFGPU_MASS_CLASSES], sbe[GFGPU_MASS_CLASSES], sc1[GFGPU_MASS_CLASSES],
        sc2[GFGPU_MASS_CLASSES], sc3[GFGPU_MASS_CLASSES];
    const int tid = threadIdx.x;
    if (tid < GFGPU_MASS_CLASSES) {
        smi[tid] = tab.mi[tid];
        sbe[tid] = tab.be[tid];
        sc1[tid] = tab.c1[tid];
        sc2[tid] = tab.c2[tid];
        sc3[tid] = tab.c3[tid];
    }
    const int nx = p.nx, ny = p.ny, W = nx + 1;
    const int x0 = blockIdx.x * kPairTX, y0 = blockIdx.y * kPairTY;
    // this thread's node
    const int tx = tid % kPairTX, ty = tid / kPairTX;
    const int ix = x0 + tx, iy = y0 + ty;
    const bool own = ix <= nx && iy <= ny;
    const int node = iy * W + ix;
    // node-phase inputs, loaded first so that they are in flight during the element phase
    float4 vq = make_float4(0.f, 0.f, 0.f, 0.f), aq = vq, fq = vq;
    uchar2 cl = make_uchar2(GFGPU_PRESCRIBED_CLASS, GFGPU_PRESCRIBED_CLASS);
    if (own) {
        vq = p.v[node];
        aq = p.a[node];
        cl = __ldg(p.mcls + node);
        if (p.fext) fq = __ldg(p.fext + node);
    }
    // displacement tile: nodes (x0 - 1 .. x0 + TX, y0 - 1 .. y0 + TY), zero outside the mesh
    for (int k = tid; k < UH * UW; k += kPairThreads) {
        const int gx = x0 - 1 + k % UW, gy = y0 - 1 + k / UW;
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gx >= 0 && gx <= nx && gy >= 0 && gy <= ny) q = __ldg(p.uin + (gy * W + gx));
        su[k] = q;
    }
    __syncthreads();
    // element phase: elements (x0 - 1 .. x0 + TX - 1, y0 - 1 .. y0 + TY - 1); zero terms for
    // elements outside the mesh
    for (int k = tid; k < EH * EW; k += kPairThreads) {
        const int lx = k % EW, ly = k / EW;
        const int ex = x0 - 1 + lx, ey = y0 - 1 + ly;
        float4 S = make_float4(0.f, 0.f, 0.f, 0.f), D = S, H = S;
        if (ex >= 0 && ex < nx && ey >= 0 && ey < ny) {
            const int e = ey * nx + ex;
            const int b = ly * UW + lx; // node (ex, ey) in the tile
            const float4 q0 = su[b], q1 = su[b + 1], q2 = su[b + UW + 1], q3 = su[b + UW];
            const float4 cln = __ldg(p.cLN + e);
            pair_element(px_(q0), py_(q0), px_(q1), py_(q1), px_(q2), py_(q2), px_(q3), py_(q3), px_(cln),
                         py_(cln), pf(__ldg(p.cH + ey * p.nxp + ex)), S, D, H);
        }
        sS[k] = S;
        sD[k] = D;
        sH[k] = H;
    }
    __syncthreads();
    if (!own) return;
    // node (ix, iy): element a = (ix-1, iy-1) holds it as local node 2, b = (ix, iy-1) as 3,
    // c = (ix-1, iy) as 1, d = (ix, iy) as 0; with f(0) = H - S, f(1) = D - H, f(2) = S + H,
    // f(3) = -(D + H): f = (S_a - S_d) + (D_c - D_b) + ((H_a - H_b) + (H_d - H_c))
    const int ka = ty * EW + tx, kb = ka + 1, kc = ka + EW, kd = kc + 1;
    const float4 Sa = sS[ka], Sd = sS[kd], Db = sD[kb], Dc = sD[kc];
    const float4 Ha = sH[ka], Hb = sH[kb], Hc = sH[kc], Hd = sH[kd];
    const ffv fxn = ff_norm(ff_add(ff_add(ff_sub(lo2(Sa), lo2(Sd)), ff_sub(lo2(Dc), lo2(Db))),
                                   ff_add(ff_sub(lo2(Ha), lo2(Hb)), ff_sub(lo2(Hd), lo2(Hc)))));
    const ffv fyn = ff_norm(ff_add(ff_add(ff_sub(hi2(Sa), hi2(Sd)), ff_sub(hi2(Dc), hi2(Db))),
                                   ff_add(ff_sub(hi2(Ha), hi2(Hb)), ff_sub(hi2(Hd), hi2(Hc)))));
    const ffv dt = pf(p.dt);
    const bool hf = p.fext != nullptr;
    ffv vx, ax, vy, ay;
    pair_update(cl.x, fxn, px_(fq), hf, px_(vq), px_(aq), smi, sbe, sc1, sc2, sc3, dt, vx, ax);
    pair_update(cl.y, fyn, py_(fq), hf, py_(vq), py_(aq), smi, sbe, sc1, sc2, sc3, dt, vy, ay);
    p.v[node] = ppack(vx, vy);
    p.a[node] = ppack(ax, ay);
    if (p.advance) {
        const float4 uq = su[(ty + 1) * UW + tx + 1];
        const ffv cc = pf(p.cc);
        const ffv ux = ff_norm(ff_add(ff_add(px_(uq), ff_mul(dt, vx)), ff_mul(cc, ax)));
        const ffv uy = ff_norm(ff_add(ff_add(py_(uq), ff_mul(dt, vy)), ff_mul(cc, ay)));
        p.uout[node] = ppack(ux, uy);
    }
}

// ------------------------------------------------------------------ persistent TMA form
//
// The same increment as k_verlet_pair_quad4, restructured for latency hiding and fewer
// instructions:
//  * persistent CTAs walk the node tiles (tile = blockIdx.x + i gridDim.x); the inputs of the
//    next tile (displacement tile + halo, v, a, the per-element coefficients of the tile's
//    elements) are fetched by TMA (cp.async.bulk.tensor, one thread, completion on an mbarrier)
//    into the other of two shared-memory stages while the current tile is computed. Outside the
//    mesh the copies read zeros, so elements beyond the edges have zero coefficients and
//    contribute nothing: the element phase needs no bounds checks.
//  * a tile is 31 x TY nodes (TY = 15 by default, or 7) with the 32 x (TY + 1) elements around
//    them: the element phase is one element per thread (lane = element column, warp = element
//    row), and in the node phase warp w, lane j owns node (x0 + j, y0 + w) (lane 31 and the last
//    warp only help with the columns).
//  * the x and y components of a node (and the two components of every element term) travel
//    together as the two lanes of packed FP32x2 float-float values (ffpair2.cuh): the state and
//    the {L, N} coefficients are stored {x.h, y.h, x.l, y.l}, so a 16-byte load is one ff2.
//  * the element phase stores only the element terms P0, P1 (= Q0), Q1, H0, H1; the node phase
//    forms, per column of elements below/above a node row, with A = P0_lo + P0_hi,
//    B = P1_lo - P1_hi, C = H0_lo - H0_hi (x; y with P1, Q1, H1):
//      Pcol = (A + C) + B,  Qcol = (A + C) - B,  f_x(ix, iy) = Pcol(ix - 1) - Qcol(ix),
//    which is the four-element sum (S_a - S_d) + (D_c - D_b) + (H_a - H_b) + (H_d - H_c) of the
//    tile kernel regrouped (S = P0 + P1, D = P0 - P1): 33 instead of 40 pair additions per node.
//    Lane j forms the column left of its node, the right column's Qcol comes from lane j + 1.
//  * every wait is bounded: a CTA whose copies do not arrive sets g_pair_timeout, waits (again
//    bounded) for the copies it issued and returns.
__device__ int g_pair_timeout = 0;
constexpr long kPairSpin = 1L << 22;

// Tile geometry of the persistent kernel: TX x TY owned nodes, the (TX + 1) x (TY + 1) = one
// per thread elements around them, the displacement tile with its one-node halo.
template <int TY>
struct TmaGeom {
    static constexpr int TX = 31, EW = TX + 1, EH = TY + 1, UW = TX + 2, UH = TY + 2;
    static constexpr int threads = EW * EH;
    static constexpr int HW = 68; // kH floats per element row box
    static constexpr uint32_t UBytes = UW * UH * 16, VBytes = TX * TY * 16, LBytes = EW * EH * 16,
                              HBytes = HW * EH * 4;
    static constexpr uint32_t StageTx = UBytes + 2 * VBytes + LBytes + HBytes;
    static constexpr uint32_t pad(uint32_t b) { return (b + 127u) / 128u * 128u; }
    // stage layout: u | v | a | cLN | cH, each 128-byte aligned
    static constexpr uint32_t OffV = pad(UBytes), OffA = OffV + pad(VBytes), OffL = OffA + pad(VBytes),
                              OffH = OffL + pad(LBytes), StageBytes = OffH + pad(HBytes);
    static constexpr uint32_t ElemBytes = threads * 48; // (P0, P1), (P1, Q1), (H0, H1) as ff2
    static constexpr uint32_t Smem = 128 + 2 * StageBytes + pad(ElemBytes) + 64;
    static constexpr int min_blocks = threads <= 256 ? 4 : 2;
};
static_assert(TmaGeom<7>::EW == 32, "one warp per element row");
constexpr int kTmaTX = 31;

struct PairTmaStep {
    float4* uout;
    float4* v;
    float4* a;
    const float4* fext;
    const uchar2* mcls;
    int nx, ny, ntx, ntiles;
    int gdx, gdy;        // gridDim.x = gdy ntx + gdx: the tile step in tile columns and rows
    int advance;
    float2 dt, cc;
    unsigned long long nz; // kF2NegZero (the addend of the packed products, read at run time)
};

__device__ __forceinline__ bool pair_wait(uint32_t mbar, uint32_t phase)
{
    for (long it = 0; it < kPairSpin; ++it) {
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

__device__ __forceinline__ void tma_load3(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                          uint32_t mbar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tma_load2(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t mbar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ ffv shfl_down1(ffv x)
{
    return ff_make(__shfl_down_sync(0xffffffffu, x.h, 1), __shfl_down_sync(0xffffffffu, x.l, 1));
}

// first float of the kH box of a tile starting at node x0: 2 (x0 - 1) rounded down to a multiple
// of 4 floats (a 16-byte boundary, as a TMA box's innermost coordinate must be)
__host__ __device__ __forceinline__ int kh_start(int x0)
{
    return (2 * (x0 - 1)) & ~3;
}

template <int TY>
__global__ void __launch_bounds__(TmaGeom<TY>::threads, TmaGeom<TY>::min_blocks)
k_verlet_pair_tma(const __grid_constant__ CUtensorMap mu, const __grid_constant__ CUtensorMap mv,
                  const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap ml,
                  const __grid_constant__ CUtensorMap mh, const PairTmaStep p,
                  const __grid_constant__ PairClassTab tab)
{
    using Gm = TmaGeom<TY>;
    constexpr int kTmaTY = TY, kTmaEW = Gm::EW, kTmaUW = Gm::UW, kTmaThreads = Gm::threads, kTmaHW = Gm::HW;
    constexpr uint32_t kStageBytes = Gm::StageBytes, kOffV = Gm::OffV, kOffA = Gm::OffA, kOffL = Gm::OffL,
                       kOffH = Gm::OffH, kTmaStageTx = Gm::StageTx;
    extern __shared__ unsigned char pair_smem[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(pair_smem) + 127) & ~uintptr_t(127));
    unsigned char* elem = base + 2 * kStageBytes;
    // element terms (two pair lanes each): (P0, P1), (P1, Q1), (H0, H1)
    ulonglong2* sPP = reinterpret_cast<ulonglong2*>(elem);
    ulonglong2* sPQ = sPP + kTmaThreads;
    ulonglong2* sHH = sPQ + kTmaThreads;
    uint64_t* bars = reinterpret_cast<uint64_t*>(elem + Gm::pad(Gm::ElemBytes));
    // class coefficients as separate high / low floats: the two lanes' coefficients of an ff2 are
    // then two plain loads into the two halves of its registers
    __shared__ float scf[10][GFGPU_MASS_CLASSES]; // mi, be, c1, c2, c3: high parts, then low parts
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t s_bar = static_cast<uint32_t>(__cvta_generic_to_shared(bars));
    if (tid < GFGPU_MASS_CLASSES) {
        const float2 cf[5] = {tab.mi[tid], tab.be[tid], tab.c1[tid], tab.c2[tid], tab.c3[tid]};
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            scf[k][tid] = cf[k].x;
            scf[5 + k][tid] = cf[k].y;
        }
    }
    auto issue = [&](int tile, int st) {
        const int x0 = (tile % p.ntx) * kTmaTX, y0 = (tile / p.ntx) * kTmaTY;
        const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(base + st * kStageBytes));
        const uint32_t mb = s_bar + 8u * st;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb), "r"(kTmaStageTx)
                     : "memory");
        tma_load3(d, &mu, 0, x0 - 1, y0 - 1, mb);
        tma_load3(d + kOffV, &mv, 0, x0, y0, mb);
        tma_load3(d + kOffA, &ma, 0, x0, y0, mb);
        tma_load3(d + kOffL, &ml, 0, x0 - 1, y0 - 1, mb);
        tma_load2(d + kOffH, &mh, kh_start(x0), y0 - 1, mb);
    };
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_bar) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_bar + 8u) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&mu)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&mv)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&ma)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&ml)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&mh)) : "memory");
        if (static_cast<int>(blockIdx.x) < p.ntiles) issue(blockIdx.x, 0);
    }
    const int nx = p.nx, ny = p.ny, W = nx + 1;
    const ffv dt = pf(p.dt), cc = pf(p.cc);
    const ff2 DT = ff2_bcast(dt), CC = ff2_bcast(cc);
    const f2 NZ = p.nz;
    const bool hf = p.fext != nullptr;
    // element phase: this thread's element (x0 - 1 + lane, y0 - 1 + warp); its nodes in the tile
    const int b0 = warp * kTmaUW + lane;
    int i = 0;
    int tcol = static_cast<int>(blockIdx.x) % p.ntx, trow = static_cast<int>(blockIdx.x) / p.ntx;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++i) {
        const int st = i & 1;
        __syncthreads(); // the other stage and the element terms are free; barriers initialised
        const int next = tile + gridDim.x;
        if (tid == 0 && next < p.ntiles) issue(next, st ^ 1);
        const int x0 = tcol * kTmaTX, y0 = trow * kTmaTY;
        tcol += p.gdx;
        trow += p.gdy;
        if (tcol >= p.ntx) {
            tcol -= p.ntx;
            ++trow;
        }
        const int ix = x0 + lane, iy = y0 + warp;
        const bool own = lane < kTmaTX && warp < kTmaTY && ix <= nx && iy <= ny;
        const int node = iy * W + ix;
        uchar2 cl = make_uchar2(GFGPU_PRESCRIBED_CLASS, GFGPU_PRESCRIBED_CLASS);
        float4 fq = make_float4(0.f, 0.f, 0.f, 0.f);
        if (own) {
            cl = __ldg(p.mcls + node);
            if (hf) fq = __ldg(p.fext + node);
        }
        const bool ok = pair_wait(s_bar + 8u * st, (i >> 1) & 1);
        const unsigned char* sg = base + st * kStageBytes;
        const ulonglong2* su = reinterpret_cast<const ulonglong2*>(sg);
        auto ldu = [&](int k) {
            const ulonglong2 q = su[k];
            return ff2_make(q.x, q.y);
        };
        if (ok) {
            // both components at once (ff2 lanes x, y)
            const ff2 U0 = ldu(b0), U1 = ldu(b0 + 1), U2 = ldu(b0 + kTmaUW + 1), U3 = ldu(b0 + kTmaUW);
            const ff2 P = ff2_sub(U2, U0), Q = ff2_sub(U1, U3);
            const ff2 A1 = ff2_add(P, Q), A2 = ff2_sub(P, Q);
            const ff2 A3 = ff2_sub(ff2_add(U0, U2), ff2_add(U1, U3));
            // (t, s) = (A1x + A2y, A1y + A2x); (Lt, P1) = (L t, N s)
            const ff2 A2s = ff2_make(f2_make(f2_hi(A2.h), f2_lo(A2.h)), f2_make(f2_hi(A2.l), f2_lo(A2.l)));
            const ff2 ts = ff2_add(A1, A2s);
            const ulonglong2 cq = reinterpret_cast<const ulonglong2*>(sg + kOffL)[tid]; // {L, N} packed
            const ff2 LN = ff2_make(cq.x, cq.y);
            const ff2 LtP1 = ff2_mul(LN, ts, NZ);
            // (P0, Q1) = M (A1x, A2y) + (Lt, Lt), M = 2N
            const ffv N = ff2_lane1(LN), Lt = ff2_lane0(LtP1);
            const ff2 M2 = ff2_bcast(ff_twice(N));
            const ff2 dg = ff2_make(f2_make(f2_lo(A1.h), f2_hi(A2.h)), f2_make(f2_lo(A1.l), f2_hi(A2.l)));
            const ff2 PQ = ff2_add(ff2_mul(M2, dg, NZ), ff2_bcast(Lt));
            const int kr = (2 * (x0 - 1) - kh_start(x0)) >> 1; // 0 or 1 pairs into the box row
            const ffv kH = pf(reinterpret_cast<const float2*>(sg + kOffH)[warp * (kTmaHW / 2) + kr + lane]);
            const ff2 H = ff2_mul(ff2_bcast(kH), A3, NZ); // (H0, H1)
            // element terms (P0, P1), (P1, Q1), (H0, H1)
            sPP[tid] = make_ulonglong2(f2_make(f2_lo(PQ.h), f2_hi(LtP1.h)), f2_make(f2_lo(PQ.l), f2_hi(LtP1.l)));
            sPQ[tid] = make_ulonglong2(f2_make(f2_hi(LtP1.h), f2_hi(PQ.h)), f2_make(f2_hi(LtP1.l), f2_hi(PQ.l)));
            sHH[tid] = make_ulonglong2(H.h, H.l);
        }
        // the element terms are complete; a CTA whose copies did not arrive stops here
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                // let the copies this CTA issued land (bounded) before its shared memory is released
                atomicExch(&g_pair_timeout, 1);
                pair_wait(s_bar + 8u * st, (i >> 1) & 1);
                if (next < p.ntiles) pair_wait(s_bar + 8u * (st ^ 1), ((i + 1) >> 1) & 1);
            }
            return;
        }
        if (warp >= kTmaTY) continue; // the last element row only feeds the node rows below it
        // node phase: the element column left of node (x0 + lane, y0 + warp): lo = element row
        // warp (below the node row), hi = warp + 1; lane x: A = P0lo + P0hi, B = P1lo - P1hi,
        // C = H0lo - H0hi; lane y: A = P1lo + P1hi, B = Q1lo - Q1hi, C = H1lo - H1hi
        const int kl = tid, kh = tid + kTmaEW;
        auto lde = [](const ulonglong2* t, int k) {
            const ulonglong2 q = t[k];
            return ff2_make(q.x, q.y);
        };
        const ff2 Ac = ff2_add(lde(sPP, kl), lde(sPP, kh));
        const ff2 Bc = ff2_sub(lde(sPQ, kl), lde(sPQ, kh));
        const ff2 Ec = ff2_add(Ac, ff2_sub(lde(sHH, kl), lde(sHH, kh)));
        const ff2 Qc = ff2_sub(Ec, Bc);
        const ff2 Qr = ff2_make(__shfl_down_sync(0xffffffffu, Qc.h, 1), __shfl_down_sync(0xffffffffu, Qc.l, 1));
        if (!own) continue;
        const ff2 F = ff2_sub(ff2_add(Ec, Bc), Qr); // (f_x, f_y)
        const int ln = warp * kTmaTX + lane;
        const ulonglong2 vq = reinterpret_cast<const ulonglong2*>(sg + kOffV)[ln];
        const ulonglong2 aq = reinterpret_cast<const ulonglong2*>(sg + kOffA)[ln];
        const ff2 VN = ff2_make(vq.x, vq.y), AN = ff2_make(aq.x, aq.y);
        const ff2 FX = ff2_make(f2_make(fq.x, fq.y), f2_make(fq.z, fq.w));
        ff2 VV, AA;
        if (cl.x < GFGPU_MASS_CLASSES && cl.y < GFGPU_MASS_CLASSES) {
            const int cx = cl.x, cy = cl.y;
            auto coef = [&](int k) {
                return ff2_make(f2_make(scf[k][cx], scf[k][cy]), f2_make(scf[5 + k][cx], scf[5 + k][cy]));
            };
            const ff2 R = hf ? ff2_sub(FX, F) : ff2_neg(F);
            const ff2 mR = ff2_mul(coef(0), R, NZ);
            VV = ff2_norm(ff2_add(ff2_add(ff2_mul(coef(2), VN, NZ), ff2_mul(coef(3), AN, NZ)), ff2_mul(coef(4), mR, NZ)));
            AA = ff2_norm(ff2_sub(mR, ff2_mul(coef(1), VV, NZ)));
        }
        else {
            // a prescribed component (boundary rows): lane by lane
            ffv vl[2], al[2];
            const ffv fl[2] = {ff2_lane0(F), ff2_lane1(F)}, xl[2] = {ff2_lane0(FX), ff2_lane1(FX)};
            const ffv vn[2] = {ff2_lane0(VN), ff2_lane1(VN)}, an[2] = {ff2_lane0(AN), ff2_lane1(AN)};
            const int cs[2] = {cl.x, cl.y};
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int c = cs[k];
                if (c < GFGPU_MASS_CLASSES) {
                    const ffv R = hf ? ff_sub(xl[k], fl[k]) : ff_neg(fl[k]);
                    const ffv mR = ff_mul(ff_make(scf[0][c], scf[5][c]), R);
                    vl[k] = ff_norm(ff_add(ff_add(ff_mul(ff_make(scf[2][c], scf[7][c]), vn[k]),
                                                  ff_mul(ff_make(scf[3][c], scf[8][c]), an[k])),
                                           ff_mul(ff_make(scf[4][c], scf[9][c]), mR)));
                    al[k] = ff_norm(ff_sub(mR, ff_mul(ff_make(scf[1][c], scf[6][c]), vl[k])));
                }
                else {
                    al[k] = an[k];
                    vl[k] = ff_norm(ff_add(vn[k], ff_mul(dt, an[k])));
                }
            }
            VV = ff2_from(vl[0], vl[1]);
            AA = ff2_from(al[0], al[1]);
        }
        reinterpret_cast<ulonglong2*>(p.v)[node] = make_ulonglong2(VV.h, VV.l);
        reinterpret_cast<ulonglong2*>(p.a)[node] = make_ulonglong2(AA.h, AA.l);
        if (p.advance) {
            const ff2 U = ldu((warp + 1) * kTmaUW + lane + 1);
            const ff2 UN = ff2_norm(ff2_add(ff2_add(U, ff2_mul(DT, VV, NZ)), ff2_mul(CC, AA, NZ)));
            reinterpret_cast<ulonglong2*>(p.uout)[node] = make_ulonglong2(UN.h, UN.l);
        }
    }
}

// ------------------------------------------------------------------ element kernel + CSR node kernel
//
// The pair path for Quad4 meshes that are not the Regular square-element case: an element kernel
// writes the element forces as pairs, fe[e * 4 + m] = {fx.h, fx.l, fy.h, fy.l}, and a node kernel
// gathers them through the dof CSR (ascending flat elemvec index, the order of Vector.h:724-741;
// periodic ties allowed) and takes the three velocity estimates and the predictor, all on pairs.
// Element forces: the square closed form (pair_element) on uniform square elements, otherwise the
// stored element stiffness K_e times u_e. The stiffness is K_e[(m,j),(n,l)] = sum_q vol_q (lam
// dNx(m,j) dNx(n,l) + G (delta_jl dNx(m,.).dNx(n,.) + dNx(m,l) dNx(n,j))), the linear map of the
// reference's chain symGradN -> stress -> int_gradN_dot_tensor2_dV (ElementQuad4.h:407-491) for
// sigma = K tr(eps) I + 2 G dev(eps). It is symmetric, and a rigid translation gives no force
// (sum_n dNx(n,.) = 0), so sum_n K_e[(m,j),(n,l)] = 0 for every m, j, l: the diagonal node blocks
// follow from the off-diagonal ones, and f_(m,j) = sum_{n != m} sum_l K_e[(m,j),(n,l)]
// (u_(n,l) - u_(m,l)). Only the 6 off-diagonal 2 x 2 node blocks are stored: 24 pairs per element
// instead of 36 for the symmetric matrix (a third fewer bytes in the HBM-bound element kernel).

// node pairs (m, n), m < n, in storage order, and the storage index of K_e[(m,j),(n,l)]
__host__ __device__ constexpr int pair_m(int p)
{
    return p < 3 ? 0 : (p < 5 ? 1 : 2);
}

__host__ __device__ constexpr int pair_n(int p)
{
    return p < 3 ? p + 1 : (p < 5 ? p - 1 : 3);
}

__host__ __device__ constexpr int tri8(int r, int c)
{
    // packed upper triangle of an 8 x 8 matrix, r <= c, row by row
    return r * 8 - r * (r - 1) / 2 + (c - r);
}

__global__ void k_pair_stiffness(const double* __restrict__ dNx, const double* __restrict__ vol,
                                 const double* __restrict__ Km, const double* __restrict__ Gm, int64_t nelem,
                                 int nip, float2* __restrict__ Ke)
{
    GF_FOR(e, nelem)
    {
        double k[36];
#pragma unroll
        for (int i = 0; i < 36; ++i) k[i] = 0.0;
        const double G = Gm[e], lam = Km[e] - 2.0 * G / 3.0;
        for (int q = 0; q < nip; ++q) {
            double g[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) g[i] = dNx[(e * nip + q) * 8 + i];
            const double v = vol[e * nip + q];
#pragma unroll
            for (int r = 0; r < 8; ++r)
#pragma unroll
                for (int c = r; c < 8; ++c) {
                    const int m = r / 2, j = r % 2, n = c / 2, l = c % 2;
                    const double dd = g[m * 2] * g[n * 2] + g[m * 2 + 1] * g[n * 2 + 1];
                    const double val = lam * g[m * 2 + j] * g[n * 2 + l] + G * ((j == l ? dd : 0.0) + g[m * 2 + l] * g[n * 2 + j]);
                    k[tri8(r, c)] += v * val;
                }
        }
        // the off-diagonal node blocks K_e[(m,j),(n,l)], m < n: 24 pairs
#pragma unroll
        for (int p = 0; p < 6; ++p)
#pragma unroll
            for (int jl = 0; jl < 4; ++jl) {
                const int r = 2 * pair_m(p) + jl / 2, c = 2 * pair_n(p) + jl % 2;
                const ffv x = ff_from_double(k[tri8(r, c)]);
                Ke[(p * 4 + jl) * nelem + e] = make_float2(x.h, x.l);
            }
    }
}

// element-indexed pair coefficients of the square closed form: cLN[e] = {L, N}, cH[e] = kH
__global__ void k_pair_coef_elem(const double* __restrict__ Km, const double* __restrict__ Gm, int64_t nelem,
                                 double g2, float4* __restrict__ cLN, float2* __restrict__ cH)
{
    GF_FOR(e, nelem)
    {
        const double K = Km[e], G = Gm[e];
        const double lam = K - 2.0 * G / 3.0;
        cLN[e] = pack(ff_from_double(0.25 * lam), ff_from_double(0.25 * G));
        const ffv kH = ff_from_double(0.25 * g2 * (lam + 3.0 * G));
        cH[e] = make_float2(kH.h, kH.l);
    }
}

__global__ void k_pair_split(const double* __restrict__ x, int64_t n, float2* __restrict__ out)
{
    GF_FOR(i, n)
    {
        const ffv y = ff_from_double(x[i]);
        out[i] = make_float2(y.h, y.l);
    }
}

__global__ void k_pair_join(const float2* __restrict__ in, int64_t n, double* __restrict__ out)
{
    GF_FOR(i, n) out[i] = ff_to_double(pf(in[i]));
}

__global__ void __launch_bounds__(256)
k_pair_elem_square(const int32_t* __restrict__ conn, const float4* __restrict__ u, const float4* __restrict__ cLN,
                   const float2* __restrict__ cH, int64_t nelem, float4* __restrict__ fe)
{
    GF_FOR(e, nelem)
    {
        const int4 cn = __ldg(reinterpret_cast<const int4*>(conn) + e);
        float4 S, D, H;
        const float4 q0 = __ldg(u + cn.x), q1 = __ldg(u + cn.y), q2 = __ldg(u + cn.z), q3 = __ldg(u + cn.w);
        const float4 cln = __ldg(cLN + e);
        pair_element(lo2(q0), hi2(q0), lo2(q1), hi2(q1), lo2(q2), hi2(q2), lo2(q3), hi2(q3), lo2(cln), hi2(cln),
                     pf(__ldg(cH + e)), S, D, H);
        const ffv Sx = lo2(S), Sy = hi2(S), Dx = lo2(D), Dy = hi2(D), H0 = lo2(H), H1 = hi2(H);
        float4* o = fe + e * 4;
        o[0] = pack(ff_norm(ff_sub(H0, Sx)), ff_norm(ff_sub(H1, Sy)));
        o[1] = pack(ff_norm(ff_sub(Dx, H0)), ff_norm(ff_sub(Dy, H1)));
        o[2] = pack(ff_norm(ff_add(Sx, H0)), ff_norm(ff_add(Sy, H1)));
        o[3] = pack(ff_norm(ff_neg(ff_add(Dx, H0))), ff_norm(ff_neg(ff_add(Dy, H1))));
    }
}

// Element forces of uniform square Quad4 elements in pair arithmetic with FP64 input and output
// (the static solvers' operator and the explicit step's element kernel in "mixed" arithmetic): the
// node differences of the square closed form are formed in FP64 (8 subtractions), split into pairs
// on the integer pipe, the closed form runs on pairs (pair_element_diff) and the forces are joined
// to FP64 into fe [nelem, 4, 2] (the layout of k_elem_force_quad4_square that the FP64 gathers and
// node kernels read): 16 FP64 instructions per element instead of 34. Forming the differences in
// FP64 keeps the pair rounding relative to them: an applied affine displacement cancels as in FP64.
// PAIR_OUT: the forces stay pairs, normalised, fe [nelem, 4] of float4 {x.h, x.l, y.h, y.l} (8 bytes
// per value like the FP64 layout; the mixed node kernel gathers them).
template <bool PAIR_OUT>
__global__ void __launch_bounds__(256)
k_pair_elem_square_f64(const int32_t* __restrict__ conn, const double2* __restrict__ u,
                       const float4* __restrict__ cLN, const float2* __restrict__ cH, int64_t nelem,
                       double2* __restrict__ fe)
{
    GF_FOR(e, nelem)
    {
        const int4 cn = __ldg(reinterpret_cast<const int4*>(conn) + e);
        const double2 q0 = __ldg(u + cn.x), q1 = __ldg(u + cn.y), q2 = __ldg(u + cn.z), q3 = __ldg(u + cn.w);
        const float4 cln = __ldg(cLN + e);
        float4 S, D, H;
        pair_element_diff(ff_from_double(q2.x - q0.x), ff_from_double(q2.y - q0.y), ff_from_double(q1.x - q3.x),
                          ff_from_double(q1.y - q3.y), ff_from_double(q0.x - q1.x), ff_from_double(q0.y - q1.y),
                          ff_from_double(q2.x - q3.x), ff_from_double(q2.y - q3.y), lo2(cln), hi2(cln),
                          pf(__ldg(cH + e)), S, D, H);
        const ffv Sx = lo2(S), Sy = hi2(S), Dx = lo2(D), Dy = hi2(D), H0 = lo2(H), H1 = hi2(H);
        const ffv f[8] = {ff_sub(H0, Sx), ff_sub(H1, Sy), ff_sub(Dx, H0), ff_sub(Dy, H1),
                          ff_add(Sx, H0), ff_add(Sy, H1), ff_neg(ff_add(Dx, H0)), ff_neg(ff_add(Dy, H1))};
        if constexpr (PAIR_OUT) {
            float4* o = reinterpret_cast<float4*>(fe) + e * 4;
#pragma unroll
            for (int m = 0; m < 4; ++m) o[m] = pack(ff_norm(f[2 * m]), ff_norm(f[2 * m + 1]));
        }
        else {
            double2* o = fe + e * 4;
#pragma unroll
            for (int m = 0; m < 4; ++m) o[m] = make_double2(ff_to_double(f[2 * m]), ff_to_double(f[2 * m + 1]));
        }
    }
}

// The node update of mixed arithmetic (FP64 state, pair element forces from
// k_pair_elem_square_f64<true>): a dof's pair forces gathered in the CSR's order (or by index
// arithmetic on a Regular numbering, the same order), the closed form of the three velocity
// estimates with the lumped-mass class's coefficients on pairs (v and a split from FP64 on the
// integer pipe), v' and a' returned to FP64, and the predictor u + dt v' + c a' in FP64 as in
// k_verlet_node_cls. 4 FP64 instructions per free dof instead of 10; prescribed dofs as there.
struct MixedNodeStep {
    const int32_t *dofs, *ptr, *idx;
    const uint8_t* mclass;
    const float2* fe; // [nelem * nne * ndim] pair element forces
    const double* fext;
    double *u, *v, *a;
    int64_t n, reg_nx, reg_ny;
    const int4* ell;
    double dt, h, c;
    int advance;
};

__global__ void __launch_bounds__(256)
k_mixed_node(const MixedNodeStep p, const __grid_constant__ PairClassTab tab)
{
    __shared__ float2 smi[GFGPU_MASS_CLASSES], sbe[GFGPU_MASS_CLASSES], sc1[GFGPU_MASS_CLASSES],
        sc2[GFGPU_MASS_CLASSES], sc3[GFGPU_MASS_CLASSES];
    if (threadIdx.x < GFGPU_MASS_CLASSES) {
        const int c = threadIdx.x;
        smi[c] = tab.mi[c];
        sbe[c] = tab.be[c];
        sc1[c] = tab.c1[c];
        sc2[c] = tab.c2[c];
        sc3[c] = tab.c3[c];
    }
    __syncthreads();
    GF_FOR(t, p.n)
    {
        ffv f = ff_make(0.f, 0.f);
        if (p.reg_nx > 0) {
            const uint32_t nx = static_cast<uint32_t>(p.reg_nx), ny = static_cast<uint32_t>(p.reg_ny);
            const uint32_t tt = static_cast<uint32_t>(t), node = tt >> 1, i = tt & 1u, W = nx + 1u;
            const uint32_t iy = node / W, ix = node - iy * W;
            bool first = true;
            auto add = [&](uint32_t e, uint32_t m) {
                const ffv g = pf(__ldg(p.fe + (e * 4u + m) * 2u + i));
                f = first ? g : ff_add(f, g);
                first = false;
            };
            if (iy > 0u && ix > 0u) add((iy - 1u) * nx + ix - 1u, 2u);
            if (iy > 0u && ix < nx) add((iy - 1u) * nx + ix, 3u);
            if (iy < ny && ix > 0u) add(iy * nx + ix - 1u, 1u);
            if (iy < ny && ix < nx) add(iy * nx + ix, 0u);
        }
        else if (p.ell) {
            f = gather_ell_pair(p.ell, p.fe, t);
        }
        else {
            const int32_t d = __ldg(p.dofs + t);
            const int32_t b = __ldg(p.ptr + d), en = __ldg(p.ptr + d + 1);
            for (int32_t j = b; j < en; ++j) {
                const ffv g = pf(__ldg(p.fe + __ldg(p.idx + j)));
                f = j == b ? g : ff_add(f, g);
            }
        }
        const int c = __ldg(p.mclass + t);
        const double vn = p.v[t], an = p.a[t];
        double vv, aa;
        if (c < GFGPU_MASS_CLASSES) {
            const ffv R = p.fext ? ff_sub(ff_from_double(__ldg(p.fext + t)), f) : ff_neg(f);
            const ffv mR = ff_mul(pf(smi[c]), R);
            const ffv V = ff_add(ff_add(ff_mul(pf(sc1[c]), ff_from_double(vn)), ff_mul(pf(sc2[c]), ff_from_double(an))),
                                 ff_mul(pf(sc3[c]), mR));
            const ffv Vn = ff_norm(V);
            const ffv Ac = ff_sub(mR, ff_mul(pf(sbe[c]), Vn));
            vv = ff_to_double(Vn);
            aa = ff_to_double(Ac);
        }
        else {
            aa = an;
            vv = fma(p.h, an + an, vn);
        }
        p.v[t] = vv;
        p.a[t] = aa;
        if (p.advance) p.u[t] = fma(p.c, aa, fma(p.dt, vv, p.u[t]));
    }
}

__global__ void __launch_bounds__(128)
k_pair_elem_stiff(const int32_t* __restrict__ conn, const float4* __restrict__ u, const float2* __restrict__ Ke,
                  int64_t nelem, float4* __restrict__ fe)
{
    GF_FOR(e, nelem)
    {
        const int4 cn = __ldg(reinterpret_cast<const int4*>(conn) + e);
        const float4 q[4] = {__ldg(u + cn.x), __ldg(u + cn.y), __ldg(u + cn.z), __ldg(u + cn.w)};
        ffv f[8];
        bool first[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            f[r] = ff_make(0.f, 0.f);
            first[r] = true;
        }
        auto acc = [&](int r, ffv t) {
            f[r] = first[r] ? t : ff_add(f[r], t);
            first[r] = false;
        };
        // per node pair (m, n), m < n: D = u_n - u_m; f_m += B D, f_n -= B^T D (B = K_e[(m,.),(n,.)])
#pragma unroll
        for (int p = 0; p < 6; ++p) {
            const int m = pair_m(p), n = pair_n(p);
            const ffv D0 = ff_sub(lo2(q[n]), lo2(q[m])), D1 = ff_sub(hi2(q[n]), hi2(q[m]));
            ffv B[4];
#pragma unroll
            for (int jl = 0; jl < 4; ++jl) B[jl] = pf(__ldg(Ke + (p * 4 + jl) * nelem + e));
            acc(2 * m, ff_add(ff_mul(B[0], D0), ff_mul(B[1], D1)));
            acc(2 * m + 1, ff_add(ff_mul(B[2], D0), ff_mul(B[3], D1)));
            acc(2 * n, ff_neg(ff_add(ff_mul(B[0], D0), ff_mul(B[2], D1))));
            acc(2 * n + 1, ff_neg(ff_add(ff_mul(B[1], D0), ff_mul(B[3], D1))));
        }
        float4* o = fe + e * 4;
#pragma unroll
        for (int m = 0; m < 4; ++m) o[m] = pack(ff_norm(f[2 * m]), ff_norm(f[2 * m + 1]));
    }
}

struct PairCsrStep {
    const int32_t *dofs, *ptr, *idx, *part;
    int64_t nnu, n;
    const uint8_t* mclass;  // per nodevec entry, or null: per-dof inverse mass minv
    const float2* minv;     // [nnu] pair inverse lumped mass (no classes)
    const float2* fe;       // [nelem * nne * ndim] element forces
    const float2* fext;     // per nodevec entry or null
    float2 *u, *v, *a;      // per nodevec entry
    float2 dt, h, cc, eta;
    int advance;
    // Mesh::Quad4::Regular(reg_nx, reg_ny) numbering with plain dofs (gfgpu_verlet_detect_regular):
    // a dof's element forces found by index arithmetic in the CSR's order (same bits, no tables)
    int64_t reg_nx, reg_ny;
    const int4* ell; // else, when set: the CSR entries per nodevec entry (gfgpu_verlet_build_ell)
};


__global__ void __launch_bounds__(256)
k_pair_node_csr(const PairCsrStep p, const __grid_constant__ PairClassTab tab)
{
    __shared__ float2 smi[GFGPU_MASS_CLASSES], sbe[GFGPU_MASS_CLASSES], sc1[GFGPU_MASS_CLASSES],
        sc2[GFGPU_MASS_CLASSES], sc3[GFGPU_MASS_CLASSES];
    if (threadIdx.x < GFGPU_MASS_CLASSES) {
        const int c = threadIdx.x;
        smi[c] = tab.mi[c];
        sbe[c] = tab.be[c];
        sc1[c] = tab.c1[c];
        sc2[c] = tab.c2[c];
        sc3[c] = tab.c3[c];
    }
    __syncthreads();
    const ffv dt = pf(p.dt), h = pf(p.h), cc = pf(p.cc);
    GF_FOR(t, p.n)
    {
        ffv f = ff_make(0.f, 0.f);
        if (p.reg_nx > 0) {
            // node (ix, iy): elements (ix-1, iy-1) node 2, (ix, iy-1) node 3, (ix-1, iy) node 1,
            // (ix, iy) node 0, i.e. ascending flat elemvec index as in the CSR
            const uint32_t nx = static_cast<uint32_t>(p.reg_nx), ny = static_cast<uint32_t>(p.reg_ny);
            const uint32_t tt = static_cast<uint32_t>(t), node = tt >> 1, i = tt & 1u, W = nx + 1u;
            const uint32_t iy = node / W, ix = node - iy * W;
            bool first = true;
            auto add = [&](uint32_t e, uint32_t m) {
                const ffv g = pf(__ldg(p.fe + (e * 4u + m) * 2u + i));
                f = first ? g : ff_add(f, g);
                first = false;
            };
            if (iy > 0u && ix > 0u) add((iy - 1u) * nx + ix - 1u, 2u);
            if (iy > 0u && ix < nx) add((iy - 1u) * nx + ix, 3u);
            if (iy < ny && ix > 0u) add(iy * nx + ix - 1u, 1u);
            if (iy < ny && ix < nx) add(iy * nx + ix, 0u);
        }
        else if (p.ell) {
            f = gather_ell_pair(p.ell, p.fe, t);
        }
        else {
            const int32_t d = __ldg(p.dofs + t);
            const int32_t b = __ldg(p.ptr + d), en = __ldg(p.ptr + d + 1);
            for (int32_t j = b; j < en; ++j) {
                const ffv g = pf(__ldg(p.fe + __ldg(p.idx + j)));
                f = j == b ? g : ff_add(f, g);
            }
        }
        f = ff_norm(f);
        const ffv fx = p.fext ? pf(__ldg(p.fext + t)) : ff_make(0.f, 0.f);
        const ffv vn = pf(p.v[t]), an = pf(p.a[t]);
        ffv vv, aa;
        if (p.mclass) {
            pair_update(__ldg(p.mclass + t), f, fx, p.fext != nullptr, vn, an, smi, sbe, sc1, sc2, sc3, dt, vv, aa);
        }
        else {
            const int32_t q = __ldg(p.part + t);
            if (q < p.nnu) {
                // the closed form of the three estimates with this dof's coefficients (MassClassTab)
                const ffv mi = pf(__ldg(p.minv + q));
                const ffv be = ff_mul(mi, pf(p.eta));
                const ffv x = ff_norm(ff_mul(h, be));
                const ffv omh = ff_norm(ff_sub(ff_make(1.f, 0.f), x));
                const ffv x2 = ff_mul(x, x);
                const ffv c1 = ff_add(omh, x2), c3 = ff_mul(h, omh);
                const ffv c2 = ff_add(c3, ff_mul(x2, dt));
                const ffv R = p.fext ? ff_sub(fx, f) : ff_neg(f);
                const ffv mR = ff_mul(mi, R);
                vv = ff_norm(ff_add(ff_add(ff_mul(c1, vn), ff_mul(c2, an)), ff_mul(c3, mR)));
                aa = ff_norm(ff_sub(mR, ff_mul(be, vv)));
            }
            else {
                aa = an;
                vv = ff_norm(ff_add(vn, ff_mul(dt, an)));
            }
        }
        p.v[t] = make_float2(vv.h, vv.l);
        p.a[t] = make_float2(aa.h, aa.l);
        if (p.advance) {
            const ffv un = pf(p.u[t]);
            const ffv uu = ff_norm(ff_add(ff_add(un, ff_mul(dt, vv)), ff_mul(cc, aa)));
            p.u[t] = make_float2(uu.h, uu.l);
        }
    }
}

// FP64 in: the predictor u + dt v + dt^2/2 a of the first increment (FP64, as k_predict), then
// u, v, a (and fext) as pairs
// packed: pair path 1's layout {x.h, y.h, x.l, y.l}, else interleaved {x.h, x.l, y.h, y.l}
__device__ __forceinline__ float4 lay(ffv x, ffv y, bool packed)
{
    return packed ? ppack(x, y) : pack(x, y);
}

__global__ void k_pair_begin(const double2* __restrict__ u, const double2* __restrict__ v,
                             const double2* __restrict__ a, const double2* __restrict__ fext,
                             int64_t nnode, double dt, double c, int packed, float4* __restrict__ pu,
                             float4* __restrict__ pv, float4* __restrict__ pa, float4* __restrict__ pf_)
{
    GF_FOR(n, nnode)
    {
        const double2 un = u[n], vn = v[n], an = a[n];
        const double ux = fma(c, an.x, fma(dt, vn.x, un.x)), uy = fma(c, an.y, fma(dt, vn.y, un.y));
        pu[n] = lay(ff_from_double(ux), ff_from_double(uy), packed);
        pv[n] = lay(ff_from_double(vn.x), ff_from_double(vn.y), packed);
        pa[n] = lay(ff_from_double(an.x), ff_from_double(an.y), packed);
        if (fext) {
            const double2 fn = fext[n];
            pf_[n] = lay(ff_from_double(fn.x), ff_from_double(fn.y), packed);
        }
    }
}

__global__ void k_pair_end(const float4* __restrict__ pu, const float4* __restrict__ pv,
                           const float4* __restrict__ pa, int64_t nnode, int packed, double2* __restrict__ u,
                           double2* __restrict__ v, double2* __restrict__ a)
{
    GF_FOR(n, nnode)
    {
        const float4 qu = pu[n], qv = pv[n], qa = pa[n];
        if (packed) {
            u[n] = make_double2(ff_to_double(px_(qu)), ff_to_double(py_(qu)));
            v[n] = make_double2(ff_to_double(px_(qv)), ff_to_double(py_(qv)));
            a[n] = make_double2(ff_to_double(px_(qa)), ff_to_double(py_(qa)));
        }
        else {
            u[n] = make_double2(ff_to_double(lo2(qu)), ff_to_double(hi2(qu)));
            v[n] = make_double2(ff_to_double(lo2(qv)), ff_to_double(hi2(qv)));
            a[n] = make_double2(ff_to_double(lo2(qa)), ff_to_double(hi2(qa)));
        }
    }
}

// per-element pair coefficients: cLN[e] = {L, N}, cH[ey * nxp + ex] = kH (see pair_element);
// one thread per entry of the padded kH rows, the pad entries zero
__global__ void k_pair_coef(const double* __restrict__ Km, const double* __restrict__ Gm, int nx, int ny,
                            int nxp, double g2, float4* __restrict__ cLN, float2* __restrict__ cH)
{
    GF_FOR(t, static_cast<int64_t>(ny) * nxp)
    {
        const int ey = static_cast<int>(t / nxp), ex = static_cast<int>(t - static_cast<int64_t>(ey) * nxp);
        if (ex >= nx) {
            cH[t] = make_float2(0.f, 0.f);
            continue;
        }
        const int64_t e = static_cast<int64_t>(ey) * nx + ex;
        const double K = Km[e], G = Gm[e];
        const double lam = K - 2.0 * G / 3.0;
        const ffv L = ff_from_double(0.25 * lam), N = ff_from_double(0.25 * G);
        const ffv kH = ff_from_double(0.25 * g2 * (lam + 3.0 * G));
        cLN[e] = ppack(L, N);
        cH[t] = make_float2(kH.h, kH.l);
    }
}

static float2 split_host(double x)
{
    const float h = static_cast<float>(x);
    return make_float2(h, static_cast<float>(x - static_cast<double>(h)));
}

// the pair class coefficients of a descriptor's lumped-mass classes (those of k_verlet_node_cls)
static PairClassTab pair_class_tab(const gfgpu_verlet_desc* d)
{
    const double dt = d->dt, h = 0.5 * dt;
    PairClassTab tab{};
    for (int k = 0; k < d->ncls; ++k) {
        const double mi = d->mclass_inv[k], be = mi * d->eta, omh = 1.0 - h * be;
        tab.mi[k] = split_host(mi);
        tab.be[k] = split_host(be);
        tab.c1[k] = split_host(omh + h * h * be * be);
        tab.c2[k] = split_host(h * omh + h * h * be * be * dt);
        tab.c3[k] = split_host(h * omh);
    }
    return tab;
}


// The pair path applies to: uniform square Quad4 elements (coefficients), Mesh::Quad4::Regular
// numbering with plain dofs (verified on the device), lumped-mass classes.
static int pair_applicable(const gfgpu_verlet_desc* d, std::string* why)
{
    const char* w = nullptr;
    if (d->nne != 4 || d->ndim != 2) w = "Quad4 only";
    else if (!d->uniform) w = "uniform square elements only (gfgpu_verlet_detect_uniform)";
    else if (std::fabs(d->hx - d->hy) > 1e-12 * d->hx) w = "square elements only";
    else if (d->reg_nx <= 0 || d->reg_ny <= 0 || d->reg_nz != 0)
        w = "Mesh::Quad4::Regular numbering only (gfgpu_verlet_detect_regular)";
    else if (!d->mclass || !d->mclass_inv || d->ncls <= 0) w = "lumped-mass classes required (gfgpu_verlet_classify)";
    else if ((d->reg_nx + 1) * (d->reg_ny + 1) >= INT32_MAX / 2) w = "mesh too large";
    if (w && why) *why = w;
    return w ? GFGPU_ERR_UNSUPPORTED : GFGPU_OK;
}

// Which pair path a descriptor can take: 1 = the Regular square-element tile kernel
// (pair_applicable), 2 = element kernel + dof-CSR node kernel with the square closed form (uniform
// square Quad4 elements, any numbering, periodic ties allowed), 3 = the same with stored element
// stiffness matrices (any Quad4 mesh with the Gauss rule); 0 = none (why says why).
static int pair_mode_for(const gfgpu_verlet_desc* d, std::string* why)
{
    if (pair_applicable(d, why) == GFGPU_OK) return 1;
    if (d->nne != 4 || d->ndim != 2) {
        if (why) *why = "Quad4 only";
        return 0;
    }
    if (d->nelem * 8 >= INT32_MAX || d->nnode * 2 >= INT32_MAX) {
        if (why) *why = "mesh too large";
        return 0;
    }
    if (d->uniform && std::fabs(d->hx - d->hy) <= 1e-12 * d->hx) return 2;
    if (d->dNx && d->vol && d->nip == 4) return 3;
    if (why) *why = "needs the Gauss-rule dNx and vol of the mesh";
    return 0;
}

static bool pair_has_classes(const gfgpu_verlet_desc* d)
{
    return d->mclass && d->mclass_inv && d->ncls > 0;
}

} // namespace gfgpu

using namespace gfgpu;

int64_t gfgpu_internal_pair_workspace_bytes(const gfgpu_verlet_desc* d)
{
    if (!d || !d->coef_pair) return 0;
    const int64_t f4 = static_cast<int64_t>(sizeof(float4));
    if (d->pair_mode == 1) return (d->fext ? 5 : 4) * d->nnode * f4;
    // u, v, a (fext) pair nodevecs and the element forces [nelem * nne] of float4
    return (d->fext ? 4 : 3) * d->nnode * f4 + d->nelem * 4 * f4;
}

static int encode_map(CUtensorMap* map, const void* ptr, cuuint32_t rank, const cuuint64_t* dims,
                      const cuuint64_t* strides, const cuuint32_t* box)
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
    const cuuint32_t estr[3] = {1, 1, 1};
    // zero fill outside the tensor (CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE)
    CUresult rc = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank, const_cast<void*>(ptr), dims, strides, box,
                         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (rc != CUDA_SUCCESS) return fail(GFGPU_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(rc)) + ")");
    return GFGPU_OK;
}

// a pair nodevec [H][W] of float4 as a 3-d FP32 tensor {4, W, H}
static int nodevec_map(CUtensorMap* map, const float4* ptr, int W, int H, int bw, int bh)
{
    const cuuint64_t dims[3] = {4, static_cast<cuuint64_t>(W), static_cast<cuuint64_t>(H)};
    const cuuint64_t strides[2] = {16, 16ull * static_cast<cuuint64_t>(W)};
    const cuuint32_t box[3] = {4, static_cast<cuuint32_t>(bw), static_cast<cuuint32_t>(bh)};
    return encode_map(map, ptr, 3, dims, strides, box);
}

static int nxp_of(int64_t nx)
{
    return static_cast<int>(nx + (nx & 1));
}

template <int TY>
static int launch_tma(PairTmaStep p, const CUtensorMap* mu, const CUtensorMap& mv, const CUtensorMap& ma,
                      const CUtensorMap& ml, const CUtensorMap& mh, const PairClassTab& tab, int64_t first,
                      int64_t count, int advance_last, float4* const* ub, int sms, cudaStream_t s)
{
    using Gm = TmaGeom<TY>;
    static bool attr = false;
    if (!attr) {
        GF_TRY(check_cuda(cudaFuncSetAttribute(k_verlet_pair_tma<TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(Gm::Smem)),
                          "cudaFuncSetAttribute"));
        attr = true;
    }
    int per_sm = 0;
    GF_TRY(check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_verlet_pair_tma<TY>, Gm::threads,
                                                                    Gm::Smem),
                      "occupancy"));
    GF_REQUIRE(per_sm >= 1, "pair kernel does not fit on an SM");
    p.ntiles = p.ntx * ((p.ny + TY) / TY);
    const int grid = std::min(p.ntiles, sms * per_sm);
    p.gdx = grid % p.ntx;
    p.gdy = grid / p.ntx;
    for (int64_t it = first; it < first + count; ++it) {
        p.uout = ub[(it + 1) & 1];
        p.advance = (it + 1 < first + count || advance_last) ? 1 : 0;
        k_verlet_pair_tma<TY><<<grid, Gm::threads, Gm::Smem, s>>>(mu[it & 1], mv, ma, ml, mh, p, tab);
        GF_TRY(check_launch("verlet pair kernel (TMA)"));
    }
    return GFGPU_OK;
}

// The pair state of a descriptor in the workspace: the displacement double-buffered (increment
// `it` reads ub[it & 1] and writes the next displacement into ub[(it + 1) & 1]), v, a, fext.
struct PairState {
    float4 *ub[2], *v, *a, *fext;
};

static PairState pair_state(const gfgpu_verlet_desc* d, void* workspace)
{
    const int64_t nn = d->nnode;
    float4* base = static_cast<float4*>(workspace);
    if (d->pair_mode != 1) // one displacement buffer: the element and node phases are two kernels
        return PairState{{base, base}, base + nn, base + 2 * nn, d->fext ? base + 3 * nn : nullptr};
    return PairState{{base, base + nn}, base + 2 * nn, base + 3 * nn, d->fext ? base + 4 * nn : nullptr};
}

// element forces of the CSR pair path, after the state vectors
static float4* pair_fe(const gfgpu_verlet_desc* d, void* workspace)
{
    return static_cast<float4*>(workspace) + (d->fext ? 4 : 3) * d->nnode;
}

static int pair_check(const gfgpu_verlet_desc* d, const void* workspace)
{
    std::string why;
    const int mode = pair_mode_for(d, &why);
    if (mode == 0) return fail(GFGPU_ERR_UNSUPPORTED, "pair arithmetic: " + why);
    GF_REQUIRE(d->coef_pair, "pair arithmetic: d->coef_pair not set (gfgpu_verlet_precompute_pair)");
    GF_REQUIRE(d->pair_mode == mode, "pair arithmetic: the descriptor changed since gfgpu_verlet_precompute_pair");
    GF_REQUIRE(workspace && (reinterpret_cast<uintptr_t>(workspace) & 15u) == 0,
               "pair arithmetic: workspace missing or not 16-byte aligned");
    GF_REQUIRE(!d->fext || reinterpret_cast<uintptr_t>(d->fext) % 16 == 0, "fext must be 16-byte aligned");
    return GFGPU_OK;
}

static int pair_begin(const gfgpu_verlet_desc* d, const double* u, const double* v, const double* a,
                      void* workspace, cudaStream_t s)
{
    GF_REQUIRE(u && v && a, "bad argument");
    GF_REQUIRE((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(v) | reinterpret_cast<uintptr_t>(a)) % 16 == 0,
               "u, v, a must be 16-byte aligned");
    const PairState ps = pair_state(d, workspace);
    const double dt = d->dt, c = 0.5 * std::pow(dt, 2.0);
    k_pair_begin<<<grid_for(d->nnode), kBlock, 0, s>>>(reinterpret_cast<const double2*>(u), reinterpret_cast<const double2*>(v),
                                                       reinterpret_cast<const double2*>(a),
                                                       reinterpret_cast<const double2*>(d->fext), d->nnode, dt, c,
                                                       d->pair_mode == 1 ? 1 : 0, ps.ub[0], ps.v, ps.a, ps.fext);
    return check_launch("pair begin");
}

static int pair_increments(const gfgpu_verlet_desc* d, int64_t first, int64_t count, int advance_last,
                           void* workspace, cudaStream_t s)
{
    if (count <= 0) return GFGPU_OK;
    const PairState ps = pair_state(d, workspace);
    float4* const* ub = ps.ub;
    float4 *pv = ps.v, *pa = ps.a, *pfx = ps.fext;
    const double dt = d->dt, h = 0.5 * dt, c = 0.5 * std::pow(dt, 2.0);
    const PairClassTab tab = pair_class_tab(d);
    if (d->pair_mode != 1) {
        float4* fe = pair_fe(d, workspace);
        PairCsrStep q;
        q.reg_nx = (d->reg_nz == 0 && d->nne == 4) ? d->reg_nx : 0;
        q.reg_ny = d->reg_ny;
        q.ell = reinterpret_cast<const int4*>(d->ell);
        q.dofs = d->dofs;
        q.ptr = d->csr_ptr;
        q.idx = d->csr_idx;
        q.part = d->part;
        q.nnu = d->nnu;
        q.n = d->nnode * 2;
        const bool cls = pair_has_classes(d);
        q.mclass = cls ? d->mclass : nullptr;
        const int64_t ncoef = d->pair_mode == 2 ? 6 * d->nelem : 48 * d->nelem;
        q.minv = cls ? nullptr : reinterpret_cast<const float2*>(d->coef_pair + ncoef);
        q.fe = reinterpret_cast<const float2*>(fe);
        q.fext = reinterpret_cast<const float2*>(pfx);
        q.u = reinterpret_cast<float2*>(ub[0]);
        q.v = reinterpret_cast<float2*>(pv);
        q.a = reinterpret_cast<float2*>(pa);
        q.dt = split_host(dt);
        q.h = split_host(h);
        q.cc = split_host(c);
        q.eta = split_host(d->eta);
        for (int64_t it = first; it < first + count; ++it) {
            if (d->pair_mode == 2)
                k_pair_elem_square<<<grid_for(d->nelem), 256, 0, s>>>(
                    d->conn, ub[0], reinterpret_cast<const float4*>(d->coef_pair),
                    reinterpret_cast<const float2*>(d->coef_pair + 4 * d->nelem), d->nelem, fe);
            else
                k_pair_elem_stiff<<<grid_for(d->nelem, 128), 128, 0, s>>>(
                    d->conn, ub[0], reinterpret_cast<const float2*>(d->coef_pair), d->nelem, fe);
            GF_TRY(check_launch("pair element kernel"));
            q.advance = (it + 1 < first + count || advance_last) ? 1 : 0;
            k_pair_node_csr<<<grid_for(q.n), 256, 0, s>>>(q, tab);
            GF_TRY(check_launch("pair node kernel"));
        }
        return GFGPU_OK;
    }
    const int nx = static_cast<int>(d->reg_nx), ny = static_cast<int>(d->reg_ny), nxp = nxp_of(nx);
    const float4* cLN = reinterpret_cast<const float4*>(d->coef_pair);
    const float2* cH = reinterpret_cast<const float2*>(d->coef_pair + 4 * d->nelem);
    const uchar2* mcls = reinterpret_cast<const uchar2*>(d->mclass);
    if (pair_kernel() == 1) {
        PairStep p;
        p.v = pv;
        p.a = pa;
        p.fext = pfx;
        p.cLN = cLN;
        p.cH = cH;
        p.mcls = mcls;
        p.nx = nx;
        p.ny = ny;
        p.nxp = nxp;
        p.dt = split_host(dt);
        p.cc = split_host(c);
        const dim3 grid(static_cast<unsigned>((nx + kPairTX) / kPairTX), static_cast<unsigned>((ny + kPairTY) / kPairTY));
        for (int64_t it = first; it < first + count; ++it) {
            p.uin = ub[it & 1];
            p.uout = ub[(it + 1) & 1];
            p.advance = (it + 1 < first + count || advance_last) ? 1 : 0;
            k_verlet_pair_quad4<<<grid, kPairThreads, 0, s>>>(p, tab);
            GF_TRY(check_launch("verlet pair kernel"));
        }
        return GFGPU_OK;
    }
    CUtensorMap mu[2], mv, ma, ml, mh;
    const int TY = pair_kernel() == 2 ? 15 : 7;
    GF_TRY(nodevec_map(&mu[0], ub[0], nx + 1, ny + 1, kTmaTX + 2, TY + 2));
    GF_TRY(nodevec_map(&mu[1], ub[1], nx + 1, ny + 1, kTmaTX + 2, TY + 2));
    GF_TRY(nodevec_map(&mv, pv, nx + 1, ny + 1, kTmaTX, TY));
    GF_TRY(nodevec_map(&ma, pa, nx + 1, ny + 1, kTmaTX, TY));
    GF_TRY(nodevec_map(&ml, cLN, nx, ny, kTmaTX + 1, TY + 1));
    {
        const cuuint64_t dims[2] = {2ull * static_cast<cuuint64_t>(nxp), static_cast<cuuint64_t>(ny)};
        const cuuint64_t strides[1] = {8ull * static_cast<cuuint64_t>(nxp)};
        const cuuint32_t box[2] = {static_cast<cuuint32_t>(TmaGeom<7>::HW), static_cast<cuuint32_t>(TY + 1)};
        GF_TRY(encode_map(&mh, cH, 2, dims, strides, box));
    }
    int dev = 0, sms = 0;
    GF_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
    GF_TRY(check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr"));
    PairTmaStep p;
    p.v = pv;
    p.a = pa;
    p.fext = pfx;
    p.mcls = mcls;
    p.nx = nx;
    p.ny = ny;
    p.ntx = (nx + kTmaTX) / kTmaTX;
    p.dt = split_host(dt);
    p.cc = split_host(c);
    p.nz = kF2NegZero;
    if (TY == 15) return launch_tma<15>(p, mu, mv, ma, ml, mh, tab, first, count, advance_last, ub, sms, s);
    return launch_tma<7>(p, mu, mv, ma, ml, mh, tab, first, count, advance_last, ub, sms, s);
}

static int pair_end(const gfgpu_verlet_desc* d, int64_t last, double* u, double* v, double* a, void* workspace,
                    cudaStream_t s)
{
    GF_REQUIRE(u && v && a && last >= 0, "bad argument");
    const PairState ps = pair_state(d, workspace);
    k_pair_end<<<grid_for(d->nnode), kBlock, 0, s>>>(ps.ub[last & 1], ps.v, ps.a, d->nnode, d->pair_mode == 1 ? 1 : 0,
                                                     reinterpret_cast<double2*>(u),
                                                     reinterpret_cast<double2*>(v), reinterpret_cast<double2*>(a));
    return check_launch("pair end");
}

// gfgpu_verlet_step's pair path (d->coef_pair set, fast arithmetic)
int gfgpu_internal_verlet_pair(const gfgpu_verlet_desc* d, double* u, double* v, double* a,
                               int64_t nsteps, void* workspace, cudaStream_t s)
{
    GF_TRY(pair_check(d, workspace));
    GF_TRY(pair_begin(d, u, v, a, workspace, s));
    GF_TRY(pair_increments(d, 0, nsteps, 0, workspace, s));
    // the last increment does not advance: its displacement is the one it read
    return pair_end(d, nsteps - 1, u, v, a, workspace, s);
}

// Element forces of a uniform square Quad4 mesh in pair arithmetic, FP64 in and out (the static
// solvers' iterations, pcg.cu / learned.cu, and the explicit step in mixed arithmetic, dynamics.cu):
// coef = d->pcg_pair as written by gfgpu_internal_pair_coef_square.
int gfgpu_internal_pair_element_forces_f64(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                           cudaStream_t s)
{
    if (d->nelem == 0) return GFGPU_OK;
    const float* c = d->pcg_pair;
    k_pair_elem_square_f64<false><<<grid_for(d->nelem), 256, 0, s>>>(
        d->conn, reinterpret_cast<const double2*>(u), reinterpret_cast<const float4*>(c),
        reinterpret_cast<const float2*>(c + 4 * d->nelem), d->nelem, reinterpret_cast<double2*>(fe));
    return check_launch("pair element kernel (static operator)");
}

// One increment of mixed arithmetic after the FP64 predictor (dynamics.cu): the pair element
// forces into fe (8 bytes per value) and the mixed node kernel; needs lumped-mass classes.
int gfgpu_internal_mixed_increment(const gfgpu_verlet_desc* d, double* fe, int advance, double* u, double* v,
                                   double* a, cudaStream_t s)
{
    const float* c = d->pcg_pair;
    k_pair_elem_square_f64<true><<<grid_for(d->nelem), 256, 0, s>>>(
        d->conn, reinterpret_cast<const double2*>(u), reinterpret_cast<const float4*>(c),
        reinterpret_cast<const float2*>(c + 4 * d->nelem), d->nelem, reinterpret_cast<double2*>(fe));
    GF_TRY(check_launch("pair element kernel (mixed)"));
    MixedNodeStep q;
    q.dofs = d->dofs;
    q.ptr = d->csr_ptr;
    q.idx = d->csr_idx;
    q.mclass = d->mclass;
    q.fe = reinterpret_cast<const float2*>(fe);
    q.fext = d->fext;
    q.u = u;
    q.v = v;
    q.a = a;
    q.n = d->nnode * d->ndim;
    q.reg_nx = (d->reg_nz == 0 && d->nne == 4) ? d->reg_nx : 0;
    q.reg_ny = d->reg_ny;
    q.ell = reinterpret_cast<const int4*>(d->ell);
    q.dt = d->dt;
    q.h = 0.5 * d->dt;
    q.c = 0.5 * std::pow(d->dt, 2.0);
    q.advance = advance;
    k_mixed_node<<<grid_for(q.n), 256, 0, s>>>(q, pair_class_tab(d));
    return check_launch("mixed node kernel");
}

// {L, N} [nelem] interleaved pairs, then kH [nelem] (6 floats per element) of a uniform square Quad4
// mesh, the layout k_pair_elem_square_f64 reads
int gfgpu_internal_pair_coef_square(const gfgpu_verlet_desc* d, float* coef, cudaStream_t s)
{
    if (d->nelem == 0) return GFGPU_OK;
    const double g = 1.0 / std::sqrt(3.0);
    k_pair_coef_elem<<<grid_for(d->nelem), kBlock, 0, s>>>(d->K, d->G, d->nelem, g * g,
                                                           reinterpret_cast<float4*>(coef),
                                                           reinterpret_cast<float2*>(coef + 4 * d->nelem));
    return check_launch("pair coefficients (static operator)");
}

extern "C" {

int gfgpu_verlet_pair_begin(const gfgpu_verlet_desc* d, const double* u, const double* v, const double* a,
                            void* workspace, gfgpu_stream_t stream)
{
    GF_REQUIRE(d, "null descriptor");
    GF_TRY(pair_check(d, workspace));
    return pair_begin(d, u, v, a, workspace, S(stream));
}

int gfgpu_verlet_pair_increments(const gfgpu_verlet_desc* d, int64_t first, int64_t count, int32_t advance_last,
                                 void* workspace, gfgpu_stream_t stream)
{
    GF_REQUIRE(d && first >= 0 && count >= 0, "bad argument");
    GF_TRY(pair_check(d, workspace));
    return pair_increments(d, first, count, advance_last ? 1 : 0, workspace, S(stream));
}

int gfgpu_verlet_pair_end(const gfgpu_verlet_desc* d, int64_t last, double* u, double* v, double* a,
                          void* workspace, gfgpu_stream_t stream)
{
    GF_REQUIRE(d, "null descriptor");
    GF_TRY(pair_check(d, workspace));
    return pair_end(d, last, u, v, a, workspace, S(stream));
}

int gfgpu_verlet_pair_displacement(const gfgpu_verlet_desc* d, int64_t it, void* workspace, void** ptr)
{
    GF_REQUIRE(d && ptr && it >= 0, "bad argument");
    GF_TRY(pair_check(d, workspace));
    *ptr = pair_state(d, workspace).ub[it & 1];
    return GFGPU_OK;
}

int gfgpu_pairs_from_f64(const double* x, int64_t n, float* out, gfgpu_stream_t stream)
{
    GF_REQUIRE(n >= 0 && (n == 0 || (x && out)), "bad argument");
    GF_REQUIRE(reinterpret_cast<uintptr_t>(out) % 8 == 0, "out must be 8-byte aligned");
    if (n == 0) return GFGPU_OK;
    k_pair_split<<<grid_for(n), kBlock, 0, S(stream)>>>(x, n, reinterpret_cast<float2*>(out));
    return check_launch("pairs_from_f64");
}

int gfgpu_pairs_to_f64(const float* in, int64_t n, double* out, gfgpu_stream_t stream)
{
    GF_REQUIRE(n >= 0 && (n == 0 || (in && out)), "bad argument");
    GF_REQUIRE(reinterpret_cast<uintptr_t>(in) % 8 == 0, "in must be 8-byte aligned");
    if (n == 0) return GFGPU_OK;
    k_pair_join<<<grid_for(n), kBlock, 0, S(stream)>>>(reinterpret_cast<const float2*>(in), n, out);
    return check_launch("pairs_to_f64");
}

int64_t gfgpu_verlet_pair_coef_floats(const gfgpu_verlet_desc* d)
{
    if (!d) return 0;
    const int mode = pair_mode_for(d, nullptr);
    if (mode == 1) return 4 * d->reg_nx * d->reg_ny + 2 * static_cast<int64_t>(nxp_of(d->reg_nx)) * d->reg_ny;
    if (mode == 0) return 0;
    const int64_t minv = pair_has_classes(d) ? 0 : 2 * d->nnu;
    return (mode == 2 ? 6 : 48) * d->nelem + minv;
}

int gfgpu_verlet_precompute_pair(gfgpu_verlet_desc* d, float* coef_pair, gfgpu_stream_t stream)
{
    GF_REQUIRE(d && coef_pair, "bad argument");
    GF_REQUIRE((reinterpret_cast<uintptr_t>(coef_pair) & 15u) == 0, "coef_pair must be 16-byte aligned");
    std::string why;
    const int mode = pair_mode_for(d, &why);
    if (mode == 0) return fail(GFGPU_ERR_UNSUPPORTED, "gfgpu_verlet_precompute_pair: " + why);
    GF_REQUIRE(d->K && d->G, "null material");
    d->pair_mode = mode;
    if (d->nelem == 0) return GFGPU_OK;
    cudaStream_t s = S(stream);
    const double g = 1.0 / std::sqrt(3.0);
    if (mode == 1) {
        const int nx = static_cast<int>(d->reg_nx), ny = static_cast<int>(d->reg_ny), nxp = nxp_of(nx);
        float4* cLN = reinterpret_cast<float4*>(coef_pair);
        float2* cH = reinterpret_cast<float2*>(coef_pair + 4 * d->nelem);
        k_pair_coef<<<grid_for(static_cast<int64_t>(ny) * nxp), kBlock, 0, s>>>(d->K, d->G, nx, ny, nxp, g * g, cLN,
                                                                              cH);
        return check_launch("verlet_precompute_pair");
    }
    if (mode == 2)
        k_pair_coef_elem<<<grid_for(d->nelem), kBlock, 0, s>>>(d->K, d->G, d->nelem, g * g,
                                                               reinterpret_cast<float4*>(coef_pair),
                                                               reinterpret_cast<float2*>(coef_pair + 4 * d->nelem));
    else
        k_pair_stiffness<<<grid_for(d->nelem, 128), 128, 0, s>>>(d->dNx, d->vol, d->K, d->G, d->nelem, d->nip,
                                                                 reinterpret_cast<float2*>(coef_pair));
    GF_TRY(check_launch("verlet_precompute_pair"));
    if (!pair_has_classes(d) && d->nnu > 0) {
        GF_REQUIRE(d->inv, "null inverse mass");
        const int64_t ncoef = (mode == 2 ? 6 : 48) * d->nelem;
        k_pair_split<<<grid_for(d->nnu), kBlock, 0, s>>>(d->inv, d->nnu, reinterpret_cast<float2*>(coef_pair + ncoef));
        GF_TRY(check_launch("verlet_precompute_pair (inverse mass)"));
    }
    return GFGPU_OK;
}

int gfgpu_verlet_pair_status(void)
{
    int flag = 0;
    GF_TRY(check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize"));
    GF_TRY(check_cuda(cudaMemcpyFromSymbol(&flag, g_pair_timeout, sizeof(int)), "cudaMemcpyFromSymbol"));
    if (flag) {
        const int zero = 0;
        GF_TRY(check_cuda(cudaMemcpyToSymbol(g_pair_timeout, &zero, sizeof(int)), "cudaMemcpyToSymbol"));
        return fail(GFGPU_ERR_TIMEOUT, "gfgpu_verlet_pair_status: a pair kernel's wait for its TMA copies gave up");
    }
    return GFGPU_OK;
}

} // extern "C"
