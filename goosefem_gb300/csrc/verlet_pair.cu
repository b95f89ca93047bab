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
#include <cmath>

#include "common.cuh"
#include "ffpair.cuh"

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
    const float2* cH;    // [nelem] {kH.h, kH.l}
    const uchar2* mcls;  // [nnode] lumped-mass class per component
    int nx, ny;
    int advance;         // write uout
    float2 dt, cc;       // dt and dt^2 / 2 as pairs
};

__device__ __forceinline__ ffv lo2(float4 q) { return ff_make(q.x, q.y); }
__device__ __forceinline__ ffv hi2(float4 q) { return ff_make(q.z, q.w); }
__device__ __forceinline__ ffv pf(float2 q) { return ff_make(q.x, q.y); }
__device__ __forceinline__ float4 pack(ffv x, ffv y) { return make_float4(x.h, x.l, y.h, y.l); }

// element (ex, ey) of a square-element Regular mesh with per-element L = lam/4, N = G/4 (M = 2N)
// and kH = g^2 (lam + 3G)/4: the sums S = P0 + P1, D = P0 - P1 (x) and P1 + Q1, P1 - Q1 (y) and
// the hourglass terms H, from which the element forces are (H - S, D - H, S + H, -(D + H)) at
// nodes 0..3 (k_elem_force_quad4_square's formulas, every sum and product on pairs)
__device__ __forceinline__ void pair_element(float4 q0, float4 q1, float4 q2, float4 q3, float4 cln,
                                             float2 ch, float4& S, float4& D, float4& H)
{
    const ffv u0x = lo2(q0), u0y = hi2(q0), u1x = lo2(q1), u1y = hi2(q1);
    const ffv u2x = lo2(q2), u2y = hi2(q2), u3x = lo2(q3), u3y = hi2(q3);
    const ffv px = ff_sub(u2x, u0x), qx = ff_sub(u1x, u3x);
    const ffv py = ff_sub(u2y, u0y), qy = ff_sub(u1y, u3y);
    const ffv A1x = ff_add(px, qx), A2x = ff_sub(px, qx);
    const ffv A1y = ff_add(py, qy), A2y = ff_sub(py, qy);
    const ffv A3x = ff_sub(ff_add(u0x, u2x), ff_add(u1x, u3x));
    const ffv A3y = ff_sub(ff_add(u0y, u2y), ff_add(u1y, u3y));
    const ffv L = lo2(cln), N = hi2(cln), kH = pf(ch);
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
            pair_element(su[b], su[b + 1], su[b + UW + 1], su[b + UW], __ldg(p.cLN + e), __ldg(p.cH + e), S, D, H);
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
    pair_update(cl.x, fxn, lo2(fq), hf, lo2(vq), lo2(aq), smi, sbe, sc1, sc2, sc3, dt, vx, ax);
    pair_update(cl.y, fyn, hi2(fq), hf, hi2(vq), hi2(aq), smi, sbe, sc1, sc2, sc3, dt, vy, ay);
    p.v[node] = pack(vx, vy);
    p.a[node] = pack(ax, ay);
    if (p.advance) {
        const float4 uq = su[(ty + 1) * UW + tx + 1];
        const ffv cc = pf(p.cc);
        const ffv ux = ff_norm(ff_add(ff_add(lo2(uq), ff_mul(dt, vx)), ff_mul(cc, ax)));
        const ffv uy = ff_norm(ff_add(ff_add(hi2(uq), ff_mul(dt, vy)), ff_mul(cc, ay)));
        p.uout[node] = pack(ux, uy);
    }
}

// FP64 in: the predictor u + dt v + dt^2/2 a of the first increment (FP64, as k_predict), then
// u, v, a (and fext) as pairs
__global__ void k_pair_begin(const double2* __restrict__ u, const double2* __restrict__ v,
                             const double2* __restrict__ a, const double2* __restrict__ fext,
                             int64_t nnode, double dt, double c, float4* __restrict__ pu,
                             float4* __restrict__ pv, float4* __restrict__ pa, float4* __restrict__ pf_)
{
    GF_FOR(n, nnode)
    {
        const double2 un = u[n], vn = v[n], an = a[n];
        const double ux = fma(c, an.x, fma(dt, vn.x, un.x)), uy = fma(c, an.y, fma(dt, vn.y, un.y));
        pu[n] = pack(ff_from_double(ux), ff_from_double(uy));
        pv[n] = pack(ff_from_double(vn.x), ff_from_double(vn.y));
        pa[n] = pack(ff_from_double(an.x), ff_from_double(an.y));
        if (fext) {
            const double2 fn = fext[n];
            pf_[n] = pack(ff_from_double(fn.x), ff_from_double(fn.y));
        }
    }
}

__global__ void k_pair_end(const float4* __restrict__ pu, const float4* __restrict__ pv,
                           const float4* __restrict__ pa, int64_t nnode, double2* __restrict__ u,
                           double2* __restrict__ v, double2* __restrict__ a)
{
    GF_FOR(n, nnode)
    {
        const float4 qu = pu[n], qv = pv[n], qa = pa[n];
        u[n] = make_double2(ff_to_double(lo2(qu)), ff_to_double(hi2(qu)));
        v[n] = make_double2(ff_to_double(lo2(qv)), ff_to_double(hi2(qv)));
        a[n] = make_double2(ff_to_double(lo2(qa)), ff_to_double(hi2(qa)));
    }
}

// per-element pair coefficients: cLN[e] = {L, N}, cH[e] = kH (see pair_element)
__global__ void k_pair_coef(const double* __restrict__ Km, const double* __restrict__ Gm, int64_t nelem,
                            double g2, float4* __restrict__ cLN, float2* __restrict__ cH)
{
    GF_FOR(e, nelem)
    {
        const double K = Km[e], G = Gm[e];
        const double lam = K - 2.0 * G / 3.0;
        const ffv L = ff_from_double(0.25 * lam), N = ff_from_double(0.25 * G);
        const ffv kH = ff_from_double(0.25 * g2 * (lam + 3.0 * G));
        cLN[e] = pack(L, N);
        cH[e] = make_float2(kH.h, kH.l);
    }
}

static float2 split_host(double x)
{
    const float h = static_cast<float>(x);
    return make_float2(h, static_cast<float>(x - static_cast<double>(h)));
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

} // namespace gfgpu

using namespace gfgpu;

int64_t gfgpu_internal_pair_workspace_bytes(const gfgpu_verlet_desc* d)
{
    if (!d || !d->coef_pair) return 0;
    const int64_t vecs = d->fext ? 5 : 4;
    return vecs * d->nnode * static_cast<int64_t>(sizeof(float4));
}

// gfgpu_verlet_step's pair path (d->coef_pair set, fast arithmetic)
int gfgpu_internal_verlet_pair(const gfgpu_verlet_desc* d, double* u, double* v, double* a,
                               int64_t nsteps, void* workspace, cudaStream_t s)
{
    std::string why;
    if (pair_applicable(d, &why) != GFGPU_OK)
        return fail(GFGPU_ERR_UNSUPPORTED, "gfgpu_verlet_step (pair arithmetic): " + why);
    GF_REQUIRE((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(v) | reinterpret_cast<uintptr_t>(a)) % 16 == 0,
               "u, v, a must be 16-byte aligned");
    GF_REQUIRE(!d->fext || reinterpret_cast<uintptr_t>(d->fext) % 16 == 0, "fext must be 16-byte aligned");
    const int64_t nn = d->nnode;
    float4* base = static_cast<float4*>(workspace);
    float4* ub[2] = {base, base + nn};
    float4* pv = base + 2 * nn;
    float4* pa = base + 3 * nn;
    float4* pfx = d->fext ? base + 4 * nn : nullptr;
    const double dt = d->dt, h = 0.5 * dt, c = 0.5 * std::pow(dt, 2.0);
    PairClassTab tab{};
    for (int k = 0; k < d->ncls; ++k) {
        // the coefficients of k_verlet_node_cls (MassClassTab), as pairs
        const double mi = d->mclass_inv[k], be = mi * d->eta, omh = 1.0 - h * be;
        tab.mi[k] = split_host(mi);
        tab.be[k] = split_host(be);
        tab.c1[k] = split_host(omh + h * h * be * be);
        tab.c2[k] = split_host(h * omh + h * h * be * be * dt);
        tab.c3[k] = split_host(h * omh);
    }
    k_pair_begin<<<grid_for(nn), kBlock, 0, s>>>(reinterpret_cast<const double2*>(u), reinterpret_cast<const double2*>(v),
                                                 reinterpret_cast<const double2*>(a),
                                                 reinterpret_cast<const double2*>(d->fext), nn, dt, c, ub[0], pv,
                                                 pa, pfx);
    GF_TRY(check_launch("pair begin"));
    PairStep p;
    p.v = pv;
    p.a = pa;
    p.fext = pfx;
    p.cLN = reinterpret_cast<const float4*>(d->coef_pair);
    p.cH = reinterpret_cast<const float2*>(d->coef_pair + 4 * d->nelem);
    p.mcls = reinterpret_cast<const uchar2*>(d->mclass);
    p.nx = static_cast<int>(d->reg_nx);
    p.ny = static_cast<int>(d->reg_ny);
    p.dt = split_host(dt);
    p.cc = split_host(c);
    const dim3 grid(static_cast<unsigned>((d->reg_nx + kPairTX) / kPairTX),
                    static_cast<unsigned>((d->reg_ny + kPairTY) / kPairTY));
    for (int64_t it = 0; it < nsteps; ++it) {
        p.uin = ub[it & 1];
        p.uout = ub[(it + 1) & 1];
        p.advance = it + 1 < nsteps ? 1 : 0;
        k_verlet_pair_quad4<<<grid, kPairThreads, 0, s>>>(p, tab);
        GF_TRY(check_launch("verlet pair kernel"));
    }
    // the last increment does not advance: its displacement is the one it read
    k_pair_end<<<grid_for(nn), kBlock, 0, s>>>(ub[(nsteps - 1) & 1], pv, pa, nn, reinterpret_cast<double2*>(u),
                                               reinterpret_cast<double2*>(v), reinterpret_cast<double2*>(a));
    return check_launch("pair end");
}

extern "C" {

int gfgpu_verlet_precompute_pair(const gfgpu_verlet_desc* d, float* coef_pair, gfgpu_stream_t stream)
{
    GF_REQUIRE(d && coef_pair, "bad argument");
    GF_REQUIRE((reinterpret_cast<uintptr_t>(coef_pair) & 15u) == 0, "coef_pair must be 16-byte aligned");
    std::string why;
    if (pair_applicable(d, &why) != GFGPU_OK) return fail(GFGPU_ERR_UNSUPPORTED, "gfgpu_verlet_precompute_pair: " + why);
    GF_REQUIRE(d->K && d->G, "null material");
    if (d->nelem == 0) return GFGPU_OK;
    const double g = 1.0 / std::sqrt(3.0);
    float4* cLN = reinterpret_cast<float4*>(coef_pair);
    float2* cH = reinterpret_cast<float2*>(coef_pair + 4 * d->nelem);
    k_pair_coef<<<grid_for(d->nelem), kBlock, 0, S(stream)>>>(d->K, d->G, d->nelem, g * g, cLN, cH);
    return check_launch("verlet_precompute_pair");
}

} // extern "C"
