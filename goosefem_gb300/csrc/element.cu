// Element quadrature kernels: Quadrature set-up (shape functions, compute_dN) and the
// element-by-element operators of GooseFEM's QuadratureBaseCartesian, for Quad4 (nne=4, ndim=2)
// and Hex8 (nne=8, ndim=3). One thread per (element, integration point) for point-wise
// operators, one thread per element for the integrals that sum over the integration points, so
// every output entry is summed in the reference's order.
#include "common.cuh"

namespace gfgpu {

// ---------------------------------------------------------------- loads

template <int N>
__device__ __forceinline__ void load(const double* __restrict__ p, double (&o)[N])
{
    if constexpr (N % 2 == 0) {
        const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
        for (int k = 0; k < N / 2; ++k) {
            double2 v = __ldg(q + k);
            o[2 * k] = v.x;
            o[2 * k + 1] = v.y;
        }
    }
    else {
#pragma unroll
        for (int k = 0; k < N; ++k) o[k] = __ldg(p + k);
    }
}

template <int N>
__device__ __forceinline__ void store(double* __restrict__ p, const double (&o)[N])
{
#pragma unroll
    for (int k = 0; k < N; ++k) p[k] = o[k];
}

// ---------------------------------------------------------------- shape functions

// ElementQuad4.h:277-300 (N and dN/dxi), evaluated with the reference's operation order.
__device__ __forceinline__ void quad4_shape(double x0, double x1, double* N, double* dn)
{
    double a0 = __dsub_rn(1.0, x0), b0 = __dadd_rn(1.0, x0);
    double a1 = __dsub_rn(1.0, x1), b1 = __dadd_rn(1.0, x1);
    if (N) {
        N[0] = __dmul_rn(__dmul_rn(0.25, a0), a1);
        N[1] = __dmul_rn(__dmul_rn(0.25, b0), a1);
        N[2] = __dmul_rn(__dmul_rn(0.25, b0), b1);
        N[3] = __dmul_rn(__dmul_rn(0.25, a0), b1);
    }
    dn[0 * 2 + 0] = __dmul_rn(-0.25, a1);
    dn[1 * 2 + 0] = __dmul_rn(+0.25, a1);
    dn[2 * 2 + 0] = __dmul_rn(+0.25, b1);
    dn[3 * 2 + 0] = __dmul_rn(-0.25, b1);
    dn[0 * 2 + 1] = __dmul_rn(-0.25, a0);
    dn[1 * 2 + 1] = __dmul_rn(-0.25, b0);
    dn[2 * 2 + 1] = __dmul_rn(+0.25, b0);
    dn[3 * 2 + 1] = __dmul_rn(+0.25, a0);
}

// ElementHex8.h:255-295.
__device__ __forceinline__ void hex8_shape(double x0, double x1, double x2, double* N, double* dn)
{
    const int sx[8] = {-1, +1, +1, -1, -1, +1, +1, -1};
    const int sy[8] = {-1, -1, +1, +1, -1, -1, +1, +1};
    const int sz[8] = {-1, -1, -1, -1, +1, +1, +1, +1};
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        double fa = sx[m] < 0 ? __dsub_rn(1.0, x0) : __dadd_rn(1.0, x0);
        double fb = sy[m] < 0 ? __dsub_rn(1.0, x1) : __dadd_rn(1.0, x1);
        double fc = sz[m] < 0 ? __dsub_rn(1.0, x2) : __dadd_rn(1.0, x2);
        if (N) N[m] = __dmul_rn(__dmul_rn(__dmul_rn(0.125, fa), fb), fc);
        dn[m * 3 + 0] = __dmul_rn(__dmul_rn(sx[m] < 0 ? -0.125 : 0.125, fb), fc);
        dn[m * 3 + 1] = __dmul_rn(__dmul_rn(sy[m] < 0 ? -0.125 : 0.125, fa), fc);
        dn[m * 3 + 2] = __dmul_rn(__dmul_rn(sz[m] < 0 ? -0.125 : 0.125, fa), fb);
    }
}

__global__ void k_shape(const double* xi, int nip, int nd, double* N, double* dNxi)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nip) return;
    if (nd == 2) {
        double n[4], d[8];
        quad4_shape(xi[q * 2], xi[q * 2 + 1], n, d);
        if (N)
            for (int k = 0; k < 4; ++k) N[q * 4 + k] = n[k];
        if (dNxi)
            for (int k = 0; k < 8; ++k) dNxi[q * 8 + k] = d[k];
    }
    else {
        double n[8], d[24];
        hex8_shape(xi[q * 3], xi[q * 3 + 1], xi[q * 3 + 2], n, d);
        if (N)
            for (int k = 0; k < 8; ++k) N[q * 8 + k] = n[k];
        if (dNxi)
            for (int k = 0; k < 24; ++k) dNxi[q * 24 + k] = d[k];
    }
}

// ElementQuad4.h:493-532 + detail.h:26-36. Strict arithmetic: dNx and vol are bit-exact.
// QuadraturePlanar (ElementQuad4Planar.h:280-318) is the same with vol = w * det(J) * thick; for
// plain Quad4 thick = 1 (an exact product, so the bits are unchanged).
__global__ void k_quad4_compute_dN(const double* __restrict__ x, int64_t nelem,
                                   const double* __restrict__ xi, const double* __restrict__ w,
                                   int nip, double thick, double* __restrict__ dNx,
                                   double* __restrict__ vol)
{
    GF_FOR(t, nelem * nip)
    {
        int64_t e = t / nip;
        int q = static_cast<int>(t - e * nip);
        double dn[8];
        quad4_shape(xi[q * 2], xi[q * 2 + 1], nullptr, dn);
        double xe[8];
        load<8>(x + e * 8, xe);
        double J[2][2];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j)
                J[i][j] = __dadd_rn(
                    __dadd_rn(__dadd_rn(__dmul_rn(dn[0 + i], xe[0 + j]), __dmul_rn(dn[2 + i], xe[2 + j])),
                              __dmul_rn(dn[4 + i], xe[4 + j])),
                    __dmul_rn(dn[6 + i], xe[6 + j]));
        double det = __dsub_rn(__dmul_rn(J[0][0], J[1][1]), __dmul_rn(J[0][1], J[1][0]));
        double i00 = __ddiv_rn(J[1][1], det);
        double i01 = __ddiv_rn(__dmul_rn(-1.0, J[0][1]), det);
        double i10 = __ddiv_rn(__dmul_rn(-1.0, J[1][0]), det);
        double i11 = __ddiv_rn(J[0][0], det);
        double o[8];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            o[m * 2 + 0] = __dadd_rn(__dmul_rn(i00, dn[m * 2 + 0]), __dmul_rn(i01, dn[m * 2 + 1]));
            o[m * 2 + 1] = __dadd_rn(__dmul_rn(i10, dn[m * 2 + 0]), __dmul_rn(i11, dn[m * 2 + 1]));
        }
        store<8>(dNx + t * 8, o);
        vol[t] = __dmul_rn(__dmul_rn(w[q], det), thick);
    }
}

// Element.h:1178-1229 (generic, used by Hex8) + detail.h:49-69, restated as written
// (including dNx(m,i) += Jinv(i,j) * dNxi(m,i), Element.h:1220). Strict arithmetic.
__global__ void k_hex8_compute_dN(const double* __restrict__ x, int64_t nelem,
                                  const double* __restrict__ xi, const double* __restrict__ w,
                                  int nip, double* __restrict__ dNx, double* __restrict__ vol)
{
    GF_FOR(t, nelem * nip)
    {
        int64_t e = t / nip;
        int q = static_cast<int>(t - e * nip);
        double dn[24];
        hex8_shape(xi[q * 3], xi[q * 3 + 1], xi[q * 3 + 2], nullptr, dn);
        double xe[24];
        load<24>(x + e * 24, xe);
        double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
        for (int m = 0; m < 8; ++m)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    A[i][j] = __dadd_rn(A[i][j], __dmul_rn(dn[m * 3 + i], xe[m * 3 + j]));
        auto M3 = [](double a, double b, double c) { return __dmul_rn(__dmul_rn(a, b), c); };
        double det = __dsub_rn(
            __dadd_rn(__dadd_rn(M3(A[0][0], A[1][1], A[2][2]), M3(A[0][1], A[1][2], A[2][0])),
                      M3(A[0][2], A[1][0], A[2][1])),
            __dadd_rn(__dadd_rn(M3(A[0][2], A[1][1], A[2][0]), M3(A[0][1], A[1][0], A[2][2])),
                      M3(A[0][0], A[1][2], A[2][1])));
        auto D = [](double a, double b, double c, double d) {
            return __dsub_rn(__dmul_rn(a, b), __dmul_rn(c, d));
        };
        double B[3][3];
        B[0][0] = __ddiv_rn(D(A[1][1], A[2][2], A[1][2], A[2][1]), det);
        B[0][1] = __ddiv_rn(D(A[0][2], A[2][1], A[0][1], A[2][2]), det);
        B[0][2] = __ddiv_rn(D(A[0][1], A[1][2], A[0][2], A[1][1]), det);
        B[1][0] = __ddiv_rn(D(A[1][2], A[2][0], A[1][0], A[2][2]), det);
        B[1][1] = __ddiv_rn(D(A[0][0], A[2][2], A[0][2], A[2][0]), det);
        B[1][2] = __ddiv_rn(D(A[0][2], A[1][0], A[0][0], A[1][2]), det);
        B[2][0] = __ddiv_rn(D(A[1][0], A[2][1], A[1][1], A[2][0]), det);
        B[2][1] = __ddiv_rn(D(A[0][1], A[2][0], A[0][0], A[2][1]), det);
        B[2][2] = __ddiv_rn(D(A[0][0], A[1][1], A[0][1], A[1][0]), det);
        double* o = dNx + t * 24;
#pragma unroll
        for (int m = 0; m < 8; ++m)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                double acc = 0.0;
#pragma unroll
                for (int j = 0; j < 3; ++j) acc = __dadd_rn(acc, __dmul_rn(B[i][j], dn[m * 3 + i]));
                o[m * 3 + i] = acc;
            }
        vol[t] = __dmul_rn(w[q], det);
    }
}

// ---------------------------------------------------------------- point-wise operators

template <bool S>
__device__ __forceinline__ double dot4(const double* a, int sa, const double* b, int sb)
{
    // ((a0 b0 + a1 b1) + a2 b2) + a3 b3, the reference's left-to-right sum
    double r = mul<S>(a[0], b[0]);
    r = madd<S>(a[sa], b[sb], r);
    r = madd<S>(a[2 * sa], b[2 * sb], r);
    r = madd<S>(a[3 * sa], b[3 * sb], r);
    return r;
}

// mode 0: GradN_vector, 1: GradN_vector_T, 2: SymGradN_vector. TD: tensor dimension of the
// output (TD = 3 with ND = 2: QuadraturePlanar, ElementQuad4Planar.h:130-221, the in-plane block
// of a zero-filled 3x3 tensor).
template <bool S, int NNE, int ND, int MODE, int TD = ND>
__global__ void k_grad(const double* __restrict__ dNx, const double* __restrict__ elemvec,
                       int64_t nelem, int nip, double* __restrict__ qtensor)
{
    GF_FOR(t, nelem * nip)
    {
        int64_t e = t / nip;
        double g[NNE * ND], u[NNE * ND];
        load<NNE * ND>(dNx + t * NNE * ND, g);
        load<NNE * ND>(elemvec + e * NNE * ND, u);
        double o[ND * ND];
        if constexpr (NNE == 4 && ND == 2) {
            // ElementQuad4.h:349-434 (hand-unrolled overrides)
            double g00 = dot4<S>(g + 0, 2, u + 0, 2);
            double g01 = dot4<S>(g + 0, 2, u + 1, 2);
            double g10 = dot4<S>(g + 1, 2, u + 0, 2);
            double g11 = dot4<S>(g + 1, 2, u + 1, 2);
            if constexpr (MODE == 0) {
                o[0] = g00; o[1] = g01; o[2] = g10; o[3] = g11;
            }
            else if constexpr (MODE == 1) {
                o[0] = g00; o[2] = g01; o[1] = g10; o[3] = g11;
            }
            else {
                // 0.5 * (8-term left-to-right sum)
                double s = g01;
                s = madd<S>(g[1], u[0], s);
                s = madd<S>(g[3], u[2], s);
                s = madd<S>(g[5], u[4], s);
                s = madd<S>(g[7], u[6], s);
                s = mul<S>(0.5, s);
                o[0] = g00; o[3] = g11; o[1] = s; o[2] = s;
            }
        }
        else {
            // Element.h:925-1022 (generic loops from a zero-filled output)
#pragma unroll
            for (int k = 0; k < ND * ND; ++k) o[k] = 0.0;
#pragma unroll
            for (int m = 0; m < NNE; ++m)
#pragma unroll
                for (int i = 0; i < ND; ++i)
#pragma unroll
                    for (int j = 0; j < ND; ++j) {
                        if constexpr (MODE == 0) {
                            o[i * ND + j] = madd<S>(g[m * ND + i], u[m * ND + j], o[i * ND + j]);
                        }
                        else if constexpr (MODE == 1) {
                            o[j * ND + i] = madd<S>(g[m * ND + i], u[m * ND + j], o[j * ND + i]);
                        }
                        else {
                            double h = mul<S>(0.5, g[m * ND + i]);
                            o[i * ND + j] = madd<S>(h, u[m * ND + j], o[i * ND + j]);
                            o[j * ND + i] = madd<S>(h, u[m * ND + j], o[j * ND + i]);
                        }
                    }
        }
        if constexpr (TD == ND) {
            store<ND * ND>(qtensor + t * ND * ND, o);
        }
        else {
            double* out = qtensor + t * TD * TD;
#pragma unroll
            for (int i = 0; i < TD; ++i)
#pragma unroll
                for (int j = 0; j < TD; ++j) out[i * TD + j] = (i < ND && j < ND) ? o[i * ND + j] : 0.0;
        }
    }
}

// InterpQuad_vector: ElementQuad4.h:325-346 (n = 2, unrolled) / Element.h:893-922.
template <bool S>
__global__ void k_interp(const double* __restrict__ N, const double* __restrict__ elemvec,
                         int64_t nelem, int nne, int nip, int n, double* __restrict__ qvector)
{
    GF_FOR(t, nelem * nip)
    {
        int64_t e = t / nip;
        int q = static_cast<int>(t - e * nip);
        const double* Nq = N + q * nne;
        const double* u = elemvec + e * nne * n;
        double* o = qvector + t * n;
        for (int i = 0; i < n; ++i) {
            double acc;
            if (nne == 4 && n == 2) {
                acc = mul<S>(Nq[0], u[i]);
                for (int m = 1; m < 4; ++m) acc = madd<S>(Nq[m], u[m * n + i], acc);
            }
            else {
                acc = 0.0;
                for (int m = 0; m < nne; ++m) acc = madd<S>(Nq[m], u[m * n + i], acc);
            }
            o[i] = acc;
        }
    }
}

// ---------------------------------------------------------------- integrals (thread per element)

// Int_gradN_dot_tensor2_dV: ElementQuad4.h:467-491 / ElementHex8.h:355-383.
// TD = 3 with ND = 2: QuadraturePlanar (ElementQuad4Planar.h:254-277), the in-plane block of
// each 3x3 tensor.
template <bool S, int NNE, int ND, int TD = ND>
__global__ void k_int_grad_tensor2(const double* __restrict__ dNx, const double* __restrict__ vol,
                                   const double* __restrict__ qtensor, int64_t nelem, int nip,
                                   double* __restrict__ elemvec)
{
    GF_FOR(e, nelem)
    {
        double f[NNE * ND];
#pragma unroll
        for (int k = 0; k < NNE * ND; ++k) f[k] = 0.0;
        for (int q = 0; q < nip; ++q) {
            int64_t t = e * nip + q;
            double g[NNE * ND], s[ND * ND];
            load<NNE * ND>(dNx + t * NNE * ND, g);
            if constexpr (ND == 2 && TD == 2) load<4>(qtensor + t * 4, s);
            else if constexpr (ND == 2) {
                s[0] = __ldg(qtensor + t * 9 + 0);
                s[1] = __ldg(qtensor + t * 9 + 1);
                s[2] = __ldg(qtensor + t * 9 + 3);
                s[3] = __ldg(qtensor + t * 9 + 4);
            }
            else {
#pragma unroll
                for (int k = 0; k < 9; ++k) s[k] = __ldg(qtensor + t * 9 + k);
            }
            double v = __ldg(vol + t);
#pragma unroll
            for (int m = 0; m < NNE; ++m)
#pragma unroll
                for (int j = 0; j < ND; ++j) {
                    double acc = mul<S>(g[m * ND + 0], s[0 * ND + j]);
#pragma unroll
                    for (int i = 1; i < ND; ++i) acc = madd<S>(g[m * ND + i], s[i * ND + j], acc);
                    f[m * ND + j] = madd<S>(acc, v, f[m * ND + j]);
                }
        }
        store<NNE * ND>(elemvec + e * NNE * ND, f);
    }
}

// Int_N_vector_dV: Element.h:1025-1056.
template <bool S>
__global__ void k_int_n_vector(const double* __restrict__ N, const double* __restrict__ vol,
                               const double* __restrict__ qvector, int64_t nelem, int nne, int nip,
                               int n, double* __restrict__ elemvec)
{
    GF_FOR(t, nelem * nne * n)
    {
        int64_t e = t / (nne * n);
        int r = static_cast<int>(t - e * nne * n);
        int m = r / n, i = r - m * n;
        double acc = 0.0;
        for (int q = 0; q < nip; ++q)
            acc = madd<S>(mul<S>(N[q * nne + m], qvector[(e * nip + q) * n + i]), vol[e * nip + q],
                          acc);
        elemvec[t] = acc;
    }
}

// Int_N_scalar_NT_dV: ElementQuad4.h:437-464 / ElementHex8.h:324-352. Thread per elemmat entry.
template <bool S>
__global__ void k_int_n_scalar(const double* __restrict__ N, const double* __restrict__ vol,
                               const double* __restrict__ qscalar, int64_t nelem, int nne,
                               int nip, int nd, double* __restrict__ elemmat)
{
    int K = nne * nd;
    GF_FOR(t, nelem * K * K)
    {
        int64_t e = t / (K * K);
        int rc = static_cast<int>(t - e * K * K);
        int r = rc / K, c = rc - r * K;
        double acc = 0.0;
        if (r % nd == c % nd) {
            int m = r / nd, n = c / nd;
            for (int q = 0; q < nip; ++q)
                acc = madd<S>(mul<S>(mul<S>(N[q * nne + m], qscalar[e * nip + q]), N[q * nne + n]),
                              vol[e * nip + q], acc);
        }
        elemmat[t] = acc;
    }
}

// Diagonal of Int_N_scalar_NT_dV only (the lumped mass of MatrixDiagonal::assemble,
// MatrixDiagonal.h:151-167): thread per (e, m), out elemvec (e, m, i) = elemmat(e, m*nd+i, m*nd+i)
// with k_int_n_scalar's operations for that entry (same bits). With offdiag != null the row's
// off-diagonal entries (m, n != m) are summed too and *offdiag is cleared if one exceeds
// DBL_EPSILON in magnitude (Element::isDiagonal, Element.h:122-145); nothing of the full
// [nelem, nne*nd, nne*nd] matrix is stored.
template <bool S>
__global__ void k_int_n_scalar_diag(const double* __restrict__ N, const double* __restrict__ vol,
                                    const double* __restrict__ qscalar, int64_t nelem, int nne,
                                    int nip, int nd, double* __restrict__ out, int* __restrict__ offdiag)
{
    const double eps = 2.220446049250313080847e-16; // DBL_EPSILON
    GF_FOR(t, nelem * nne)
    {
        const int64_t e = t / nne;
        const int m = static_cast<int>(t - e * nne);
        double acc = 0.0;
        for (int q = 0; q < nip; ++q)
            acc = madd<S>(mul<S>(mul<S>(N[q * nne + m], qscalar[e * nip + q]), N[q * nne + m]),
                          vol[e * nip + q], acc);
        for (int i = 0; i < nd; ++i) out[t * nd + i] = acc;
        if (offdiag) {
            for (int n = 0; n < nne; ++n) {
                if (n == m) continue;
                double o = 0.0;
                for (int q = 0; q < nip; ++q)
                    o = madd<S>(mul<S>(mul<S>(N[q * nne + m], qscalar[e * nip + q]), N[q * nne + n]),
                                vol[e * nip + q], o);
                if (fabs(o) > eps) *offdiag = 0;
            }
        }
    }
}

// Int_gradN_dot_tensor4_dot_gradNT_dV: Element.h:1132-1176. Thread per elemmat entry; the
// entry (m*nd+j, n*nd+k) accumulates over q, then i, then l as in the reference loop nest.
// td: tensor dimension of C (td = 3 with nd = 2: QuadraturePlanar, the in-plane indices of a
// [3,3,3,3] tensor).
template <bool S>
__global__ void k_int_tensor4(const double* __restrict__ dNx, const double* __restrict__ vol,
                              const double* __restrict__ C, int64_t nelem, int nne, int nip,
                              int nd, int td, double* __restrict__ elemmat)
{
    int K = nne * nd;
    GF_FOR(t, nelem * K * K)
    {
        int64_t e = t / (K * K);
        int rc = static_cast<int>(t - e * K * K);
        int r = rc / K, c = rc - r * K;
        int m = r / nd, j = r - m * nd, n = c / nd, k = c - n * nd;
        double acc = 0.0;
        for (int q = 0; q < nip; ++q) {
            const double* g = dNx + (e * nip + q) * nne * nd;
            const double* Cq = C + (e * nip + q) * td * td * td * td;
            double v = vol[e * nip + q];
            for (int i = 0; i < nd; ++i)
                for (int l = 0; l < nd; ++l)
                    acc = madd<S>(mul<S>(mul<S>(g[m * nd + i], Cq[((i * td + j) * td + k) * td + l]),
                                         g[n * nd + l]),
                                  v, acc);
        }
        elemmat[t] = acc;
    }
}

// Linear elastic stress (plane strain for nd = 2), same operation order as the oracle.
template <bool S>
__global__ void k_stress(const double* __restrict__ eps, const double* __restrict__ K,
                         const double* __restrict__ G, int64_t nelem, int nip, int nd,
                         double* __restrict__ sig)
{
    GF_FOR(t, nelem * nip)
    {
        int64_t e = t / nip;
        const double* s = eps + t * nd * nd;
        double* o = sig + t * nd * nd;
        double g2 = mul<S>(2.0, G[e]);
        double tr = 0.0;
        for (int i = 0; i < nd; ++i) tr = add<S>(tr, s[i * nd + i]);
        double Kt = mul<S>(K[e], tr);
        double m = __ddiv_rn(tr, 3.0);
        for (int i = 0; i < nd; ++i)
            for (int j = 0; j < nd; ++j)
                o[i * nd + j] = (i == j) ? madd<S>(g2, sub<S>(s[i * nd + j], m), Kt)
                                         : mul<S>(g2, s[i * nd + j]);
    }
}

static bool aligned16(const void* p)
{
    return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

static int check_elem(int nne, int nd)
{
    if ((nne == 4 && nd == 2) || (nne == 8 && nd == 3)) return GFGPU_OK;
    return fail(GFGPU_ERR_UNSUPPORTED, "only Quad4 (nne=4, ndim=2) and Hex8 (nne=8, ndim=3)");
}

} // namespace gfgpu

using namespace gfgpu;

#define DISPATCH_S(...)                                                                         \
    do {                                                                                        \
        if (strict_mode()) {                                                                    \
            constexpr bool kS = true;                                                           \
            __VA_ARGS__;                                                                        \
        }                                                                                       \
        else {                                                                                  \
            constexpr bool kS = false;                                                          \
            __VA_ARGS__;                                                                        \
        }                                                                                       \
    } while (0)

template <int MODE>
static int grad(const double* dNx, const double* elemvec, int64_t nelem, int32_t nne, int32_t nip,
                int32_t nd, double* qtensor, gfgpu_stream_t stream, bool planar = false)
{
    GF_REQUIRE(dNx && elemvec && qtensor && nip > 0, "bad argument");
    GF_TRY(check_elem(nne, nd));
    GF_REQUIRE(!too_big(nelem * nip * 24), "too many elements");
    GF_REQUIRE(aligned16(dNx) && aligned16(elemvec), "dNx and elemvec must be 16-byte aligned");
    if (nelem == 0) return GFGPU_OK;
    unsigned g = grid_for(nelem * nip);
    if (planar)
        DISPATCH_S(k_grad<kS, 4, 2, MODE, 3><<<g, kBlock, 0, S(stream)>>>(dNx, elemvec, nelem, nip, qtensor));
    else if (nd == 2)
        DISPATCH_S(k_grad<kS, 4, 2, MODE><<<g, kBlock, 0, S(stream)>>>(dNx, elemvec, nelem, nip, qtensor));
    else
        DISPATCH_S(k_grad<kS, 8, 3, MODE><<<g, kBlock, 0, S(stream)>>>(dNx, elemvec, nelem, nip, qtensor));
    return check_launch("grad_n_vector");
}

extern "C" {

static int compute_dN(int nd, const double* x, int64_t nelem, const double* xi, const double* w,
                      int32_t nip, double* N, double* dNxi, double* dNx, double* vol,
                      gfgpu_stream_t stream, double thick = 1.0)
{
    GF_REQUIRE(x && xi && w && dNx && vol && nip > 0 && nelem >= 0, "bad argument");
    GF_REQUIRE(!too_big(nelem * nip * 24), "too many elements");
    GF_REQUIRE(aligned16(x) && aligned16(dNx), "x and dNx must be 16-byte aligned");
    if (N || dNxi) k_shape<<<1, 64, 0, S(stream)>>>(xi, nip, nd, N, dNxi);
    if (nelem > 0) {
        if (nd == 2)
            k_quad4_compute_dN<<<grid_for(nelem * nip), kBlock, 0, S(stream)>>>(x, nelem, xi, w, nip,
                                                                              thick, dNx, vol);
        else
            k_hex8_compute_dN<<<grid_for(nelem * nip), kBlock, 0, S(stream)>>>(x, nelem, xi, w, nip,
                                                                             dNx, vol);
    }
    return check_launch("compute_dN");
}

int gfgpu_quad4_compute_dN(const double* x, int64_t nelem, const double* xi, const double* w,
                           int32_t nip, double* N, double* dNxi, double* dNx, double* vol,
                           gfgpu_stream_t stream)
{
    return compute_dN(2, x, nelem, xi, w, nip, N, dNxi, dNx, vol, stream);
}

int gfgpu_hex8_compute_dN(const double* x, int64_t nelem, const double* xi, const double* w,
                          int32_t nip, double* N, double* dNxi, double* dNx, double* vol,
                          gfgpu_stream_t stream)
{
    return compute_dN(3, x, nelem, xi, w, nip, N, dNxi, dNx, vol, stream);
}

int gfgpu_interp_quad_vector(const double* N, const double* elemvec, int64_t nelem, int32_t nne,
                             int32_t nip, int32_t n, double* qvector, gfgpu_stream_t stream)
{
    GF_REQUIRE(N && elemvec && qvector && nne > 0 && nip > 0 && n > 0, "bad argument");
    GF_REQUIRE(!too_big(nelem * nip * n), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    DISPATCH_S(k_interp<kS><<<grid_for(nelem * nip), kBlock, 0, S(stream)>>>(N, elemvec, nelem, nne,
                                                                             nip, n, qvector));
    return check_launch("interp_quad_vector");
}

int gfgpu_grad_n_vector(const double* dNx, const double* elemvec, int64_t nelem, int32_t nne,
                        int32_t nip, int32_t ndim, double* qtensor, gfgpu_stream_t stream)
{
    return grad<0>(dNx, elemvec, nelem, nne, nip, ndim, qtensor, stream);
}

int gfgpu_grad_n_vector_T(const double* dNx, const double* elemvec, int64_t nelem, int32_t nne,
                          int32_t nip, int32_t ndim, double* qtensor, gfgpu_stream_t stream)
{
    return grad<1>(dNx, elemvec, nelem, nne, nip, ndim, qtensor, stream);
}

int gfgpu_sym_grad_n_vector(const double* dNx, const double* elemvec, int64_t nelem, int32_t nne,
                            int32_t nip, int32_t ndim, double* qtensor, gfgpu_stream_t stream)
{
    return grad<2>(dNx, elemvec, nelem, nne, nip, ndim, qtensor, stream);
}

int gfgpu_int_n_vector_dv(const double* N, const double* vol, const double* qvector,
                          int64_t nelem, int32_t nne, int32_t nip, int32_t n, double* elemvec,
                          gfgpu_stream_t stream)
{
    GF_REQUIRE(N && vol && qvector && elemvec && nne > 0 && nip > 0 && n > 0, "bad argument");
    GF_REQUIRE(!too_big(nelem * nne * n), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    DISPATCH_S(k_int_n_vector<kS><<<grid_for(nelem * nne * n), kBlock, 0, S(stream)>>>(
        N, vol, qvector, nelem, nne, nip, n, elemvec));
    return check_launch("int_n_vector_dv");
}

int gfgpu_int_n_scalar_nt_dv(const double* N, const double* vol, const double* qscalar,
                             int64_t nelem, int32_t nne, int32_t nip, int32_t ndim,
                             double* elemmat, gfgpu_stream_t stream)
{
    GF_REQUIRE(N && vol && qscalar && elemmat && nip > 0, "bad argument");
    GF_TRY(check_elem(nne, ndim));
    int64_t K = nne * ndim;
    GF_REQUIRE(!too_big(nelem * K * K), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    DISPATCH_S(k_int_n_scalar<kS><<<grid_for(nelem * K * K), kBlock, 0, S(stream)>>>(
        N, vol, qscalar, nelem, nne, nip, ndim, elemmat));
    return check_launch("int_n_scalar_nt_dv");
}

int gfgpu_int_n_scalar_nt_dv_diag(const double* N, const double* vol, const double* qscalar,
                                  int64_t nelem, int32_t nne, int32_t nip, int32_t ndim,
                                  double* elemvec, int* is_diag, gfgpu_stream_t stream)
{
    GF_REQUIRE(N && vol && qscalar && elemvec && nip > 0, "bad argument");
    GF_TRY(check_elem(nne, ndim));
    GF_REQUIRE(!too_big(nelem * nne * ndim), "too many elements");
    cudaStream_t s = S(stream);
    int* flag = nullptr;
    if (is_diag) {
        GF_TRY(check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&flag), sizeof(int), s), "cudaMallocAsync"));
        const int one = 1;
        int rc = check_cuda(cudaMemcpyAsync(flag, &one, sizeof(int), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        if (rc != GFGPU_OK) {
            cudaFreeAsync(flag, s);
            return rc;
        }
    }
    int rc = GFGPU_OK;
    if (nelem > 0) {
        DISPATCH_S(k_int_n_scalar_diag<kS><<<grid_for(nelem * nne), kBlock, 0, s>>>(
            N, vol, qscalar, nelem, nne, nip, ndim, elemvec, flag));
        rc = check_launch("int_n_scalar_nt_dv_diag");
    }
    if (!is_diag) return rc;
    *is_diag = 0;
    if (rc == GFGPU_OK) rc = check_cuda(cudaMemcpyAsync(is_diag, flag, sizeof(int), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    const int rc_free = check_cuda(cudaFreeAsync(flag, s), "cudaFreeAsync");
    if (rc == GFGPU_OK) rc = rc_free;
    if (rc == GFGPU_OK) rc = check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return rc;
}

int gfgpu_int_grad_n_dot_tensor2_dv(const double* dNx, const double* vol, const double* qtensor,
                                    int64_t nelem, int32_t nne, int32_t nip, int32_t ndim,
                                    double* elemvec, gfgpu_stream_t stream)
{
    GF_REQUIRE(dNx && vol && qtensor && elemvec && nip > 0, "bad argument");
    GF_TRY(check_elem(nne, ndim));
    GF_REQUIRE(!too_big(nelem * nip * 24), "too many elements");
    GF_REQUIRE(aligned16(dNx) && aligned16(qtensor), "dNx and qtensor must be 16-byte aligned");
    if (nelem == 0) return GFGPU_OK;
    unsigned g = grid_for(nelem, 128);
    if (ndim == 2)
        DISPATCH_S(k_int_grad_tensor2<kS, 4, 2><<<g, 128, 0, S(stream)>>>(dNx, vol, qtensor, nelem,
                                                                          nip, elemvec));
    else
        DISPATCH_S(k_int_grad_tensor2<kS, 8, 3><<<g, 128, 0, S(stream)>>>(dNx, vol, qtensor, nelem,
                                                                          nip, elemvec));
    return check_launch("int_grad_n_dot_tensor2_dv");
}

int gfgpu_int_grad_n_dot_tensor4_dot_grad_nt_dv(const double* dNx, const double* vol,
                                                const double* qtensor4, int64_t nelem,
                                                int32_t nne, int32_t nip, int32_t ndim,
                                                double* elemmat, gfgpu_stream_t stream)
{
    GF_REQUIRE(dNx && vol && qtensor4 && elemmat && nip > 0, "bad argument");
    GF_TRY(check_elem(nne, ndim));
    int64_t K = nne * ndim;
    GF_REQUIRE(!too_big(nelem * K * K), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    DISPATCH_S(k_int_tensor4<kS><<<grid_for(nelem * K * K), kBlock, 0, S(stream)>>>(
        dNx, vol, qtensor4, nelem, nne, nip, ndim, ndim, elemmat));
    return check_launch("int_grad_n_dot_tensor4_dot_grad_nt_dv");
}

// ---------------------------------------------------------------- QuadraturePlanar

int gfgpu_quad4_planar_compute_dN(const double* x, int64_t nelem, const double* xi,
                                  const double* w, int32_t nip, double thick, double* N,
                                  double* dNxi, double* dNx, double* vol, gfgpu_stream_t stream)
{
    return compute_dN(2, x, nelem, xi, w, nip, N, dNxi, dNx, vol, stream, thick);
}

int gfgpu_grad_n_vector_planar(const double* dNx, const double* elemvec, int64_t nelem,
                               int32_t nip, double* qtensor, gfgpu_stream_t stream)
{
    return grad<0>(dNx, elemvec, nelem, 4, nip, 2, qtensor, stream, true);
}

int gfgpu_grad_n_vector_T_planar(const double* dNx, const double* elemvec, int64_t nelem,
                                 int32_t nip, double* qtensor, gfgpu_stream_t stream)
{
    return grad<1>(dNx, elemvec, nelem, 4, nip, 2, qtensor, stream, true);
}

int gfgpu_sym_grad_n_vector_planar(const double* dNx, const double* elemvec, int64_t nelem,
                                   int32_t nip, double* qtensor, gfgpu_stream_t stream)
{
    return grad<2>(dNx, elemvec, nelem, 4, nip, 2, qtensor, stream, true);
}

int gfgpu_int_grad_n_dot_tensor2_dv_planar(const double* dNx, const double* vol,
                                           const double* qtensor, int64_t nelem, int32_t nip,
                                           double* elemvec, gfgpu_stream_t stream)
{
    GF_REQUIRE(dNx && vol && qtensor && elemvec && nip > 0, "bad argument");
    GF_REQUIRE(!too_big(nelem * nip * 9), "too many elements");
    GF_REQUIRE(aligned16(dNx), "dNx must be 16-byte aligned");
    if (nelem == 0) return GFGPU_OK;
    unsigned g = grid_for(nelem, 128);
    DISPATCH_S(k_int_grad_tensor2<kS, 4, 2, 3><<<g, 128, 0, S(stream)>>>(dNx, vol, qtensor, nelem,
                                                                         nip, elemvec));
    return check_launch("int_grad_n_dot_tensor2_dv_planar");
}

int gfgpu_int_grad_n_dot_tensor4_dot_grad_nt_dv_planar(const double* dNx, const double* vol,
                                                       const double* qtensor4, int64_t nelem,
                                                       int32_t nip, double* elemmat,
                                                       gfgpu_stream_t stream)
{
    GF_REQUIRE(dNx && vol && qtensor4 && elemmat && nip > 0, "bad argument");
    GF_REQUIRE(!too_big(nelem * 64) && !too_big(nelem * nip * 81), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    DISPATCH_S(k_int_tensor4<kS><<<grid_for(nelem * 64), kBlock, 0, S(stream)>>>(
        dNx, vol, qtensor4, nelem, 4, nip, 2, 3, elemmat));
    return check_launch("int_grad_n_dot_tensor4_dot_grad_nt_dv_planar");
}

int gfgpu_elastic_stress(const double* eps, const double* K, const double* G, int64_t nelem,
                         int32_t nip, int32_t ndim, double* sig, gfgpu_stream_t stream)
{
    GF_REQUIRE(eps && K && G && sig && nip > 0 && (ndim == 2 || ndim == 3), "bad argument");
    GF_REQUIRE(!too_big(nelem * nip * 9), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    DISPATCH_S(k_stress<kS><<<grid_for(nelem * nip), kBlock, 0, S(stream)>>>(eps, K, G, nelem, nip,
                                                                            ndim, sig));
    return check_launch("elastic_stress");
}

} // extern "C"
