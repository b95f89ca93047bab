/*
 * gfgpu — GB300-native (sm_103a) element hot path of GooseFEM behind a plain C ABI.
 *
 * Conventions (every entry point):
 *  - returns GFGPU_OK (0) or a negative GFGPU_ERR_* code; gfgpu_last_error() has the message;
 *  - arrays are row-major, FP64 values, int32 indices (the reference's size_t tables are
 *    narrowed once at set-up; sizes above 2^31-1 entries are rejected with GFGPU_ERR_ARG);
 *  - functions named gfgpu_host_* take HOST pointers and run on the CPU (set-up / bookkeeping);
 *    every other function takes DEVICE pointers and enqueues work on `stream`
 *    (a cudaStream_t; NULL = legacy default stream) and returns without synchronising,
 *    unless its comment says otherwise;
 *  - storage names follow GooseFEM: "dofval" [ndof], "nodevec" [nnode, ndim],
 *    "elemvec" [nelem, nne, ndim], "elemmat" [nelem, nne*ndim, nne*ndim],
 *    "qscalar" [nelem, nip], "qvector" [nelem, nip, n], "qtensor" [nelem, nip, ndim, ndim].
 *
 * Reference paths cited below are relative to the GooseFEM source tree.
 */
#ifndef GFGPU_H
#define GFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* gfgpu_stream_t;

enum {
    GFGPU_OK = 0,
    GFGPU_ERR_ARG = -1,          /* bad size / shape / null pointer (GOOSEFEM_ASSERT) */
    GFGPU_ERR_INDEX = -2,        /* index table out of range */
    GFGPU_ERR_CUDA = -3,         /* CUDA runtime error */
    GFGPU_ERR_TIMEOUT = -4,      /* bounded device wait gave up */
    GFGPU_ERR_NAN = -5,          /* non-finite value detected */
    GFGPU_ERR_NOT_DIAGONAL = -6, /* MatrixDiagonal::assemble on a non-diagonal elemmat */
    GFGPU_ERR_UNSUPPORTED = -7,  /* element type / quadrature not supported by this entry */
    GFGPU_ERR_DIVERGED = -8      /* iterative solver did not converge */
};

/* Message of the last failing call on this host thread. */
const char* gfgpu_last_error(void);
/* Library version string. */
const char* gfgpu_version(void);

/* Arithmetic mode of the operator kernels and of the general-path explicit step:
 * 0 = fast (FMA contraction and reassociation allowed; agreement with the reference ~1e-15),
 * 1 = strict (every product and sum rounded separately in the reference's order, which
 *     reproduces the reference's FP64 results bit for bit). Default 0. Process-wide.
 * The closed-form uniform element kernels are never bit-exact (they sum differently). */
int gfgpu_set_strict(int strict);

/* Kernel variants of the fast explicit increment (process-wide, default 0 / 0):
 * elem_variant 1 = two neighbouring elements per thread in the uniform square Quad4 kernel,
 * node_variant 1 = both dofs of a node per thread in the node kernel. Same results. */
int gfgpu_set_variant(int elem_variant, int node_variant);
/* Kernel of the float-float explicit increment (gfgpu_verlet_precompute_pair), process-wide:
 * 2 (default) = persistent CTAs of 512 threads that prefetch the next 31 x 15 node tile's inputs
 * by TMA into a second shared-memory stage while computing the current one, x and y of a node in
 * the packed FP32x2 instructions; 0 = the same with 31 x 7 node tiles and 256 threads; 1 = one
 * 32 x 8 node tile per CTA with plain loads and scalar FP32. Same arithmetic (0 and 2 bit-identical),
 * the four-element sums grouped differently in 1 (agreement ~1e-14). */
int gfgpu_set_pair_kernel(int kernel);
/* Timeout flag of the pair kernels' bounded waits for their TMA copies: GFGPU_ERR_TIMEOUT if a
 * wait gave up since the last call (the increment's results are then invalid), else GFGPU_OK.
 * Clears the flag. Synchronises the device. */
int gfgpu_verlet_pair_status(void);
/* Tensor-core instructions of the network's 32 -> 32 layers (process-wide): 0 = mma.sync m16n8k16,
 * 1 = tcgen05.mma with TMEM accumulators, one tile per CTA, 2 (default) = tcgen05.mma in a
 * persistent pipeline fed by TMA (cp.async.bulk.tensor) with 2-3 shared-memory stages of whole
 * halo tiles and double-buffered TMEM, 3 = the same pipeline with a ring of halo rows that
 * consecutive tiles of a column strip share (each row loaded once per run of tiles). Same
 * arithmetic (BF16 products, FP32 accumulation); the summation order differs between 0, 1 and
 * 2/3 (2 and 3 give identical bits). */
int gfgpu_set_nn_tensor_path(int path);
/* Programmatic dependent launch between the network's layers on path 2 (process-wide, default
 * 1): each layer lets the next one launch once its CTAs are resident; the next one sets up
 * (TMEM, barriers, weights) and executes griddepcontrol.wait before it reads the previous layer's
 * output or writes anything. 0 = ordinary stream-ordered launches. Same results bit for bit. */
int gfgpu_set_nn_pdl(int on);
/* Error flag of the tcgen05 layers' bounded waits: GFGPU_ERR_TIMEOUT if a wait for the tensor
 * cores gave up since the last call (the layer's output is then invalid), else GFGPU_OK. Clears
 * the flag. Synchronises the device. */
int gfgpu_nn_tc_status(void);

/* ============================ device memory helpers ======================================= */

/* Thin wrappers of the CUDA runtime so that a host program can use the library without
 * including CUDA headers (the C++ layer include/gfgpu/GooseFEM.hpp uses them). */
int gfgpu_malloc(void** ptr, int64_t bytes);
int gfgpu_free(void* ptr);
int gfgpu_memcpy_h2d(void* dst, const void* src, int64_t bytes);
int gfgpu_memcpy_d2h(void* dst, const void* src, int64_t bytes);
int gfgpu_memcpy_d2d(void* dst, const void* src, int64_t bytes);
int gfgpu_memset(void* ptr, int value, int64_t bytes);
int gfgpu_synchronize(void);

/* ============================ set-up on the host (integer bookkeeping) ==================== */

/* Mesh::Quad4::Regular coor/conn (MeshQuad4.h:87-126). coor [nnode,2], conn [nelem,4]. */
int gfgpu_host_quad4_regular(int64_t nx, int64_t ny, double h, double* coor, int32_t* conn);
/* Mesh::Hex8::Regular coor/conn (MeshHex8.h:77-130). coor [nnode,3], conn [nelem,8]. */
int gfgpu_host_hex8_regular(int64_t nx, int64_t ny, int64_t nz, double h, double* coor,
                            int32_t* conn);
/* Mesh::dofs (Mesh.h:93-96): arange(nnode*ndim).reshape(nnode, ndim). */
int gfgpu_host_dofs(int64_t nnode, int32_t ndim, int32_t* dofs);
/* RegularBase2d::nodesPeriodic (Mesh.h:511-540) of Quad4 Regular; out [(nx-1)+(ny-1)+3, 2]. */
int gfgpu_host_quad4_nodes_periodic(int64_t nx, int64_t ny, int32_t* out, int64_t* nper);
/* RegularBase3d::nodesPeriodic for Mesh::Hex8::Regular (Mesh.h:1577-1692 with the face / edge /
 * corner sets of MeshHex8.h:214-600): 7 corner pairs, the open edges, then the open faces.
 * `out` holds 7 + 3((nx-1) + (ny-1) + (nz-1)) + (nx-1)(ny-1) + (ny-1)(nz-1) + (nx-1)(nz-1)
 * rows of (independent, dependent). */
int gfgpu_host_hex8_nodes_periodic(int64_t nx, int64_t ny, int64_t nz, int32_t* out, int64_t* nper);
/* RegularBase::dofsPeriodic (Mesh.h:291-306) given a nodesPeriodic table. */
int gfgpu_host_dofs_periodic(int64_t nnode, int32_t ndim, const int32_t* nodes_periodic,
                             int64_t nper, int32_t* dofs);
/* Mesh::Renumber (Mesh.h:114-166): index of each entry in the sorted unique list. */
int gfgpu_host_renumber(const int32_t* in, int64_t n, int32_t* out);
/* VectorPartitioned / MatrixDiagonalPartitioned bookkeeping (VectorPartitioned.h:72-88):
 * iiu = setdiff1d(dofs, iip) (sorted unique), part = Reorder({iiu, iip}).apply(dofs)
 * (Mesh.h:2384-2450). iiu needs room for n entries; *nnu receives its length. */
int gfgpu_host_partition(const int32_t* dofs, int64_t n, const int32_t* iip, int64_t nnp,
                         int32_t* iiu, int32_t* part, int64_t* nnu);
/* Mesh::coordination (Mesh.h:2462-2477). */
int gfgpu_host_coordination(const int32_t* conn, int64_t nelem, int32_t nne, int64_t nnode,
                            int32_t* N);
/* Mesh::elem2node, sorted (Mesh.h:2485-2513) as CSR: ptr [nnode+1], idx [nelem*nne]. */
int gfgpu_host_elem2node(const int32_t* conn, int64_t nelem, int32_t nne, int64_t nnode,
                         int32_t* ptr, int32_t* idx);
/* Dof-centric incidence CSR behind the deterministic assembly (replaces the serial scatter of
 * Vector.h:724-741 and MatrixDiagonal.h:151-167): for dof d, idx[ptr[d]:ptr[d+1]] lists the
 * flat elemvec indices (e*nne+m)*ndim+i with dofs[conn[e,m], i] == d in ascending order, i.e.
 * the reference's serial summation order. ptr [ndof+1], idx [nelem*nne*ndim]. `dofs` may be
 * any dof numbering (GooseFEM dofs, or the partitioned numbering `part`). */
int gfgpu_host_dof_csr(const int32_t* conn, const int32_t* dofs, int64_t nelem, int32_t nne,
                       int64_t nnode, int32_t ndim, int64_t ndof, int32_t* ptr, int32_t* idx);
/* Same for nodevec sources (Vector.h:703-718): idx lists flat nodevec indices m*ndim+i. */
int gfgpu_host_dof_csr_nodevec(const int32_t* dofs, int64_t nnode, int32_t ndim, int64_t ndof,
                               int32_t* ptr, int32_t* idx);

/* ============================ Element quadrature (device) ================================= */

/* Quadrature(x, xi, w) set-up: shape functions and compute_dN.
 * Quad4: ElementQuad4.h:277-318 + compute_dN_impl :493-532 (detail.h:26-36 inverse).
 * Hex8:  ElementHex8.h:255-317 + Element.h:1178-1229 (detail.h:49-69), restated as written.
 * x elemvec [nelem,nne,ndim]; xi [nip,ndim]; w [nip]; out: N [nip,nne], dNxi [nip,nne,ndim]
 * (either may be NULL), dNx [nelem,nip,nne,ndim], vol [nelem,nip]. Always strict (bit-exact). */
int gfgpu_quad4_compute_dN(const double* x, int64_t nelem, const double* xi, const double* w,
                           int32_t nip, double* N, double* dNxi, double* dNx, double* vol,
                           gfgpu_stream_t stream);
int gfgpu_hex8_compute_dN(const double* x, int64_t nelem, const double* xi, const double* w,
                          int32_t nip, double* N, double* dNxi, double* dNx, double* vol,
                          gfgpu_stream_t stream);

/* InterpQuad_vector (ElementQuad4.h:325-346; Element.h:893-922): qvector [nelem,nip,n]. */
int gfgpu_interp_quad_vector(const double* N, const double* elemvec, int64_t nelem, int32_t nne,
                             int32_t nip, int32_t n, double* qvector, gfgpu_stream_t stream);
/* GradN_vector / GradN_vector_T / SymGradN_vector (ElementQuad4.h:349-434; Element.h:925-1022).
 * dNx [nelem,nip,nne,ndim], elemvec [nelem,nne,ndim] -> qtensor [nelem,nip,ndim,ndim]. */
int gfgpu_grad_n_vector(const double* dNx, const double* elemvec, int64_t nelem, int32_t nne,
                        int32_t nip, int32_t ndim, double* qtensor, gfgpu_stream_t stream);
int gfgpu_grad_n_vector_T(const double* dNx, const double* elemvec, int64_t nelem, int32_t nne,
                          int32_t nip, int32_t ndim, double* qtensor, gfgpu_stream_t stream);
int gfgpu_sym_grad_n_vector(const double* dNx, const double* elemvec, int64_t nelem, int32_t nne,
                            int32_t nip, int32_t ndim, double* qtensor, gfgpu_stream_t stream);
/* Int_N_vector_dV (Element.h:1025-1056): qvector [nelem,nip,n] -> elemvec [nelem,nne,n]. */
int gfgpu_int_n_vector_dv(const double* N, const double* vol, const double* qvector,
                          int64_t nelem, int32_t nne, int32_t nip, int32_t n, double* elemvec,
                          gfgpu_stream_t stream);
/* Int_N_scalar_NT_dV (ElementQuad4.h:437-464; ElementHex8.h:324-352): -> elemmat. */
int gfgpu_int_n_scalar_nt_dv(const double* N, const double* vol, const double* qscalar,
                             int64_t nelem, int32_t nne, int32_t nip, int32_t ndim,
                             double* elemmat, gfgpu_stream_t stream);
/* Diagonal of Int_N_scalar_NT_dV only, for the lumped mass of MatrixDiagonal::assemble
 * (ElementQuad4.h:437-464, ElementHex8.h:324-352, MatrixDiagonal.h:151-167): elemvec
 * [nelem,nne,ndim] with elemvec(e,m,i) = elemmat(e, m*ndim+i, m*ndim+i), the same operations and
 * bits as gfgpu_int_n_scalar_nt_dv's diagonal, without the [nelem, nne*ndim, nne*ndim] matrix.
 * Assemble it with gfgpu_assemble_dofs on the dof CSR (gfgpu_host_dof_csr; the CSR on `part` for
 * MatrixDiagonalPartitioned): the same sums in the same order as gfgpu_diag_assemble. With
 * is_diag != NULL the off-diagonal entries are formed too (not stored) and *is_diag (host int)
 * receives Element::isDiagonal's verdict (Element.h:122-145: every |off-diagonal| <= DBL_EPSILON);
 * the call then synchronises `stream`. */
int gfgpu_int_n_scalar_nt_dv_diag(const double* N, const double* vol, const double* qscalar,
                                  int64_t nelem, int32_t nne, int32_t nip, int32_t ndim,
                                  double* elemvec, int* is_diag, gfgpu_stream_t stream);
/* Int_gradN_dot_tensor2_dV (ElementQuad4.h:467-491; ElementHex8.h:355-383): -> elemvec. */
int gfgpu_int_grad_n_dot_tensor2_dv(const double* dNx, const double* vol, const double* qtensor,
                                    int64_t nelem, int32_t nne, int32_t nip, int32_t ndim,
                                    double* elemvec, gfgpu_stream_t stream);
/* Int_gradN_dot_tensor4_dot_gradNT_dV (Element.h:1132-1176): qtensor4 [nelem,nip,d,d,d,d]. */
int gfgpu_int_grad_n_dot_tensor4_dot_grad_nt_dv(const double* dNx, const double* vol,
                                                const double* qtensor4, int64_t nelem,
                                                int32_t nne, int32_t nip, int32_t ndim,
                                                double* elemmat, gfgpu_stream_t stream);

/* Element::Quad4::QuadraturePlanar (ElementQuad4Planar.h): Quad4 with 3x3 quadrature-point
 * tensors (plane strain) and an out-of-plane thickness.
 * compute_dN: ElementQuad4Planar.h:81-123, 280-318, vol = w det(J) thick. The gradients
 * (:130-221) write the in-plane block of a zero-filled qtensor [nelem,nip,3,3];
 * Int_gradN_dot_tensor2_dV (:254-277) reads the in-plane block of [nelem,nip,3,3];
 * Int_gradN_dot_tensor4_dot_gradNT_dV (Element.h:1132-1176) the in-plane indices of
 * [nelem,nip,3,3,3,3]. InterpQuad_vector, Int_N_vector_dV and Int_N_scalar_NT_dV are the Quad4
 * entry points (gfgpu_interp_quad_vector, ...) with this vol. Stress: gfgpu_elastic_stress with
 * ndim = 3 on the 3x3 strain gives the plane-strain stress including sigma_zz. */
int gfgpu_quad4_planar_compute_dN(const double* x, int64_t nelem, const double* xi,
                                  const double* w, int32_t nip, double thick, double* N,
                                  double* dNxi, double* dNx, double* vol, gfgpu_stream_t stream);
int gfgpu_grad_n_vector_planar(const double* dNx, const double* elemvec, int64_t nelem,
                               int32_t nip, double* qtensor, gfgpu_stream_t stream);
int gfgpu_grad_n_vector_T_planar(const double* dNx, const double* elemvec, int64_t nelem,
                                 int32_t nip, double* qtensor, gfgpu_stream_t stream);
int gfgpu_sym_grad_n_vector_planar(const double* dNx, const double* elemvec, int64_t nelem,
                                   int32_t nip, double* qtensor, gfgpu_stream_t stream);
int gfgpu_int_grad_n_dot_tensor2_dv_planar(const double* dNx, const double* vol,
                                           const double* qtensor, int64_t nelem, int32_t nip,
                                           double* elemvec, gfgpu_stream_t stream);
int gfgpu_int_grad_n_dot_tensor4_dot_grad_nt_dv_planar(const double* dNx, const double* vol,
                                                       const double* qtensor4, int64_t nelem,
                                                       int32_t nip, double* elemmat,
                                                       gfgpu_stream_t stream);

/* Linear elastic stress (external GMat in the reference; convention of
 * docs/theory/examples/cartesian_linear-elasticity.py:146-186): sigma = K tr(eps) I + 2G dev(eps)
 * with a 3-d trace (ndim=2: plane strain). K, G per element [nelem]. */
int gfgpu_elastic_stress(const double* eps, const double* K, const double* G, int64_t nelem,
                         int32_t nip, int32_t ndim, double* sig, gfgpu_stream_t stream);

/* ============================ Vector (device) ============================================= */

/* Vector::asElement nodevec -> elemvec (Vector.h:681-697). */
int gfgpu_as_element(const int32_t* conn, int64_t nelem, int32_t nne, int32_t ndim,
                     const double* nodevec, double* elemvec, gfgpu_stream_t stream);
/* Vector::asElement dofval -> elemvec (Vector.h:659-675). */
int gfgpu_as_element_dofval(const int32_t* conn, const int32_t* dofs, int64_t nelem, int32_t nne,
                            int32_t ndim, const double* dofval, double* elemvec,
                            gfgpu_stream_t stream);
/* Vector::asNode dofval -> nodevec (Vector.h:615-629). */
int gfgpu_as_node(const int32_t* dofs, int64_t nnode, int32_t ndim, const double* dofval,
                  double* nodevec, gfgpu_stream_t stream);
/* Vector::asDofs (Vector.h:569-608): the last writer of each dof wins, unwritten dofs are 0.
 * `last` [ndof] holds the flat source index of the last writer (or -1); it is the final entry of
 * each CSR segment (gfgpu_host_dof_csr / _nodevec), see gfgpu_csr_last. */
int gfgpu_as_dofs(const int32_t* last, int64_t ndof, const double* src, double* dofval,
                  gfgpu_stream_t stream);
/* last[d] = ptr[d+1] > ptr[d] ? idx[ptr[d+1]-1] : -1. */
int gfgpu_csr_last(const int32_t* ptr, const int32_t* idx, int64_t ndof, int32_t* last,
                   gfgpu_stream_t stream);
/* Vector::assembleDofs (Vector.h:703-741): dofval[d] = sum of src[idx[k]], k in the dof's CSR
 * segment, in ascending order from 0.0 (deterministic; the reference's serial order). */
int gfgpu_assemble_dofs(const int32_t* ptr, const int32_t* idx, int64_t ndof, const double* src,
                        double* dofval, gfgpu_stream_t stream);
/* Vector::assembleNode (Vector.h:747-757): AssembleDofs then asNode, fused (no dofval). */
int gfgpu_assemble_node(const int32_t* ptr, const int32_t* idx, const int32_t* dofs,
                        int64_t nnode, int32_t ndim, const double* elemvec, double* nodevec,
                        gfgpu_stream_t stream);

/* ============================ MatrixDiagonal (device) ===================================== */

/* Element::isDiagonal (Element.h:122-145): *is_diag (host int) = 1 if every off-diagonal
 * |entry| <= DBL_EPSILON. Synchronises `stream`. */
int gfgpu_is_diagonal(const double* elemmat, int64_t nelem, int32_t K, int* is_diag,
                      gfgpu_stream_t stream);
/* MatrixDiagonal::assemble (MatrixDiagonal.h:151-167) through the dof CSR of elemvec indices:
 * A[d] = sum of elemmat diagonal entries of the dof's incidences, in the reference's order.
 * For MatrixDiagonalPartitioned (MatrixDiagonalPartitioned.h:73-98) pass the CSR built on
 * `part`; A then holds [Auu, App] back to back. */
int gfgpu_diag_assemble(const int32_t* ptr, const int32_t* idx, int64_t ndof, int32_t nne,
                        int32_t ndim, const double* elemmat, double* A, gfgpu_stream_t stream);
/* MatrixDiagonal::factorize (MatrixDiagonal.h:268-280): inv = 1 / A, n entries. */
int gfgpu_diag_factorize(const double* A, int64_t n, double* inv, gfgpu_stream_t stream);
/* MatrixDiagonal::solve nodevec (MatrixDiagonal.h:237-250) and, with nnu < ndof and
 * `dofs` = part, MatrixDiagonalPartitioned::solve (MatrixDiagonalPartitioned.h:306-322):
 * x(m,i) = inv[dofs(m,i)] * b(m,i) where dofs(m,i) < nnu; other entries of x are untouched. */
int gfgpu_diag_solve_nodevec(const int32_t* dofs, int64_t nnode, int32_t ndim, int64_t nnu,
                             const double* inv, const double* b, double* x,
                             gfgpu_stream_t stream);
/* MatrixDiagonal::dot nodevec (MatrixDiagonal.h:213-222): b(m,i) = A[dofs(m,i)] * x(m,i). */
int gfgpu_diag_dot_nodevec(const int32_t* dofs, int64_t nnode, int32_t ndim, const double* A,
                           const double* x, double* b, gfgpu_stream_t stream);
/* MatrixDiagonalPartitioned::reaction nodevec (MatrixDiagonalPartitioned.h:378-392):
 * b(m,i) = App[part(m,i) - nnu] * x(m,i) where part(m,i) >= nnu. */
int gfgpu_diagp_reaction_nodevec(const int32_t* part, int64_t nnode, int32_t ndim, int64_t nnu,
                                 const double* App, const double* x, double* b,
                                 gfgpu_stream_t stream);
/* Element-wise dofval products: MatrixDiagonal::dot / solve dofval (MatrixDiagonal.h:224-259):
 * out[k] = a[k] * b[k]. */
int gfgpu_dofval_mul(const double* a, const double* b, int64_t n, double* out,
                     gfgpu_stream_t stream);

/* asTensor (Allocate.h asTensor / Element.h:215-246 QuadratureBase::AsTensor): out[i * k + j] =
 * src[i], e.g. a qscalar [nelem, nip] repeated into a qtensor [nelem, nip, tdim^rank]. */
int gfgpu_broadcast(const double* src, int64_t n, int64_t k, double* out, gfgpu_stream_t stream);
/* VectorPartitioned::dofsFromParitioned / nodeFromPartitioned (VectorPartitioned.h:276-365):
 * out[t] = idx[t] < nnu ? u[idx[t]] : p[idx[t] - nnu], n entries. For a dofval pass as `idx` the
 * position of every dof in [iiu, iip] (ndof entries); for a nodevec pass `part` [nnode, ndim].
 * The same gather with `idx` = iiu (or iip) and nnp = 0 is asDofs_u (asDofs_p) of a dofval
 * (VectorPartitioned.h:428-458, 549-579). */
int gfgpu_from_partitioned(const int32_t* idx, int64_t n, int64_t nnu, int64_t nnp,
                           const double* u, const double* p, double* out, gfgpu_stream_t stream);
/* VectorPartitioned::elementFromPartitioned (VectorPartitioned.h:376-418):
 * elemvec(e,m,i) = [u | p][part(conn(e,m), i)]. */
int gfgpu_from_partitioned_elemvec(const int32_t* conn, const int32_t* part, int64_t nelem,
                                   int32_t nne, int32_t ndim, int64_t nnu, int64_t nnp,
                                   const double* u, const double* p, double* elemvec,
                                   gfgpu_stream_t stream);
/* VectorPartitioned::copy_u / copy_p (VectorPartitioned.h:176-270): dest(m,i) = src(m,i) where
 * lo <= part(m,i) < hi (copy_u: [0, nnu); copy_p: [nnu, ndof)); other entries untouched. */
int gfgpu_copy_partitioned_nodevec(const int32_t* part, int64_t nnode, int32_t ndim, int64_t lo,
                                   int64_t hi, const double* src, double* dest,
                                   gfgpu_stream_t stream);

/* ============================ explicit velocity-Verlet (device) =========================== */

/* One or more increments of the explicit scheme of
 * docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:110-157 (three velocity estimates,
 * docs/examples/dynamics_inertia-damping.rst:6-66) on a linear elastic Quad4/Hex8 mesh:
 *   u += dt v + dt^2/2 a;  f = assembleNode(int_gradN_dot_tensor2_dV(sigma(symGradN(u))));
 *   3x { v = v_n + ...; fres = fext - f - eta v; a = M^-1 fres (free dofs only) }.
 * The force chain runs as two kernels per increment: an element kernel writing the element
 * forces to `fe` [nelem,nne,ndim] (caller-provided scratch), then a node kernel that gathers
 * them through the dof CSR (deterministic, the reference's order) and updates v, a and the next
 * displacement. */
typedef struct {
    int64_t nelem, nnode;
    int32_t nne, ndim, nip; /* Quad4: 4,2,4; Hex8: 8,3,8 (Gauss) */
    const int32_t* conn;    /* [nelem, nne] */
    const int32_t* dofs;    /* [nnode, ndim] Vector dofs (periodic ties allowed) */
    const int32_t* csr_ptr; /* [ndof+1] dof CSR over elemvec indices (gfgpu_host_dof_csr) */
    const int32_t* csr_idx; /* [nelem*nne*ndim] */
    const int32_t* part;    /* [nnode, ndim] solve numbering: free iff part < nnu */
    int64_t nnu;
    const double* inv;      /* [nnu] inverse lumped mass of the free dofs */
    const double* dNx;      /* [nelem, nip, nne, ndim] (general path) */
    const double* vol;      /* [nelem, nip] (general path) */
    const double* K;        /* [nelem] bulk modulus */
    const double* G;        /* [nelem] shear modulus */
    const double* fext;     /* [nnode, ndim] or NULL (= 0) */
    double dt, eta;
    /* uniform-geometry fast path (set by gfgpu_verlet_detect_uniform or by the caller):
     * all elements are congruent axis-aligned boxes of edge lengths hx, hy(, hz) with the
     * reference's Gauss quadrature; 0 = general per-Gauss-point path. */
    int32_t uniform;
    double hx, hy, hz;
    /* optional per-element coefficients of the uniform square Quad4 kernel [nelem, 4]
     * (gfgpu_verlet_precompute); NULL = derive them from K and G in every increment */
    const double* coef;
    /* optional lumped-mass classes (gfgpu_verlet_classify): per nodevec entry the index of its
     * inverse lumped mass in a short table (GFGPU_PRESCRIBED_CLASS for prescribed dofs), and that
     * table on the host; the fast node kernel then takes the three velocity estimates in closed
     * form with per-class coefficients. NULL = read inv per dof. */
    const uint8_t* mclass;     /* [nnode, ndim] device */
    const double* mclass_inv;  /* [ncls] host */
    int32_t ncls;
    /* Quad4 Mesh::Quad4::Regular(reg_nx, reg_ny) numbering with dofs = node * 2 + i, verified
     * on the device by gfgpu_verlet_detect_regular: the node kernel and the static solvers'
     * operator (gfgpu_pcg_*, gfgpu_fcg_*, gfgpu_coarse_setup) then find the <= 4 element forces of
     * a node by index arithmetic instead of the CSR (same summation order, same bits).
     * 0 = use the CSR. */
    int64_t reg_nx, reg_ny;
    /* Hex8 Mesh::Hex8::Regular(reg_nx, reg_ny, reg_nz) numbering with dofs = node * 3 + i,
     * verified by gfgpu_verlet_detect_regular_hex8: the static solvers' operator gathers a node's
     * <= 8 element forces by index arithmetic (same order and bits as the CSR). 0 = Quad4 or
     * CSR. */
    int64_t reg_nz;
    /* optional float-float ("pair") coefficients of a uniform square Quad4 mesh with the
     * Regular numbering and lumped-mass classes (gfgpu_verlet_precompute_pair): when set,
     * gfgpu_verlet_step in fast mode runs its increments in pair arithmetic (two FP32 numbers per
     * value, ~48-bit significands); NULL = FP64 kernels. */
    const float* coef_pair;
    /* which pair path coef_pair belongs to (set by gfgpu_verlet_precompute_pair): 1 = the Regular
     * square-element fused tile kernel, 2 = element kernel + dof-CSR node kernel with the square
     * closed form, 3 = the same with stored element stiffness matrices */
    int32_t pair_mode;
    /* optional float-float coefficients of the element operator with FP64 state
     * (gfgpu_pcg_precompute_pair) on a Regular cube Hex8 mesh (per element {lam.h, lam.l, G.h,
     * G.l}) or a uniform square Quad4 mesh ({L, N} pairs [nelem] then kH pairs [nelem]). When set,
     * the iterations of gfgpu_pcg_solve / gfgpu_pcg_iterate (and, on Quad4, of the flexible CG
     * gfgpu_fcg_*) apply the stiffness of their search directions in pair arithmetic (~48-bit
     * significands, ~1e-13 relative to the FP64 action); the solution, the residual, the
     * preconditioned residual, the direction and every dot product stay FP64, and the initial and
     * final (true) residuals use the FP64 operator. On a uniform square Quad4 mesh with coef_pair
     * NULL, gfgpu_verlet_step in fast mode also runs in "mixed" arithmetic: FP64 state, the element
     * forces from the pair closed form on node differences formed in FP64 and, with lumped-mass
     * classes, the three velocity estimates on pairs (v and a split from FP64, v' and a' returned to
     * FP64) and the predictor in FP64; without classes the FP64 node kernel. NULL = FP64 operator. */
    const float* pcg_pair;
    /* optional gather table of the node kernels (gfgpu_verlet_build_ell): for nodevec entry t the
     * flat elemvec indices of its dof's element contributions in the dof CSR's order,
     * ell[4 t + k], padded with -1 (at most 4 per dof: Quad4 meshes, periodic ties included).
     * When set and no Regular numbering applies, the class, pair and mixed node kernels read it
     * instead of dofs / csr_ptr / csr_idx: one dependent load of 16 bytes instead of three
     * levels (same order, same bits). NULL = the CSR. */
    const int32_t* ell;
} gfgpu_verlet_desc;

#define GFGPU_MASS_CLASSES 16
#define GFGPU_PRESCRIBED_CLASS 255

/* Bytes of scratch the step needs (the element-force buffer, or the pair state when
 * d->coef_pair is set), 256-byte aligned size. */
int64_t gfgpu_verlet_workspace_bytes(const gfgpu_verlet_desc* d);
/* Checks that dNx/vol describe congruent axis-aligned boxes with the Gauss rule, within `rtol`
 * relative to the largest |dNx| (vol: relative to the box volume): first on the host for the first
 * element (dNx_host [nip,nne,ndim], vol_host [nip], host copies), then for every element of the
 * device arrays d->dNx / d->vol on `stream` (stream-ordered scratch, one synchronisation). On
 * success sets d->uniform = 1 and d->hx, hy, hz. Returns GFGPU_OK either way (d->uniform tells). */
int gfgpu_verlet_detect_uniform(gfgpu_verlet_desc* d, const double* dNx_host,
                                const double* vol_host, double rtol, gfgpu_stream_t stream);
/* Uniform square Quad4 meshes: fill coef [nelem, 4] with the element coefficients that depend on
 * K and G only (lam/4, G/2, G/4, g^2 (lam + 3G)/4, lam = K - 2G/3); uniform cube Hex8 meshes:
 * coef [nelem, 8] with the folded mode coefficients (w0 d lam, w0 d G, 2 w0 d G, w1 d lam,
 * w1 d G, 2 w1 d G, 3 w1 d G, w2 d^2 (lam + 4G); d = 1/(4h), w* the Gauss weights of the
 * constant, linear and trilinear modes). Set d->coef = coef to use them. Returns
 * GFGPU_ERR_UNSUPPORTED for other meshes. */
int gfgpu_verlet_precompute(const gfgpu_verlet_desc* d, double* coef, gfgpu_stream_t stream);
/* FP64 <-> float-float ("pair") conversion of n values on `stream` (device pointers; out / in as
 * n pairs {h, l} of floats, 8-byte aligned), on the integer pipe: h = rn_f32(x), l = rn_f32(x - h),
 * the bits of the F64->F32 conversion instruction, for x = 0 and 2^-74 <= |x| < 2^128 (short of
 * h rounding up to infinity); below 2^-74 l = 0, below 2^-126 also h = +-0. Back: x = rn_f64(h + l)
 * with h and l converted exactly (subnormal floats as +-0). */
int gfgpu_pairs_from_f64(const double* x, int64_t n, float* out, gfgpu_stream_t stream);
int gfgpu_pairs_to_f64(const float* in, int64_t n, double* out, gfgpu_stream_t stream);
/* Floats of the pair coefficients gfgpu_verlet_precompute_pair writes for this descriptor (0 if no
 * pair path applies). */
int64_t gfgpu_verlet_pair_coef_floats(const gfgpu_verlet_desc* d);
/* Float-float ("pair") arithmetic for the increments of a Quad4 mesh: values are unevaluated sums
 * of two FP32 numbers (~48-bit significands, |values| within ~1e-30 .. 1e38), computed on the
 * FP32 pipes; each increment agrees with the FP64 kernels to ~1e-14 relative. Writes coef_pair
 * (gfgpu_verlet_pair_coef_floats floats, 16-byte aligned) and sets d->pair_mode; then
 * d->coef_pair = coef_pair makes gfgpu_verlet_step (fast mode) run on pairs. u, v, a are converted
 * to pairs at the start of a call (after the FP64 predictor) and back at its end. The path:
 *  1 = uniform square elements with the Regular numbering (gfgpu_verlet_detect_regular) and
 *      lumped-mass classes (gfgpu_verlet_classify): one fused tile kernel per increment.
 *      coef_pair: {L.h, L.l, N.h, N.l} per element (element order), then {kH.h, kH.l} in rows of
 *      nxp pairs (element (ex, ey) at ey * nxp + ex, nxp = nx rounded up to even, pad pairs 0),
 *      L = lam/4, N = G/4, kH = g^2 (lam + 3G)/4 split into high and low FP32 parts;
 *  2 = uniform square elements, any numbering (periodic ties allowed): element kernel (square
 *      closed form) + dof-CSR node kernel per increment; coef_pair: {L, N} per element, then kH
 *      per element;
 *  3 = any Quad4 mesh with the Gauss rule (d->dNx, d->vol): the element stiffness matrices
 *      times u_e + the dof-CSR node kernel; coef_pair: the 6 off-diagonal 2 x 2 node blocks of
 *      each K_e (24 pairs per element, [24][nelem]; the diagonal blocks follow from translation
 *      invariance, f_m = sum_{n != m} K_mn (u_n - u_m)).
 * In paths 2 and 3 without mass classes the pair inverse masses [nnu] follow. Other meshes return
 * GFGPU_ERR_UNSUPPORTED. Strict mode ignores coef_pair. */
int gfgpu_verlet_precompute_pair(gfgpu_verlet_desc* d, float* coef_pair, gfgpu_stream_t stream);
/* The pair path of gfgpu_verlet_step in three parts, for callers that act between increments
 * (the row-block partition's halo exchange, goosefem_gb300/partition.py). The state lives in
 * `workspace` (gfgpu_verlet_workspace_bytes with d->coef_pair set). Increments are numbered from 0
 * after begin; increment `it` reads the displacement buffer of parity it & 1 and, if it advances,
 * writes the predicted displacement of increment it + 1 into the other one.
 *  begin: u, v, a (FP64 nodevecs) -> pair state, with the FP64 predictor u + dt v + dt^2/2 a of
 *         increment 0 (main.cpp:119);
 *  increments: increments first .. first + count - 1; all advance except the last one unless
 *         advance_last (the last increment of a run leaves u as it read it, as gfgpu_verlet_step);
 *  end: the pair state -> u (the displacement increment `last` read), v, a;
 *  displacement: *ptr = the pair nodevec [nnode] of float4 {x.h, x.l, y.h, y.l} that increment
 *         `it` reads (host call, no GPU work): where a halo exchange writes rows of neighbours.
 * gfgpu_verlet_step(n) = begin, increments(0, n, 0), end(n - 1): the same bits. */
int gfgpu_verlet_pair_begin(const gfgpu_verlet_desc* d, const double* u, const double* v, const double* a,
                            void* workspace, gfgpu_stream_t stream);
int gfgpu_verlet_pair_increments(const gfgpu_verlet_desc* d, int64_t first, int64_t count, int32_t advance_last,
                                 void* workspace, gfgpu_stream_t stream);
int gfgpu_verlet_pair_end(const gfgpu_verlet_desc* d, int64_t last, double* u, double* v, double* a,
                          void* workspace, gfgpu_stream_t stream);
int gfgpu_verlet_pair_displacement(const gfgpu_verlet_desc* d, int64_t it, void* workspace, void** ptr);
/* Host set-up of the lumped-mass classes: reads part and inv back from the device, and if the
 * free dofs take at most GFGPU_MASS_CLASSES distinct inverse masses (a Regular mesh with uniform
 * density: interior, edge and corner values) writes mclass [nnode*ndim] (device, uint8) and
 * mclass_inv [GFGPU_MASS_CLASSES] (host) and sets d->mclass, d->mclass_inv, d->ncls; otherwise
 * returns GFGPU_ERR_UNSUPPORTED and leaves d unchanged. Synchronises. */
int gfgpu_verlet_classify(gfgpu_verlet_desc* d, uint8_t* mclass, double* mclass_inv,
                          gfgpu_stream_t stream);
/* Checks on the device that conn is MeshQuad4.h:87-126's Regular(nx, ny) connectivity and
 * dofs = arange(nnode * 2) (no periodic ties); on success sets d->reg_nx, d->reg_ny, else leaves
 * them 0. Needs only d's sizes, conn and dofs. Returns GFGPU_OK either way. Synchronises. */
int gfgpu_verlet_detect_regular(gfgpu_verlet_desc* d, int64_t nx, int64_t ny, gfgpu_stream_t stream);
/* Fill ell [nnode * ndim * 4] (16-byte aligned) from d->dofs, csr_ptr, csr_idx and set d->ell = ell
 * when every dof has at most 4 element contributions; else leave d->ell unchanged and return
 * GFGPU_ERR_UNSUPPORTED. Synchronises. */
int gfgpu_verlet_build_ell(gfgpu_verlet_desc* d, int32_t* ell, gfgpu_stream_t stream);
/* The same for MeshHex8.h:77-130's Regular(nx, ny, nz) connectivity with dofs = arange(nnode * 3):
 * sets d->reg_nx, reg_ny, reg_nz on success (used by the static solvers' gather; the explicit
 * step's node kernels are Quad4 only). Returns GFGPU_OK either way. Synchronises. */
int gfgpu_verlet_detect_regular_hex8(gfgpu_verlet_desc* d, int64_t nx, int64_t ny, int64_t nz,
                                     gfgpu_stream_t stream);
/* Advance nsteps increments; u, v, a are nodevec [nnode, ndim] device arrays updated in place.
 * Strict mode (gfgpu_set_strict) with the general path reproduces the reference's operation
 * order bit for bit; fast mode reassociates the lumped solve (a = inv R - (inv eta) v).
 * `workspace` is device memory of gfgpu_verlet_workspace_bytes(d). */
int gfgpu_verlet_step(const gfgpu_verlet_desc* d, double* u, double* v, double* a,
                      int64_t nsteps, void* workspace, gfgpu_stream_t stream);
/* Size of the built-in scratch of gfgpu_verlet_step_noalloc, in doubles (32 MiB). */
#define GFGPU_NOALLOC_FE_DOUBLES 4194304

/* The same increments as gfgpu_verlet_step, for callers that cannot allocate device memory:
 * host codes that reach the GPU only through this C ABI and have no CUDA runtime of their own
 * to call cudaMalloc with, or codes whose device memory is owned entirely by another allocator
 * or pool, where an extra allocation is not allowed or could fail in the middle of a run.
 * This entry point has no counterpart in the reference (GooseFEM allocates its temporaries on
 * the host); it allocates nothing: the element-force scratch is a file-scope device array of
 * GFGPU_NOALLOC_FE_DOUBLES values that every GPU loading the library keeps until the process
 * exits. Meshes with nelem * nne * ndim above that size are rejected with GFGPU_ERR_ARG.
 * The array's device address is looked up on the first call in each CUDA context (with the
 * device current; a context created after cudaDeviceReset, or a caller's own driver context, gets
 * its own lookup); make the first call in a context before any stream capture. This entry point
 * always runs the FP64 kernels (the pair path of d->coef_pair needs a workspace for its state) and
 * chooses the node kernel as gfgpu_verlet_step does: the two give the same bits for the same
 * descriptor without coef_pair. All calls share the one
 * array, which keeps the last call's element forces (every increment overwrites it completely
 * before reading it); calls whose work overlaps on the GPU (for example on two streams) race on
 * it. u, v, a as in gfgpu_verlet_step. */
int gfgpu_verlet_step_noalloc(const gfgpu_verlet_desc* d, double* u, double* v, double* a,
                              int64_t nsteps, gfgpu_stream_t stream);
/* Internal force only: fint (nodevec) = assembleNode(int_gradN_dot_tensor2_dV(sigma(u))), using
 * the same element kernel as the step. */
int gfgpu_internal_force(const gfgpu_verlet_desc* d, const double* u, double* fint,
                         void* workspace, gfgpu_stream_t stream);

/* Element forces only (the element kernel of the step): fe elemvec [nelem,nne,ndim] =
 * Int_gradN_dot_tensor2_dV(sigma(SymGradN_vector(asElement(u)))). */
int gfgpu_verlet_element_forces(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                gfgpu_stream_t stream);

/* Persistent variant of gfgpu_verlet_step for uniform Quad4 meshes (used for batches of many
 * independent meshes concatenated into one block-diagonal mesh): ONE cooperative launch runs the
 * predictor and all nsteps increments; the element and node phases are separated by a grid-wide
 * barrier whose waits give up after `timeout_cycles` SM clock cycles (the kernel then returns
 * and gfgpu_verlet_persistent_status reports GFGPU_ERR_TIMEOUT). `block` = 64, 128 or 256 threads,
 * `blocks_per_sm` <= 0 = as many as fit. Workspace: gfgpu_verlet_persistent_workspace_bytes. */
int64_t gfgpu_verlet_persistent_workspace_bytes(const gfgpu_verlet_desc* d);
int gfgpu_verlet_persistent(const gfgpu_verlet_desc* d, double* u, double* v, double* a,
                            int64_t nsteps, int32_t block, int32_t blocks_per_sm,
                            int64_t timeout_cycles, void* workspace, gfgpu_stream_t stream);
/* Synchronises `stream`, then *status = GFGPU_OK or GFGPU_ERR_TIMEOUT (a barrier gave up). */
int gfgpu_verlet_persistent_status(const gfgpu_verlet_desc* d, const void* workspace,
                                   int* status, gfgpu_stream_t stream);

/* CUDA graph of nsteps increments on fixed u, v, a, workspace addresses: mode 0 = the two kernels
 * per increment of gfgpu_verlet_step, mode 1 = the persistent launch. Replay with
 * gfgpu_graph_launch; release with gfgpu_graph_destroy. */
typedef void* gfgpu_graph_t;
int gfgpu_verlet_graph_create(const gfgpu_verlet_desc* d, double* u, double* v, double* a,
                              int64_t nsteps, int32_t mode, int32_t block, int32_t blocks_per_sm,
                              int64_t timeout_cycles, void* workspace, gfgpu_graph_t* graph);
int gfgpu_graph_launch(gfgpu_graph_t graph, gfgpu_stream_t stream);
int gfgpu_graph_destroy(gfgpu_graph_t graph);

/* Failure-detection self-test of the bounded grid barrier: a one-block launch waits for an
 * arrival that never comes; *status must come back GFGPU_ERR_TIMEOUT after about
 * `timeout_cycles` SM cycles, with the context still usable. Synchronises. */
int gfgpu_barrier_selftest(int64_t timeout_cycles, int* status);

/* ============================ static solve (device) ======================================= */

/* Matrix-free replacement of the partitioned direct solve (MatrixPartitioned.h:526-642,
 * MatrixPartitionedSolver::solve: A_uu x_u = b_u - A_up x_p with b_u = 0) for linear
 * elasticity: Jacobi-preconditioned CG in FP64 on the stiffness action of the element kernel.
 * The descriptor `d` is the one of the explicit step (dt, eta, inv, fext are ignored); `part`
 * and `nnu` mark the unknown dofs (part < nnu), all other dofs are prescribed. */
int64_t gfgpu_pcg_workspace_bytes(const gfgpu_verlet_desc* d);
/* Floats of the pair coefficients gfgpu_pcg_precompute_pair writes (4 per element on a Regular
 * cube Hex8 mesh with the index-arithmetic gather, gfgpu_verlet_detect_regular_hex8, and the FP64
 * cube coefficients d->coef; 6 per element on a uniform square Quad4 mesh with d->coef), or 0 when
 * the pair operator does not apply. */
int64_t gfgpu_pcg_pair_coef_floats(const gfgpu_verlet_desc* d);
/* Float-float operator of the static solvers' iterations: writes the pair coefficients into coef
 * (16-byte aligned, gfgpu_pcg_pair_coef_floats floats) and sets d->pcg_pair = coef. Hex8 cube:
 * {lam.h, lam.l, G.h, G.l} per element (lam = K - 2G/3); the direction update also writes the
 * direction as pairs, the cube closed form runs on pairs (the folded coefficients formed from lam
 * and G in registers), and the gather sums a dof's element forces as pairs and returns them to
 * FP64. Quad4 square: {L, N} and kH pairs (L = lam/4, N = G/4, kH = g^2 (lam + 3G)/4); the element
 * kernel splits the FP64 direction into pairs, runs the square closed form on pairs and joins its
 * forces to FP64 for the FP64 gathers. Returns GFGPU_ERR_UNSUPPORTED where
 * gfgpu_pcg_pair_coef_floats is 0. Set d->pcg_pair = NULL for the FP64 operator. */
int gfgpu_pcg_precompute_pair(gfgpu_verlet_desc* d, float* coef, gfgpu_stream_t stream);
/* Diagonal of the assembled stiffness as a nodevec (Jacobi preconditioner), from dNx/vol.
 * `workspace` needs nelem*nne*ndim doubles. */
int gfgpu_elastic_diagonal(const gfgpu_verlet_desc* d, double* diag, void* workspace,
                           gfgpu_stream_t stream);
/* Solve for the unknown dofs of the nodevec x (prescribed dofs hold the prescribed values and the
 * unknown dofs the initial guess on entry). Stops when ||r|| / ||b|| <= tol (checked every
 * `check_every` iterations on the host), then verifies the true residual b - A x. Synchronises.
 * Returns GFGPU_ERR_DIVERGED when maxiter is reached first. Deterministic: fixed-grid
 * reductions in a fixed order. */
int gfgpu_pcg_solve(const gfgpu_verlet_desc* d, const double* diag, double* x, double tol,
                    int64_t maxiter, int32_t check_every, void* workspace, gfgpu_stream_t stream,
                    int64_t* iters, double* relres);

/* Step-by-step Jacobi-PCG on the same workspace as gfgpu_pcg_solve (used to generate the
 * training pairs of the learned preconditioner): begin sets b = rhs_u - (A x_p)_u (rhs may be
 * NULL: no external load), r = b - (A x)_u, z = M^-1 r, p = z; iterate runs niter iterations
 * without convergence checks; vector returns a device pointer to r (which = 0), z (1), p (2) or
 * q = A p of the last iteration's direction (3) inside the workspace; norms synchronises and
 * returns r.r and b.b. */
int gfgpu_pcg_begin(const gfgpu_verlet_desc* d, const double* diag, const double* rhs,
                    const double* x, void* workspace, gfgpu_stream_t stream);
int gfgpu_pcg_iterate(const gfgpu_verlet_desc* d, int64_t niter, double* x, void* workspace,
                      gfgpu_stream_t stream);
int gfgpu_pcg_vector(const gfgpu_verlet_desc* d, void* workspace, int32_t which, double** ptr);
int gfgpu_pcg_norms(const gfgpu_verlet_desc* d, const void* workspace, double* rr, double* bb,
                    gfgpu_stream_t stream);

/* ============================ assembled sparse matrices ================================== */

/* Matrix / MatrixPartitioned (Matrix.h:653-863, MatrixPartitioned.h:34-460) as CSR.
 * Host set-up of the pattern: for the triplets pushed by Matrix::assemble_impl (Matrix.h:704-733;
 * dmap = dofs, n = ndof) or MatrixPartitioned::assemble_impl (MatrixPartitioned.h:156-200;
 * dmap = part, n = ndof, unknowns first: the blocks uu, up, pu, pp are index ranges of this one
 * matrix), rowptr [n+1] and col [nnz] (columns ascending per row) and, per nonzero k, the flat
 * elemmat indices cidx[cptr[k]:cptr[k+1]] that Eigen's setFromTriplets sums into it, in that
 * order. col, cidx: capacity nelem*K*K, cptr: nelem*K*K + 1 (K = nne*ndim); *nnz on return. */
int gfgpu_host_matrix_pattern(const int32_t* conn, const int32_t* dmap, int64_t nelem, int32_t nne,
                              int64_t nnode, int32_t ndim, int64_t n, int32_t* rowptr,
                              int32_t* col, int32_t* cptr, int32_t* cidx, int64_t* nnz);
/* assemble(elemmat): val[k] = sum of the listed elemmat entries (first, then +=, in order). */
int gfgpu_matrix_assemble(const int32_t* cptr, const int32_t* cidx, int64_t nnz,
                          const double* elemmat, double* val, gfgpu_stream_t stream);
/* Matrix::dot on dofval (Matrix.h:810-815): b = A x, per row from 0 in ascending columns. */
int gfgpu_matrix_dot_dofval(const int32_t* rowptr, const int32_t* col, const double* val, int64_t n,
                            const double* x, double* b, gfgpu_stream_t stream);
/* MatrixPartitioned::dot / reaction on dofval (MatrixPartitioned.h:378-398, 421-433) on the
 * partitioned CSR: per row (A_.u x_u) + (A_.p x_p); iperm [ndof]: original dof of partitioned
 * index (iiu then iip); x, b in the original numbering (must not alias). dot writes every entry
 * of b, reaction only the prescribed ones. */
int gfgpu_matrixp_dot_dofval(const int32_t* rowptr, const int32_t* col, const double* val,
                             int64_t ndof, int64_t nnu, const int32_t* iperm, const double* x,
                             double* b, gfgpu_stream_t stream);
int gfgpu_matrixp_reaction_dofval(const int32_t* rowptr, const int32_t* col, const double* val,
                                  int64_t ndof, int64_t nnu, const int32_t* iperm, const double* x,
                                  double* b, gfgpu_stream_t stream);
/* MatrixSolver::solve (Matrix.h:866-912; Eigen SimplicialLDLT there) for a symmetric matrix,
 * possibly indefinite: x = A^-1 b by MINRES (Paige & Saunders) with the preconditioner
 * diag(|A_ii|), from the initial guess in x, to ||b - A x|| <= tol ||b|| (true residual).
 * Deterministic. Synchronises. */
int64_t gfgpu_matrix_solve_workspace_bytes(int64_t n);
int gfgpu_matrix_solve(const int32_t* rowptr, const int32_t* col, const double* val, int64_t n,
                       const double* b, double* x, double tol, int64_t maxiter, int32_t check_every,
                       void* workspace, gfgpu_stream_t stream, int64_t* iters, double* relres);
/* The same solve of the partitioned system as gfgpu_matrixp_solve (below) by MINRES with the
 * preconditioner diag(|A_ii|): for symmetric A_uu that may be indefinite (the reference's
 * Eigen LDLT accepts those). */
int64_t gfgpu_matrixp_solve_minres_workspace_bytes(int64_t nnu);
int gfgpu_matrixp_solve_minres(const int32_t* rowptr, const int32_t* col, const double* val,
                               int64_t ndof, int64_t nnu, const int32_t* iperm, const double* b,
                               double* x, double tol, int64_t maxiter, int32_t check_every,
                               void* workspace, gfgpu_stream_t stream, int64_t* iters,
                               double* relres);
/* MatrixPartitionedSolver::solve (MatrixPartitioned.h:583-613; Eigen SimplicialLDLT there):
 * x_u = A_uu^-1 (b_u - A_up x_p) by Jacobi-PCG in FP64 to ||r|| <= tol ||b_u - A_up x_p||, from
 * the initial guess in x; b, x dofval in the original numbering (x_p read from x, x_u written).
 * check_every iterations replay as a CUDA graph. Deterministic. Synchronises. */
int64_t gfgpu_matrixp_solve_workspace_bytes(int64_t nnu);
int gfgpu_matrixp_solve(const int32_t* rowptr, const int32_t* col, const double* val, int64_t ndof,
                        int64_t nnu, const int32_t* iperm, const double* b, double* x, double tol,
                        int64_t maxiter, int32_t check_every, void* workspace,
                        gfgpu_stream_t stream, int64_t* iters, double* relres);

/* ============================ periodic tyings ============================================= */

/* Tyings::Periodic (TyingsPeriodic.h:46-344) set-up, host: iid = flatten(dofs[tyings[:,1]]),
 * iii = setdiff1d(dofs, iid), iiu = setdiff1d(iii, iip), and the renumbering
 * Reorder({iiu, iip, iid}) (Mesh.h:2384-2450) of dofs -> dofs_out [nnode, ndim] and of
 * control_dofs -> control_out [ndim, ndim]; counts = (nnu, nnp, nni, nnd). tyings [nties, 2] =
 * (independent node, dependent node). */
int gfgpu_host_tyings_periodic(const int32_t* dofs, int64_t nnode, int32_t ndim,
                               const int32_t* control_dofs, const int32_t* tyings, int64_t nties,
                               const int32_t* iip, int64_t nnp, int32_t* dofs_out,
                               int32_t* control_out, int64_t* counts);
/* Tyings::Periodic::Cdi (TyingsPeriodic.h:238-264) as CSR [nnd = nties*ndim rows, nni columns]
 * (Eigen setFromTriplets: equal columns summed in push order, columns sorted). Cdu and Cdp
 * (:272-344) are its column ranges [0, nnu) and [nnu, nni). col, val: capacity
 * nties*ndim*(ndim+1). tdofs / tcontrol: the renumbered tables. */
int gfgpu_host_tyings_cdi(const double* coor, const int32_t* tdofs, const int32_t* tcontrol,
                          const int32_t* tyings, int64_t nties, int32_t ndim, int32_t* rowptr,
                          int32_t* col, double* val, int64_t* nnz);
/* Transpose of a CSR (rows of the result sorted by the original row): C_id = Cdi^T. */
int gfgpu_host_csr_transpose(const int32_t* rowptr, const int32_t* col, const double* val,
                             int64_t nrow, int64_t ncol, int32_t* trowptr, int32_t* tcol,
                             double* tval);
/* VectorPartitionedTyings::asDofs_i (VectorPartitionedTyings.h:208-239): dofval_i [nni] = the
 * independent entries of nodevec, plus (apply_tyings) C_id times its dependent entries.
 * work_d: nnd doubles. */
int gfgpu_tyings_as_dofs_i(const int32_t* tdofs, int64_t nnode, int32_t ndim, int64_t nni,
                           int64_t nnd, const int32_t* cid_rowptr, const int32_t* cid_col,
                           const double* cid_val, const double* nodevec, int32_t apply_tyings,
                           double* dofval_i, double* work_d, gfgpu_stream_t stream);
/* MatrixPartitionedTyingsSolver::solve nodevec (MatrixPartitionedTyings.h, solve_nodevec_impl):
 * B_u += C_ud B_d; x_u = AC_uu^-1 (B_u - AC_up x_p) with AC = the condensed matrix
 * A_uu + A_ud C_du + C_ud A_du + C_ud A_dd C_du (factorize()); x_d = C_du x_u + C_dp x_p.
 * Here: Jacobi-PCG (exact condensed diagonal) in FP64 to tol, the condensed operator applied
 * from the blocks of the assembled CSR a_* (gfgpu_matrix_assemble with dmap = tdofs, n = ndof)
 * without forming it. b, x nodevec (x_p read from x, x_u and x_d written). Synchronises. */
int64_t gfgpu_tyings_solve_workspace_bytes(int64_t nnu, int64_t nnp, int64_t nnd);
int gfgpu_tyings_solve(const int32_t* a_rowptr, const int32_t* a_col, const double* a_val,
                       const int32_t* cdi_rowptr, const int32_t* cdi_col, const double* cdi_val,
                       const int32_t* cid_rowptr, const int32_t* cid_col, const double* cid_val,
                       const int32_t* tdofs, int64_t nnode, int32_t ndim, int64_t nnu, int64_t nnp,
                       int64_t nnd, const double* b, double* x, double tol, int64_t maxiter,
                       int32_t check_every, void* workspace, gfgpu_stream_t stream, int64_t* iters,
                       double* relres);

/* ============================ learned preconditioner (device) ============================= */

/* The network: 4 convolution layers 3x3 on the nodal grid of a Regular Quad4 mesh (NHWC, the
 * nodevec [nnode, 2] is the [H, W, 2] image), channels 4 -> 32 -> 32 -> 32 -> 2, dilations
 * 1, 2, 4, 1, ReLU after layers 1-3, zero padding. Input channels: the residual scaled by its
 * RMS over the free dofs, and two nodal material channels. Parameters in one flat array: per
 * layer W [9][cin][cout] then b [cout] (gfgpu_nn_param_offset); weights are used in BF16, biases
 * and all accumulations in FP32. */
typedef struct {
    const void* weights_bf16; /* [gfgpu_nn_param_count()] BF16 bit patterns */
    const float* params_f32;  /* [gfgpu_nn_param_count()] FP32 master copy (biases read here) */
    const float* material;    /* [H, W, 2] nodal material channels */
    int32_t H, W;             /* nodal grid: ny + 1 rows of nx + 1 nodes */
} gfgpu_nn_desc;

int32_t gfgpu_nn_param_count(void);
/* Host only: the unit square Quad4 element stiffness (2x2 Gauss, plane strain) per unit bulk
 * modulus (out[0:64]) and per unit shear modulus (out[64:128]), 8 x 8 row-major, dof a*2+i for
 * local node a = (0,0), (1,0), (1,1), (0,1) and component i; the energy-norm loss uses it. */
int gfgpu_nn_unit_element_stiffness(double* out);
int32_t gfgpu_nn_param_offset(int32_t layer, int32_t bias);
/* Training (CUDA cores, FP32 accumulate) on B crops of H x W nodes. */
int64_t gfgpu_nn_train_workspace_bytes(int32_t B, int32_t H, int32_t W);
int gfgpu_nn_forward(const void* weights_bf16, const float* params_f32, const float* X, int32_t B,
                     int32_t H, int32_t W, float* Y, void* workspace, gfgpu_stream_t stream);
/* Forward, loss over the crop interior [margin, S - margin)^2 against T, backward: grads (flat,
 * like the parameters) and *loss (device float). Deterministic. With E and F null the loss is
 * the mean-squared error; with E [B, S-1, S-1, 2] (element K, G of each crop; 0 outside the mesh)
 * and F [B, S, S, 2] (1 on free dofs, else 0) it is the energy norm: sum_b e_b^T A_b e_b over
 * sum_b t_b^T A_b t_b, e = M F (y - T), t = M F T, M the interior mask and A_b crop b's stiffness
 * (unit square Quad4 elements, 2x2 Gauss, plane strain). B <= 1024. */
int gfgpu_nn_train_step(const void* weights_bf16, const float* params_f32, const float* X,
                        const float* T, const float* E, const float* F, int32_t B, int32_t S,
                        int32_t margin, float* grads, float* loss, void* workspace,
                        gfgpu_stream_t stream);
/* Adam on the FP32 master parameters; rewrites the BF16 weights. */
int gfgpu_nn_adam(float* params, const float* grads, float* m, float* v, int32_t n, float lr,
                  float beta1, float beta2, float eps, int32_t step, void* weights_bf16,
                  gfgpu_stream_t stream);
/* Crops X [B, S, S, 4] (stored scaled residual + material) and targets T [B, S, S, 2] from
 * stored pairs R, Tg [npairs, H, W, 2]; pos [B, 3] = (pair, y0, x0). Optionally (non-null Ec /
 * Fc) the crops' element moduli Ec [B, S-1, S-1, 2] from elem_kg [(H-1)(W-1), 2] and free-dof
 * masks Fc [B, S, S, 2] from free_mask [H*W*2] (float 0 / 1), both 0 outside the mesh. */
int gfgpu_nn_gather_crops(const float* R, const float* T, const float* material,
                          const float* elem_kg, const float* free_mask, const int32_t* pos,
                          int32_t B, int32_t S, int32_t H, int32_t W, float* X, float* Tc,
                          float* Ec, float* Fc, gfgpu_stream_t stream);
/* Inference on one full grid: first and last layer on the CUDA cores, the two 32 -> 32 layers
 * on the tensor cores (mma.sync BF16, FP32 accumulate): X0 [H, W, 4] -> Y [H, W, 2];
 * workspace of gfgpu_nn_infer_workspace_bytes(H, W) bytes (256-byte aligned; X0 16-byte, Y
 * 8-byte aligned). */
int64_t gfgpu_nn_infer_workspace_bytes(int32_t H, int32_t W);
int gfgpu_nn_infer(const gfgpu_nn_desc* nn, const float* X0, float* Y, void* workspace,
                   gfgpu_stream_t stream);
/* Flexible CG in FP64 on the partitioned elastic system of gfgpu_pcg_solve (Notay's truncated
 * FCG). Every iteration takes ndir search directions, the Jacobi-preconditioned residual
 * D^-1 r and, with nn != NULL, the network's correction RMS(r) * net(r / RMS(r)) (prescribed
 * dofs 0); each is A-orthogonalised against the last nkeep directions of earlier iterations and
 * the earlier directions of the same iteration, and x, r take the exact line-search step along
 * each (the energy is minimised over their span). With nn == NULL and any nkeep >= 1 this is
 * Jacobi-PCG in exact arithmetic. Once the ring of directions is full the iterations replay as a
 * CUDA graph of check_every (rounded up to the ring period) iterations; the residual is checked
 * between replays. Same stopping rule and true-residual check as gfgpu_pcg_solve. ndir = 2 with
 * a network, else 1; nkeep + ndir <= 20. Synchronises. */
int64_t gfgpu_fcg_workspace_bytes(const gfgpu_verlet_desc* d, int32_t H, int32_t W, int32_t nkeep,
                                  int32_t ndir);
int gfgpu_fcg_solve(const gfgpu_verlet_desc* d, const double* diag, const gfgpu_nn_desc* nn,
                    double* x, double tol, int64_t maxiter, int32_t nkeep, int32_t check_every,
                    void* workspace, gfgpu_stream_t stream, int64_t* iters, double* relres);

/* ---- two-level correction (no counterpart in the reference; used with gfgpu_fcg_solve_coarse) */
/* Coarse space of a Regular Quad4 grid of nx x ny elements (node iy (nx + 1) + ix): bilinear
 * hats on every hc-th node along each axis (the last interval may be shorter), ncx x ncy coarse
 * nodes, two dofs each (coarse dof (jy ncx + jx) 2 + c), restricted to the free fine dofs.
 * `ainv` is the dense FP32 inverse of the Galerkin matrix P^T A_uu P, [nc, ld] (zero padded),
 * nc = 2 ncx ncy (at most 8192), filled by gfgpu_coarse_setup. */
typedef struct {
    int32_t nx, ny, hc, ncx, ncy;
    int32_t ld; /* row stride of ainv: nc rounded up to a multiple of 32 */
    const float* ainv;
    double rhx, rlx, rhy, rly; /* 1 / hc and 1 / (length of the last interval), along x and y */
} gfgpu_coarse_desc;
/* Fills nx, ny, hc, the coarse node counts, ld and the reciprocal interval lengths; ainv = NULL. */
int gfgpu_coarse_grid(int32_t nx, int32_t ny, int32_t hc, gfgpu_coarse_desc* g);
int64_t gfgpu_coarse_setup_workspace_bytes(const gfgpu_verlet_desc* d, const gfgpu_coarse_desc* g);
/* Measures A_c = P^T A_uu P with the matrix-free operator of `d` (18 coloured probes), writes it
 * to `ac` (FP64 [nc, nc], optional), inverts it in FP64 (Gauss-Jordan; A_c is SPD) and writes the
 * FP32 inverse to `ainv`. Synchronises `stream`. GFGPU_ERR_NAN for a singular coarse matrix. */
int gfgpu_coarse_setup(const gfgpu_verlet_desc* d, const gfgpu_coarse_desc* g, float* ainv,
                       double* ac, void* workspace, gfgpu_stream_t stream);
/* z = P ainv P^T r on the free dofs (0 on prescribed); r, z [nnode * 2]; workspace 2 x
 * 256-byte-rounded nc doubles. */
int gfgpu_coarse_apply(const gfgpu_verlet_desc* d, const gfgpu_coarse_desc* g, const double* r,
                       double* z, void* workspace, gfgpu_stream_t stream);
/* gfgpu_fcg_solve with the two-level first direction D^-1 r + P ainv P^T r and an optional
 * external load `rhs` [nnode * 2] (b = rhs_u - (A x_p)_u; NULL: no load). With `nn`, the second
 * direction is the network's correction of r (post = 0) or of the residual left after the step
 * along the first direction, r - alpha_0 A p_0 (post = 1: the network as a post-smoother of the
 * two-level step; no extra operator application). Workspace: gfgpu_fcg_coarse_workspace_bytes. */
int64_t gfgpu_fcg_coarse_workspace_bytes(const gfgpu_verlet_desc* d, int32_t H, int32_t W,
                                         int32_t nkeep, int32_t ndir, const gfgpu_coarse_desc* g);
int gfgpu_fcg_solve_coarse(const gfgpu_verlet_desc* d, const double* diag, const gfgpu_nn_desc* nn,
                           const gfgpu_coarse_desc* g, int32_t post, const double* rhs, double* x,
                           double tol, int64_t maxiter, int32_t nkeep,
                           int32_t check_every, void* workspace, gfgpu_stream_t stream,
                           int64_t* iters, double* relres);

/* ============================ probes ====================================================== */

/* FP64 FMA throughput probe: a kernel of independent DFMA chains, `blocks` x 256 threads,
 * `iters` iterations of 16 chains; writes a checksum to out[0]. 2*16*iters*blocks*256 flops. */
int gfgpu_probe_fp64(int64_t blocks, int64_t iters, double* out, gfgpu_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* GFGPU_H */
