// Drives the GooseFEM-compatible C++ interface (include/gfgpu/GooseFEM.hpp) through the 64x64
// Quad4 force chain and the lumped mass, the way a GooseFEM user program would
// (docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:32-86, 123-127):
//   Vector(conn, dofs); Quadrature(vector.AsElement(coor)); QuadraturePlanar(.., thick);
//   asElement; symGradN_vector;
//   stress; int_gradN_dot_tensor2_dV; assembleNode; MatrixDiagonal::assemble(Int_N_scalar_NT_dV).
// Usage: test_api <inputs.bin> <outputs.bin>
//   inputs:  nx (int64), K[nelem], G[nelem], u[nnode*2] (float64)
//   outputs: dNx, vol, ue, eps, sig, fe, fint, M, then the planar dV, eps, sig, fe, then the
//   static solution (float64, concatenated)
#include <algorithm>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "gfgpu/GooseFEM.hpp"

namespace GF = gfgpu;

static std::vector<double> read(std::ifstream& f, size_t n)
{
    std::vector<double> v(n);
    f.read(reinterpret_cast<char*>(v.data()), n * sizeof(double));
    return v;
}

template <class A>
static void dump(std::ofstream& o, const A& a)
{
    auto h = a.to_host();
    o.write(reinterpret_cast<const char*>(h.data()), h.size() * sizeof(double));
}

int main(int argc, char** argv)
{
    if (argc < 3) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    int64_t nx = 0;
    in.read(reinterpret_cast<char*>(&nx), sizeof(nx));
    GF::Mesh::Quad4::Regular mesh(nx, nx);
    int64_t nelem = mesh.nelem(), nnode = mesh.nnode();
    auto K = read(in, nelem), G = read(in, nelem), uh = read(in, nnode * 2);

    try {
        GF::Vector vector(mesh.conn(), mesh.dofs());
        GF::Element::Quad4::Quadrature quad(vector.AsElement(GF::array<double>::from_host(mesh.coor())));
        auto u = GF::array<double>::from_host(uh.data(), {nnode, 2});
        auto Kd = GF::array<double>::from_host(K.data(), {nelem});
        auto Gd = GF::array<double>::from_host(G.data(), {nelem});

        auto ue = vector.allocate_elemvec();
        auto Eps = GF::array<double>(quad.shape_qtensor2());
        auto Sig = GF::array<double>(quad.shape_qtensor2());
        auto fe = vector.allocate_elemvec();
        auto fint = vector.allocate_nodevec();
        vector.asElement(u, ue);
        quad.symGradN_vector(ue, Eps);
        GF::check(gfgpu_elastic_stress(Eps.data(), Kd.data(), Gd.data(), nelem, quad.nip(), 2,
                                       Sig.data(), nullptr),
                  "stress");
        quad.int_gradN_dot_tensor2_dV(Sig, fe);
        vector.assembleNode(fe, fint);

        GF::Element::Quad4::Quadrature nodal(vector.AsElement(GF::array<double>::from_host(mesh.coor())),
                                             GF::Element::Quad4::Nodal::xi(),
                                             GF::Element::Quad4::Nodal::w());
        GF::host::array<double> rho({nelem, 4}, 1.0);
        GF::MatrixDiagonal M(mesh.conn(), mesh.dofs());
        M.assemble(nodal.Int_N_scalar_NT_dV(GF::array<double>::from_host(rho)));

        // QuadraturePlanar: 3x3 tensors, thickness 2
        GF::Element::Quad4::QuadraturePlanar planar(
            vector.AsElement(GF::array<double>::from_host(mesh.coor())), 2.0);
        if (planar.tdim() != 3) return 4;
        auto Eps3 = planar.SymGradN_vector(ue);
        auto Sig3 = GF::array<double>(planar.shape_qtensor2());
        GF::check(gfgpu_elastic_stress(Eps3.data(), Kd.data(), Gd.data(), nelem, planar.nip(), 3,
                                       Sig3.data(), nullptr),
                  "stress");
        auto fe3 = planar.Int_gradN_dot_tensor2_dV(Sig3);

        // static solve with the assembled stiffness: bottom edge fixed, top edge uy = -0.01
        // (MatrixPartitioned + MatrixPartitionedSolver, the pattern of
        // docs/examples/statics/FixedDisplacements_LinearElastic)
        GF::host::array<double> C4({nelem, 4, 2, 2, 2, 2});
        for (int64_t e = 0; e < nelem; ++e)
            for (int q = 0; q < 4; ++q)
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j)
                        for (int k = 0; k < 2; ++k)
                            for (int l = 0; l < 2; ++l) {
                                double dij = i == j, dkl = k == l, dik = i == k, djl = j == l,
                                       dil = i == l, djk = j == k;
                                C4[((((e * 4 + q) * 2 + i) * 2 + j) * 2 + k) * 2 + l] =
                                    K[e] * dij * dkl + G[e] * (dik * djl + dil * djk - 2.0 / 3.0 * dij * dkl);
                            }
        auto Ke = quad.Int_gradN_dot_tensor4_dot_gradNT_dV(GF::array<double>::from_host(C4));
        auto bot = mesh.nodesBottomEdge(), top = mesh.nodesTopEdge();
        GF::host::array<int32_t> iip({bot.size() * 2 + top.size()});
        std::vector<int32_t> ip;
        for (int64_t i = 0; i < bot.size(); ++i) {
            ip.push_back(bot[i] * 2);
            ip.push_back(bot[i] * 2 + 1);
        }
        for (int64_t i = 0; i < top.size(); ++i) ip.push_back(top[i] * 2 + 1);
        std::sort(ip.begin(), ip.end());
        for (size_t i = 0; i < ip.size(); ++i) iip[int64_t(i)] = ip[i];
        GF::MatrixPartitioned Kmat(mesh.conn(), mesh.dofs(), iip);
        Kmat.assemble(Ke);
        GF::host::array<double> xh({nnode, 2}, 0.0);
        for (int64_t i = 0; i < top.size(); ++i) xh(top[i], 1) = -0.01;
        auto xs = GF::array<double>::from_host(xh);
        GF::MatrixPartitionedSolver solver(1e-12);
        auto zero = GF::array<double>({nnode, 2});
        zero.fill_zero();
        solver.solve(Kmat, zero, xs);
        if (solver.relres() > 1e-12) return 5;

        // VectorPartitioned (tests/basic/VectorPartitioned.cpp "asDofs" and "copy_u, copy_p"):
        // right open edge tied to the left one, top and bottom edges prescribed
        auto dofs_lr = mesh.dofs();
        auto left = mesh.nodesLeftOpenEdge(), right = mesh.nodesRightOpenEdge();
        for (int64_t i = 0; i < left.size(); ++i)
            for (int d = 0; d < 2; ++d) dofs_lr(right[i], d) = dofs_lr(left[i], d);
        dofs_lr = GF::Mesh::renumber(dofs_lr);
        GF::host::array<int32_t> iip_lr({(bot.size() + top.size()) * 2});
        int64_t c = 0;
        for (int d = 0; d < 2; ++d)
            for (int64_t i = 0; i < top.size(); ++i) iip_lr[c++] = dofs_lr(top[i], d);
        for (int d = 0; d < 2; ++d)
            for (int64_t i = 0; i < bot.size(); ++i) iip_lr[c++] = dofs_lr(bot[i], d);
        auto uh2 = uh;
        for (int64_t i = 0; i < left.size(); ++i)
            for (int d = 0; d < 2; ++d) uh2[right[i] * 2 + d] = uh2[left[i] * 2 + d];
        auto u2 = GF::array<double>::from_host(uh2.data(), {nnode, 2});
        GF::VectorPartitioned vp(mesh.conn(), dofs_lr, iip_lr);
        auto isp = vp.dofs_is_p();
        int64_t np = 0;
        for (int64_t i = 0; i < isp.size(); ++i) np += isp[i];
        if (np != int64_t(top.size() + bot.size()) * 2) return 6;
        auto u_u = vp.AsDofs_u(u2), u_p = vp.AsDofs_p(u2);
        auto u2_back = vp.NodeFromPartitioned(u_u, u_p);
        auto v = GF::array<double>({nnode, 2});
        v.fill_zero();
        vp.copy_u(u2, v);
        vp.copy_p(u2, v);

        // MatrixDiagonalPartitioned with the lumped mass and the static solve's iip
        GF::MatrixDiagonalPartitioned Mp(mesh.conn(), mesh.dofs(), iip);
        Mp.assemble(nodal.Int_N_scalar_NT_dV(GF::array<double>::from_host(rho)));
        auto Mp_dot = Mp.Dot(u);
        auto Mp_solve = Mp.Solve(u, zero);
        auto Mp_reaction = Mp.Reaction(u, zero);

        std::ofstream out(argv[2], std::ios::binary);
        dump(out, quad.GradN());
        dump(out, quad.dV());
        dump(out, ue);
        dump(out, Eps);
        dump(out, Sig);
        dump(out, fe);
        dump(out, fint);
        dump(out, M.data());
        dump(out, planar.dV());
        dump(out, Eps3);
        dump(out, Sig3);
        dump(out, fe3);
        dump(out, xs);
        dump(out, u2_back);
        dump(out, v);
        dump(out, Mp_dot);
        dump(out, Mp_solve);
        dump(out, Mp_reaction);

        // error path: a shape mismatch is reported as std::runtime_error
        bool threw = false;
        try {
            auto bad = GF::array<double>({3, 3});
            vector.asElement(u, bad);
        }
        catch (const std::runtime_error&) {
            threw = true;
        }
        if (!threw) return 3;
    }
    catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    std::cout << "ok" << std::endl;
    return 0;
}
