// Config-1-style Poisson solve written against the C++ call surface of
// include/tsem_gpu.hpp, in the shape of TSEMLib's examples/poisson_mixBC/poisson.cpp:
// TSEM space, stiffness copy, rhs, Neumann and Dirichlet conditions, p-multigrid
// PCG, L2/H1 errors.
//
//   shim_poisson <mesh.bin> <p> <out.bin>
// mesh.bin: int32 nv, nt; double xyz[nv][3]; int32 tet[nt][4]; then int32 marks of
// vertices, edges and faces in the first-appearance numbering of Mesh::from_tets
// (nv, ne, nf values, each block preceded by its int32 length).  out.bin: int64 n,
// double x[n], double l2, double h1, int32 iterations.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "tsem_gpu.hpp"

namespace {
const double PI = 3.14159265358979323846;
double u(const double* p) { return std::sin(PI * p[0]) * std::sin(PI * p[1]) * std::sin(PI * p[2]) + p[0] * p[0]; }
double f(const double* p) {
    return 3 * PI * PI * std::sin(PI * p[0]) * std::sin(PI * p[1]) * std::sin(PI * p[2]) - 2;
}
void grad(const double* p, double* g) {
    const double sx = std::sin(PI * p[0]), sy = std::sin(PI * p[1]), sz = std::sin(PI * p[2]);
    g[0] = PI * std::cos(PI * p[0]) * sy * sz + 2 * p[0];
    g[1] = PI * sx * std::cos(PI * p[1]) * sz;
    g[2] = PI * sx * sy * std::cos(PI * p[2]);
}
double neumann(const double* p) {   // outward normal derivative on y = 0, 1 and z = 0, 1
    double g[3];
    grad(p, g);
    double out = 0;
    if (std::fabs(p[1]) < 1e-12) out = -g[1];
    if (std::fabs(p[1] - 1) < 1e-12) out = g[1];
    if (std::fabs(p[2]) < 1e-12) out = -g[2];
    if (std::fabs(p[2] - 1) < 1e-12) out = g[2];
    return out;
}
template <class T>
std::vector<T> read_block(std::ifstream& in) {
    int32_t n = 0;
    in.read(reinterpret_cast<char*>(&n), sizeof n);
    std::vector<T> v(n);
    in.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
    return v;
}
}  // namespace

int main(int argc, char** argv) {
    if (argc != 4) {
        std::cerr << "usage: shim_poisson mesh.bin p out.bin\n";
        return 2;
    }
    try {
        std::ifstream in(argv[1], std::ios::binary);
        int32_t nv = 0, nt = 0;
        in.read(reinterpret_cast<char*>(&nv), 4);
        in.read(reinterpret_cast<char*>(&nt), 4);
        std::vector<double> xyz((size_t)nv * 3);
        std::vector<int32_t> tets((size_t)nt * 4);
        in.read(reinterpret_cast<char*>(xyz.data()), (std::streamsize)(xyz.size() * 8));
        in.read(reinterpret_cast<char*>(tets.data()), (std::streamsize)(tets.size() * 4));
        tsem_gpu::Mesh mesh = tsem_gpu::Mesh::from_tets(xyz, tets);
        mesh.mark_v = read_block<int32_t>(in);
        mesh.mark_e = read_block<int32_t>(in);
        mesh.mark_f = read_block<int32_t>(in);
        if ((int)mesh.mark_e.size() != mesh.ne() || (int)mesh.mark_f.size() != mesh.nf()) {
            std::cerr << "mark arrays do not match the mesh topology\n";
            return 2;
        }
        const int M = std::atoi(argv[2]);

        tsem_gpu::TSEM tsem(M, M + 2, mesh);
        tsem_gpu::SparseMatrix sp_matrix(tsem.stiff_matrix);
        tsem_gpu::Vector rhs;
        tsem.calc_rhs(rhs, f);
        tsem.impose_boundary_condition(rhs, neumann, 2);
        tsem.impose_boundary_condition(sp_matrix, rhs, u, true, 1);

        tsem_gpu::TSEMSolver solver;
        solver.init_PMG(sp_matrix, M, tsem.calc_sum_dof(), 2, 0);
        tsem_gpu::Vector solution(tsem.n_dof_total, 0.0);
        solver.solve_PCG(sp_matrix, solution, rhs, 0.0, 1000, 4, 1, 2, 1e-12);
        const auto err = tsem.calc_errors(solution, u, grad);

        std::ofstream out(argv[3], std::ios::binary);
        const int64_t n = tsem.n_dof_total;
        out.write(reinterpret_cast<const char*>(&n), 8);
        out.write(reinterpret_cast<const char*>(solution.data()), (std::streamsize)(n * 8));
        out.write(reinterpret_cast<const char*>(&err.first), 8);
        out.write(reinterpret_cast<const char*>(&err.second), 8);
        const int32_t it = solver.last_stats.iterations;
        out.write(reinterpret_cast<const char*>(&it), 4);
        std::printf("n_dof %lld iterations %d l2 %.3e h1 %.3e\n", (long long)n, it, err.first, err.second);
    } catch (const tsem_gpu::Error& e) {
        std::cerr << "tsem error " << e.status << ": " << e.what() << "\n";
        return 1;
    }
    return 0;
}
