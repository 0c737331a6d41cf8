// Drives the C++ facade (include/simplic_solveVofEqu.hpp) the way an
// OpenFOAM solver would: dictionary -> solveVofEqu -> reconstruct/advect.
//
//   facade_driver controls <fvSolution>          print the parsed controls
//   facade_driver run <dir> <fvSolution> <steps> run steps, write alpha.out
//
// <dir> holds raw little-endian arrays written by the test: sizes.i32
// (np, nf, nfi, nc), points, face_offsets, face_points, owner, neighbour,
// C, V, Cf, Sf, magSf, alpha0, phi, U, Ub, dt.f64.
#include <cstdio>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "simplic_solveVofEqu.hpp"

template <class T>
std::vector<T> readAll(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    std::vector<char> b((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    std::vector<T> v(b.size() / sizeof(T));
    std::memcpy(v.data(), b.data(), v.size() * sizeof(T));
    return v;
}

int main(int argc, char** argv) {
    try {
        const std::string mode = argc > 1 ? argv[1] : "";
        if (mode == "controls" && argc == 3) {
            const auto d = simplic::Dictionary::read(argv[2]).solverDict("alpha.water");
            const simplic_controls c = simplic::controlsFromDict(d);
            std::printf("%.17g %d %d %.17g %d %d %d\n", c.mixed_cell_tol, c.n_alpha_bounds, c.clip, c.snap_tol,
                        c.orientation_method, c.split_warped_face, c.precision);
            return 0;
        }
        if (mode != "run" || argc != 5) {
            std::fprintf(stderr, "usage: facade_driver controls <fvSolution> | run <dir> <fvSolution> <steps>\n");
            return 2;
        }
        const std::string dir = argv[2];
        auto sz = readAll<int32_t>(dir + "/sizes.i32");
        auto pts = readAll<double>(dir + "/points");
        auto fo = readAll<int32_t>(dir + "/face_offsets");
        auto fp = readAll<int32_t>(dir + "/face_points");
        auto own = readAll<int32_t>(dir + "/owner");
        auto nei = readAll<int32_t>(dir + "/neighbour");
        auto C = readAll<double>(dir + "/C");
        auto V = readAll<double>(dir + "/V");
        auto Cf = readAll<double>(dir + "/Cf");
        auto Sf = readAll<double>(dir + "/Sf");
        auto magSf = readAll<double>(dir + "/magSf");
        std::vector<double> alpha = readAll<double>(dir + "/alpha0");
        std::vector<double> phi = readAll<double>(dir + "/phi");
        std::vector<double> U = readAll<double>(dir + "/U");
        std::vector<double> Ub = readAll<double>(dir + "/Ub");
        const double dt = readAll<double>(dir + "/dt.f64").at(0);
        simplic_mesh_desc d{};
        d.n_points = sz[0];
        d.n_faces = sz[1];
        d.n_internal_faces = sz[2];
        d.n_cells = sz[3];
        d.points = pts.data();
        d.face_offsets = fo.data();
        d.face_points = fp.data();
        d.owner = own.data();
        d.neighbour = nei.data();
        d.cell_centres = C.data();
        d.cell_volumes = V.data();
        d.face_centres = Cf.data();
        d.face_areas = Sf.data();
        d.face_mag_areas = magSf.data();
        const auto dict = simplic::Dictionary::read(argv[3]).solverDict("alpha.water");
        simplic::solveVofEqu solver(d, alpha, phi, U, dict, &Ub);
        solver.setDeltaT(dt);
        const int steps = std::atoi(argv[4]);
        for (int s = 0; s < steps; ++s) {
            solver.reconstruct();
            solver.advect();
        }
        std::ofstream out(dir + "/alpha.out", std::ios::binary);
        out.write(reinterpret_cast<const char*>(alpha.data()), alpha.size() * sizeof(double));
        std::printf("ok %zu mixed %.6f s reconstruction %.6f s advection\n", solver.mixedCells().size(),
                    solver.reconstructionTime(), solver.advectionTime());
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
