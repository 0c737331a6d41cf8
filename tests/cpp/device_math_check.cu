// Host-side check of the device helpers that compile for both sides: the
// lattice face-slot formula (simplic_device.cuh) and the FP32 cube
// fractions (cube_fraction_f32.cuh).  Driven by tests/test_device_math.py.
//
//   device_math_check slots NX NY NZ   -> "c x0 y0 ... x5 y5" per interior cell
//   device_math_check cube             -> "m1 m2 m3 a F dF inv(F)" per case
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "cube_fraction_f32.cuh"
#include "simplic_device.cuh"

int main(int argc, char** argv) {
    if (argc >= 5 && !std::strcmp(argv[1], "slots")) {
        const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
        for (int c = 0; c < nx * ny * nz; ++c) {
            int2 sl[6];
            if (!simplic::latticeSlots(c, nx, ny, nz, sl)) continue;
            std::printf("%d", c);
            for (int q = 0; q < 6; ++q) std::printf(" %d %d", sl[q].x, sl[q].y);
            std::printf("\n");
        }
        return 0;
    }
    if (argc >= 2 && !std::strcmp(argv[1], "cube")) {
        const float normals[][3] = {{0.3f, 0.5f, 0.8f}, {1.f, 1.f, 1.f}, {0.1f, -0.2f, 0.97f},
                                    {-0.7f, 0.7f, 0.1f}, {0.f, 0.f, 1.f}, {0.05f, 0.9f, -0.4f}};
        for (const auto& n : normals) {
            simplic::CubeCoef c;
            float3 p;
            if (!simplic::cubeCoefficientsF(n[0], n[1], n[2], c, p)) return 1;
            for (int k = 0; k <= 40; ++k) {
                const float a = -0.05f + 1.1f * float(k) / 40.f;
                float dF;
                const float F = simplic::cubeFractionF(a, c, dF);
                const float inv = simplic::cubeInverseF(F, c);
                std::printf("%.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", c.m1, c.m2, c.m3, a, F, dF, inv);
            }
        }
        return 0;
    }
    return 2;
}
