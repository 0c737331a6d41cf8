// Host-side check of the device helpers that compile for both sides: the
// lattice face-slot formula (simplic_device.cuh) and the FP32 cube
// fractions (cube_fraction_f32.cuh).  Driven by tests/test_device_math.py.
//
//   device_math_check slots NX NY NZ   -> "c x0 y0 ... x5 y5" per interior cell
//   device_math_check cube             -> "m1 m2 m3 a F dF inv(F)" per case
//   device_math_check angle N SEED     -> "y x planeAngle(y, x)" as hex bit patterns
//   device_math_check fdiv N SEED      -> "samples mismatches" of fastDivide
#include <cmath>
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
    if (argc >= 4 && !std::strcmp(argv[1], "angle")) {
        // planeAngle on random (y, x) pairs: "y x angle" as bit patterns
        const long long n = std::atoll(argv[2]);
        unsigned long long s = std::strtoull(argv[3], nullptr, 10) * 0x9E3779B97F4A7C15ull + 1;
        for (long long i = 0; i < n; ++i) {
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            const double y = double((long long)(s >> 11) - (1ll << 52)) * std::ldexp(1.0, -52 + int(s & 7) * 4 - 12);
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            const double x = double((long long)(s >> 11) - (1ll << 52)) * std::ldexp(1.0, -52 + int(s & 7) * 4 - 12);
            const double a = simplic::planeAngle(y, x);
            unsigned long long by, bx, ba;
            std::memcpy(&by, &y, 8);
            std::memcpy(&bx, &x, 8);
            std::memcpy(&ba, &a, 8);
            std::printf("%llx %llx %llx\n", by, bx, ba);
        }
        return 0;
    }
    if (argc >= 4 && !std::strcmp(argv[1], "fdiv")) {
        // fastDivide against the integer division: every divisor 2..4096 and
        // the lattice layer sizes up to 2048^2 with random and edge
        // numerators; prints "samples mismatches"
        const long long n = std::atoll(argv[2]);
        unsigned long long s = std::strtoull(argv[3], nullptr, 10) * 0x9E3779B97F4A7C15ull + 3;
        auto next = [&s]() {
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            return s;
        };
        long long bad = 0, cnt = 0;
        auto check = [&](uint32_t num, uint32_t d, const simplic::FastDiv& f) {
            ++cnt;
            if (simplic::fastDivide(num, f) != num / d) ++bad;
        };
        for (uint32_t d = 2; d <= 4096; ++d) {
            const simplic::FastDiv f = simplic::makeFastDiv(d);
            for (uint32_t q = 0; q < 64; ++q) {  // around multiples of d
                const unsigned long long base = (unsigned long long)(next() % (0x7fffffffull / d)) * d;
                for (int e = -1; e <= 1; ++e)
                    if ((long long)base + e >= 0 && base + e <= 0x7fffffffull) check(uint32_t(base + e), d, f);
            }
            for (long long i = 0; i < n / 4096; ++i) check(uint32_t(next() & 0x7fffffffu), d, f);
            check(0u, d, f);
            check(0x7fffffffu, d, f);
            check(0xffffffffu, d, f);
        }
        for (uint32_t nx = 3; nx <= 2048; nx += 7) {
            const uint32_t d = nx * nx;
            const simplic::FastDiv f = simplic::makeFastDiv(d);
            for (long long i = 0; i < 256; ++i) check(uint32_t(next() & 0x7fffffffu), d, f);
            check(d - 1, d, f);
            check(d, d, f);
            check(d * 7 + d - 1, d, f);
        }
        std::printf("%lld %lld\n", cnt, bad);
        return 0;
    }
    if (argc >= 4 && !std::strcmp(argv[1], "qprod")) {
        // divOfProduct(RN(x dt), dt, 1/dt, x) against IEEE division, x and
        // dt random over wide exponent ranges (and near powers of two and
        // all-ones significands); prints "samples mismatches"
        const long long n = std::atoll(argv[2]);
        unsigned long long s = std::strtoull(argv[3], nullptr, 10) * 0x9E3779B97F4A7C15ull + 7;
        auto next = [&s]() {
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            return s;
        };
        long long bad = 0;
        for (long long i = 0; i < n; ++i) {
            const unsigned long long r1 = next(), r2 = next(), r3 = next();
            const int mode = int(r3 & 7);
            int ex = 100 + int((r3 >> 8) % 1850), et = 900 + int((r3 >> 20) % 250);
            unsigned long long mx = r1 & 0xfffffffffffffull, mt = r2 & 0xfffffffffffffull;
            if (mode == 1) mx = 0;                      // x a power of two
            if (mode == 2) mx = 0xfffffffffffffull;     // all-ones significand
            if (mode == 3) mt = 0;                      // dt a power of two
            if (mode == 4) mt = 0xfffffffffffffull;
            if (mode == 5) ex = int((r3 >> 8) % 2047);  // any x
            if (mode == 6) et = 64 + int((r3 >> 20) % 1900);
            const unsigned long long ux = (mx | (static_cast<unsigned long long>(ex) << 52)) | ((r1 >> 63) << 63);
            const unsigned long long ut = mt | (static_cast<unsigned long long>(et) << 52);
            double x, dt;
            std::memcpy(&x, &ux, 8);
            std::memcpy(&dt, &ut, 8);
            if (!std::isfinite(x) || dt == 0.0 || !std::isfinite(dt)) continue;
            const double dv = x * dt;
            const double want = dv / dt, got = simplic::divOfProduct(dv, dt, 1.0 / dt, x);
            unsigned long long w, g;
            std::memcpy(&w, &want, 8);
            std::memcpy(&g, &got, 8);
            if (w != g && !(want != want && got != got)) ++bad;
        }
        std::printf("%lld %lld\n", n, bad);
        return 0;
    }
    if (argc >= 4 && !std::strcmp(argv[1], "div")) {
        // divByRecip against IEEE division: random operands over the whole
        // exponent range (and near the fallback edges), divisor reciprocal
        // y = 1/b; prints the samples and the mismatches
        const long long n = std::atoll(argv[2]);
        unsigned long long s = std::strtoull(argv[3], nullptr, 10) * 0x9E3779B97F4A7C15ull + 1;
        auto next = [&s]() {
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            return s;
        };
        long long bad = 0;
        for (long long i = 0; i < n; ++i) {
            const unsigned long long r1 = next(), r2 = next(), r3 = next();
            // exponents: uniform over the range, in the middle, or at the
            // edges of the fast range (a, and the quotient's exponent)
            const int mode = int(r3 & 7);
            int ea = 150 + int((r3 >> 8) % 1800), eb = 150 + int((r3 >> 20) % 1800);
            if (mode == 0) ea = int(r3 >> 8) % 2047;
            if (mode == 1) eb = int(r3 >> 20) % 2047;
            if (mode == 4) {
                ea = 30 + int((r3 >> 8) % 70);
                eb = 950 + int((r3 >> 20) % 150);
            }
            if (mode == 5) ea = 1950 + int((r3 >> 8) % 40);
            if (mode == 6) {
                eb = 1000 + int((r3 >> 20) % 900);
                ea = eb - 940 - int((r3 >> 8) % 40);
            }
            if (mode == 7) {
                eb = 64 + int((r3 >> 20) % 900);
                ea = eb + 940 + int((r3 >> 8) % 40);
            }
            if (((r3 >> 40) & 63) == 0) ea = 0;  // zero or subnormal numerators
            const unsigned long long ma = ((r3 >> 46) & 1) && ea == 0 ? 0 : (r1 & 0xfffffffffffffull);
            const unsigned long long mb = r2 & 0xfffffffffffffull;
            const unsigned long long ua = (ma | (static_cast<unsigned long long>(ea) << 52)) | ((r1 >> 63) << 63);
            const unsigned long long ub = (mb | (static_cast<unsigned long long>(eb) << 52)) | ((r2 >> 63) << 63);
            double a, b;
            std::memcpy(&a, &ua, 8);
            std::memcpy(&b, &ub, 8);
            if (b == 0.0 || !std::isfinite(b)) continue;
            const double want = a / b, got = simplic::divByRecip(a, b, 1.0 / b);
            unsigned long long w, g;
            std::memcpy(&w, &want, 8);
            std::memcpy(&g, &got, 8);
            if (w != g && !(want != want && got != got)) ++bad;
        }
        std::printf("%lld %lld\n", n, bad);
        return 0;
    }
    return 2;
}
