// divByRecip (simplic_device.cuh) against CUDA's double division on the
// GPU: random operands over the whole exponent range, near-multiples of the
// divisor and the divisors of the step (dt, 1/dt, cell volumes of uniform
// meshes); with a second argument "prod", divOfProduct on quotients of
// products.  Prints "samples mismatches".  Driven by tests/test_device_math.py.
#include <cstdio>
#include <cstdlib>

#include "simplic_device.cuh"

__device__ unsigned long long xorshift(unsigned long long& s) {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
}

__global__ void kCheck(long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long s = seed ^ (0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1));
        xorshift(s);
        const unsigned long long r1 = xorshift(s), r2 = xorshift(s), r3 = xorshift(s);
        const int mode = int(r3 & 15);
        int ea = 150 + int((r3 >> 8) % 1800), eb = 150 + int((r3 >> 20) % 1800);
        if (mode == 0) ea = int((r3 >> 8) % 2047);
        if (mode == 1) eb = int((r3 >> 20) % 2047);
        if (mode == 4 || mode == 8) {  // tiny numerators: the lower edge of the fast range
            ea = 30 + int((r3 >> 8) % 70);
            eb = 950 + int((r3 >> 20) % 150);
        }
        if (mode == 5) ea = 1950 + int((r3 >> 8) % 40);
        if (mode == 6) {  // quotients at the lower edge
            eb = 1000 + int((r3 >> 20) % 900);
            ea = eb - 940 - int((r3 >> 8) % 40);
        }
        if (mode == 7) {  // quotients at the upper edge
            eb = 64 + int((r3 >> 20) % 900);
            ea = eb + 940 + int((r3 >> 8) % 40);
        }
        if (((r3 >> 40) & 63) == 0) ea = 0;  // zero or subnormal numerators
        const unsigned long long ma = ((r3 >> 46) & 1) && ea == 0 ? 0ull : (r1 & 0xfffffffffffffull);
        double a = __longlong_as_double((long long)((ma | ((unsigned long long)ea << 52)) | ((r1 >> 63) << 63)));
        double b = __longlong_as_double((long long)(((r2 & 0xfffffffffffffull) | ((unsigned long long)eb << 52))));
        if (mode == 2) {  // a near a multiple of b
            a = double((r3 >> 32) % 1000000) * b;
            a = __longlong_as_double(__double_as_longlong(a) + (long long)(r1 % 5) - 2);
        } else if (mode == 3) {  // the divisors of a step
            const double ds[4] = {1.0 / 3808.0, 3808.0, 5.9604644775390625e-08, 0.0001234};
            b = ds[(r3 >> 40) & 3];
        }
        if (b == 0.0 || !isfinite(b)) continue;
        const double want = a / b, got = simplic::divByRecip(a, b, 1.0 / b);
        if (__double_as_longlong(want) != __double_as_longlong(got) && !(want != want && got != got)) ++local;
    }
    if (local) atomicAdd(bad, local);
}

// divOfProduct(RN(x dt), dt, 1/dt, x) against CUDA's division
__global__ void kCheckProd(long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long s = seed ^ (0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1));
        xorshift(s);
        const unsigned long long r1 = xorshift(s), r2 = xorshift(s), r3 = xorshift(s);
        const int mode = int(r3 & 7);
        int ex = 100 + int((r3 >> 8) % 1850), et = 900 + int((r3 >> 20) % 250);
        unsigned long long mx = r1 & 0xfffffffffffffull, mt = r2 & 0xfffffffffffffull;
        if (mode == 1) mx = 0;
        if (mode == 2) mx = 0xfffffffffffffull;
        if (mode == 3) mt = 0;
        if (mode == 4) mt = 0xfffffffffffffull;
        if (mode == 5) ex = int((r3 >> 8) % 2047);
        if (mode == 6) et = 64 + int((r3 >> 20) % 1900);
        const double x = __longlong_as_double((long long)((mx | ((unsigned long long)ex << 52)) | ((r1 >> 63) << 63)));
        const double dt = __longlong_as_double((long long)(mt | ((unsigned long long)et << 52)));
        if (!isfinite(x) || dt == 0.0 || !isfinite(dt)) continue;
        const double dv = __dmul_rn(x, dt);
        const double want = dv / dt, got = simplic::divOfProduct(dv, dt, 1.0 / dt, x);
        if (__double_as_longlong(want) != __double_as_longlong(got) && !(want != want && got != got)) ++local;
    }
    if (local) atomicAdd(bad, local);
}

int main(int argc, char** argv) {
    const long long n = argc > 1 ? std::atoll(argv[1]) : (1ll << 28);
    const bool prod = argc > 2 && argv[2][0] == 'p';
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess) return 3;
    cudaMemset(bad, 0, sizeof(*bad));
    if (prod)
        kCheckProd<<<1024, 256>>>(n, 4242ull, bad);
    else
        kCheck<<<1024, 256>>>(n, 12345ull, bad);
    unsigned long long h = 0;
    if (cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 4;
    cudaFree(bad);
    std::printf("%lld %llu\n", n, h);
    return 0;
}
