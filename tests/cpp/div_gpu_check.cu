// divByRecip (simplic_device.cuh) against CUDA's double division on the
// GPU: random operands over the whole exponent range, near-multiples of the
// divisor and the divisors of the step (dt, 1/dt, cell volumes of uniform
// meshes).  Prints "samples mismatches".  Driven by tests/test_device_math.py.
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
        const int mode = int(r3 & 7);
        const int ea = mode == 0 ? int((r3 >> 8) % 2047) : 150 + int((r3 >> 8) % 1800);
        const int eb = mode == 1 ? int((r3 >> 20) % 2047) : 150 + int((r3 >> 20) % 1800);
        double a = __longlong_as_double((long long)(((r1 & 0xfffffffffffffull) | ((unsigned long long)ea << 52)) |
                                                    ((r1 >> 63) << 63)));
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

int main(int argc, char** argv) {
    const long long n = argc > 1 ? std::atoll(argv[1]) : (1ll << 28);
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess) return 3;
    cudaMemset(bad, 0, sizeof(*bad));
    kCheck<<<1024, 256>>>(n, 12345ull, bad);
    unsigned long long h = 0;
    if (cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 4;
    cudaFree(bad);
    std::printf("%lld %llu\n", n, h);
    return 0;
}
