// kd_generate.cu -- initial conditions generated on the device, straight into a context's
// bodies (no host arrays, no host-to-device copy).
//
// Workloads:
//   ring      body 0: mass 1 at rest at the origin; bodies 1..n-1: mass 1e-14,
//             r ~ U[0.8, 1.2], phi ~ U[0, 2 pi), z ~ Normal(0, 1e-4), circular speed
//             sqrt(1/r) of G = 1 around the central mass;
//   plummer   G = 1, total mass 1, scale radius 1, equal masses: radii by the inverse
//             cumulative mass profile r = (U^(-2/3) - 1)^(-1/2), redrawn above 20; isotropic
//             directions; speeds q v_esc(r) with q by von Neumann rejection from
//             q^2 (1 - q^2)^(7/2) (Aarseth, Henon & Wielen 1974); centre of mass moved to rest
//             at the origin;
//   circular  the reference's circular_orbits(n-1) (array_particle.rs:19-44): a unit mass
//             at the origin and body i+1 at d = 0.1 + 5 i/(n-1) with angle U[0, 6.28).
// Random numbers: every body draws from its own counter-based stream (splitmix64 of seed,
// body index and draw number), so the result depends on (n, seed) only.
#include <math.h>

#include "kd_internal.cuh"

namespace kd {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// uniform double in [0, 1): draw k of body i
__device__ __forceinline__ double uni(uint64_t seed, uint64_t i, uint64_t k) {
    const uint64_t z = mix64(seed * 0x9E3779B97F4A7C15ull + mix64(i * 0xD1B54A32D192ED03ull + k));
    return (double)(z >> 11) * 0x1.0p-53;
}

__device__ __forceinline__ void put(Bodies b, uint32_t i, double x, double y, double z,
                                    double vx, double vy, double vz, double r, double m) {
    b.x[i] = x; b.y[i] = y; b.z[i] = z;
    b.vx[i] = vx; b.vy[i] = vy; b.vz[i] = vz;
    b.r[i] = r; b.m[i] = m;
}

__global__ void k_gen_ring(Bodies b, uint32_t n, uint64_t seed) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (i == 0) {
            put(b, 0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.00465047, 1.0);
            continue;
        }
        const double r = 0.8 + 0.4 * uni(seed, i, 0);
        const double phi = 2.0 * M_PI * uni(seed, i, 1);
        // Box-Muller: one normal deviate from two uniforms
        const double u3 = 1.0 - uni(seed, i, 2), u4 = uni(seed, i, 3);
        const double z = 1e-4 * sqrt(-2.0 * log(u3)) * cos(2.0 * M_PI * u4);
        const double v = sqrt(1.0 / r);
        double s, c;
        sincos(phi, &s, &c);
        put(b, i, r * c, r * s, z, -v * s, v * c, 0.0, 1e-7, 1e-14);
    }
}

__global__ void k_gen_circular(Bodies b, uint32_t n, uint64_t seed) {
    const uint32_t k = n - 1;  // circular_orbits(k) returns k + 1 bodies
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (i == 0) {
            put(b, 0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.00465047, 1.0);
            continue;
        }
        const double d = 0.1 + ((double)(i - 1) * 5.0 / (double)k);
        const double v = sqrt(1.0 / d);
        const double th = uni(seed, i, 0) * 6.28;
        double s, c;
        sincos(th, &s, &c);
        put(b, i, d * c, d * s, 0.0, -v * s, v * c, 0.0, 1e-7, 1e-14);
    }
}

__device__ __forceinline__ void iso(uint64_t seed, uint64_t i, uint64_t k, double &x, double &y,
                                    double &z) {
    const double ct = 2.0 * uni(seed, i, k) - 1.0;
    const double ph = 2.0 * M_PI * uni(seed, i, k + 1);
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    double s, c;
    sincos(ph, &s, &c);
    x = st * c;
    y = st * s;
    z = ct;
}

// Rejection loops are bounded (64 draws); the acceptance rates are 99.6 % (radius) and about
// 50 % (speed), so the fallback values are never reached in practice.
__global__ void k_gen_plummer(Bodies b, uint32_t n, uint64_t seed) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r = 1.0;
        for (int t = 0; t < 64; ++t) {
            const double u = uni(seed, i, (uint64_t)t);
            if (u <= 0.0) continue;
            const double rr = 1.0 / sqrt(pow(u, -2.0 / 3.0) - 1.0);
            if (rr <= 20.0) {
                r = rr;
                break;
            }
        }
        double q = 0.5;
        for (int t = 0; t < 64; ++t) {
            const double x = uni(seed, i, 100 + 2 * (uint64_t)t);
            const double y = 0.1 * uni(seed, i, 101 + 2 * (uint64_t)t);
            if (y < x * x * pow(1.0 - x * x, 3.5)) {
                q = x;
                break;
            }
        }
        const double vesc = sqrt(2.0) * pow(1.0 + r * r, -0.25);
        double px, py, pz, ux, uy, uz;
        iso(seed, i, 300, px, py, pz);
        iso(seed, i, 302, ux, uy, uz);
        const double v = q * vesc;
        put(b, i, r * px, r * py, r * pz, v * ux, v * uy, v * uz, 0.0, 1.0 / (double)n);
    }
}

// Mean position and velocity in a fixed reduction order (per-block partials, then one block),
// then subtracted.
__global__ void k_mean_partial(Bodies b, uint32_t n, double *part) {
    __shared__ double red[6][256];
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        s[0] += b.x[i]; s[1] += b.y[i]; s[2] += b.z[i];
        s[3] += b.vx[i]; s[4] += b.vy[i]; s[5] += b.vz[i];
    }
    for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = s[k];
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_mean_sub(Bodies b, uint32_t n, const double *part, int nblk) {
    double mean[6];
    for (int k = 0; k < 6; ++k) {
        double t = 0.0;
        for (int q = 0; q < nblk; ++q) t += part[6 * q + k];
        mean[k] = t / (double)n;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        b.x[i] -= mean[0]; b.y[i] -= mean[1]; b.z[i] -= mean[2];
        b.vx[i] -= mean[3]; b.vy[i] -= mean[4]; b.vz[i] -= mean[5];
    }
}

int launch_generate(int kind, Bodies &b, uint32_t n, uint64_t seed, double *scratch,
                    cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 8) blocks = sm_count() * 8;
    switch (kind) {
        case 0:
            k_gen_ring<<<blocks, 256, 0, st>>>(b, n, seed);
            return 1;
        case 1: {
            k_gen_plummer<<<blocks, 256, 0, st>>>(b, n, seed);
            constexpr int kPart = 256;
            k_mean_partial<<<kPart, 256, 0, st>>>(b, n, scratch);
            k_mean_sub<<<blocks, 256, 0, st>>>(b, n, scratch, kPart);
            return 3;
        }
        case 2:
            k_gen_circular<<<blocks, 256, 0, st>>>(b, n, seed);
            return 1;
        default:
            return -1;
    }
}

}  // namespace kd
