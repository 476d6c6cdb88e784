// Seeded initial conditions generated on the device (cosmos_pm_generate).
//
// The reference fills its particles on host threads with std::random_device
// (constructor CosmosCuda.cuh:929-950, addGalaxy :1071-1116), so no two runs
// agree.  Here particle i of a generated set draws its random numbers from a
// counter-based stream: draw d of particle i is SplitMix64 (Steele, Lea,
// Flood, OOPSLA 2014) of seed + GOLDEN * (16 i + d + 1).  Every float
// operation is a separately rounded IEEE float32 operation (explicit _rn
// intrinsics, no fused multiply-add), and log, exp, sin and cos are short
// series of those operations written here, so a float32 restatement on the
// host (oracle/ic_np.py) reproduces the output bit for bit.
//
// Families (positions in cells, velocities in cells per unit time, xOld =
// x - v dt):
//   UNIFORM    square of half-width `scale` around the centre, Gaussian
//              velocities of sigma `dispersion`
//   EXP_DISK   surface density ~ exp(-R/scale) (radius = gamma(2) draw,
//              redrawn beyond rmax), circular speed from the analytic enclosed
//              mass, rotation sense `spin`, Gaussian dispersion as a fraction
//              of the circular speed
//   PLUMMER    projected Plummer sphere of scale radius `scale`, truncated at
//              rmax, speeds as for the disk
//   RING_DISK  the reference's addGalaxy formula (:1071-1116) on the lattice
//              size and time step of the handle
// Masses: `mass` / count each, times exp(mass_sigma * z) for a Gaussian z.
#include <cstring>

#include "pm_common.cuh"
#include "pm_internal.h"

namespace cpm {

namespace ic {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

__device__ __forceinline__ uint64_t splitmix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t draw(uint64_t seed, uint64_t i, uint32_t d) {
    return splitmix(seed + kGolden * (16ull * i + d + 1ull));
}

__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dvd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }

// Uniform in (0, 1): an odd 24-bit integer (exact in float32) times 2^-24.
__device__ __forceinline__ float uniform_open(uint64_t h) {
    return mul(float(uint32_t(h >> 40) | 1u), 5.9604644775390625e-8f);
}
// Uniform in [0, 1): 24 bits.
__device__ __forceinline__ float uniform_closed(uint64_t h) { return mul(float(uint32_t(h >> 40)), 5.9604644775390625e-8f); }

// ln(u), u > 0 normal: u = m 2^e, m in [sqrt(1/2), sqrt(2)), s = (m-1)/(m+1),
// ln m = 2 s (1 + s^2/3 + s^4/5 + s^6/7 + s^8/9).
__device__ __forceinline__ float ln(float u) {
    const uint32_t bits = __float_as_uint(u);
    int e = int((bits >> 23) & 0xFFu) - 127;
    float m = __uint_as_float((bits & 0x7FFFFFu) | 0x3F800000u);
    if (m > 1.41421354f) {
        m = mul(m, 0.5f);
        e += 1;
    }
    const float s = dvd(sub(m, 1.0f), add(m, 1.0f));
    const float s2 = mul(s, s);
    float p = 0.111111112f;              // 1/9
    p = add(mul(p, s2), 0.142857149f);   // 1/7
    p = add(mul(p, s2), 0.200000003f);   // 1/5
    p = add(mul(p, s2), 0.333333343f);   // 1/3
    p = add(mul(p, s2), 1.0f);
    return add(mul(mul(2.0f, s), p), mul(float(e), 0.693147182f));
}

// exp(x) for x in [-80, 80]: 2^k exp(r), k = rint(x / ln 2), |r| <= ln2 / 2
// (ln 2 in two parts, the high one with 9 trailing zero bits so that k * hi is
// exact: Cody and Waite's reduction), exp(r) by its Taylor series to r^8 / 8!.
__device__ __forceinline__ float exp_(float x) {
    x = x < -80.0f ? -80.0f : (x > 80.0f ? 80.0f : x);
    const float k = rintf(mul(x, 1.44269502f));
    const float r = sub(sub(x, mul(k, 0.693145751953125f)), mul(k, 1.42860682e-6f));
    float p = 2.48015876e-5f;           // 1/8!
    p = add(mul(p, r), 1.98412701e-4f); // 1/7!
    p = add(mul(p, r), 1.38888892e-3f); // 1/6!
    p = add(mul(p, r), 8.33333377e-3f); // 1/5!
    p = add(mul(p, r), 4.16666679e-2f); // 1/4!
    p = add(mul(p, r), 0.166666672f);   // 1/3!
    p = add(mul(p, r), 0.5f);
    p = add(mul(p, r), 1.0f);
    p = add(mul(p, r), 1.0f);
    const int ki = int(k);
    return mul(p, __uint_as_float(uint32_t(ki + 127) << 23));
}

// sin and cos of 2 pi t for a 24-bit fraction t = h24 / 2^24: the quadrant
// from the top two bits, the octant by symmetry, Taylor series on [0, pi/4].
__device__ __forceinline__ void sincos_turn(uint32_t h24, float& sn, float& cs) {
    const uint32_t q = h24 >> 22;
    uint32_t f = h24 & 0x3FFFFFu;  // position within the quadrant, 22 bits
    const bool upper = f > 0x200000u;
    if (upper) f = 0x400000u - f;   // pi/2 - angle
    const float th = mul(float(f), 3.74507039e-7f);  // (pi/2) / 2^22
    const float t2 = mul(th, th);
    float ps = -2.50521079e-8f;               // -1/11!
    ps = add(mul(ps, t2), 2.75573188e-6f);    // 1/9!
    ps = add(mul(ps, t2), -1.98412701e-4f);   // -1/7!
    ps = add(mul(ps, t2), 8.33333377e-3f);    // 1/5!
    ps = add(mul(ps, t2), -0.166666672f);     // -1/3!
    ps = add(mul(ps, t2), 1.0f);
    const float s0 = mul(th, ps);
    float pc = 2.08767559e-9f;                // 1/12!
    pc = add(mul(pc, t2), -2.75573188e-7f);   // -1/10!
    pc = add(mul(pc, t2), 2.48015876e-5f);    // 1/8!
    pc = add(mul(pc, t2), -1.38888892e-3f);   // -1/6!
    pc = add(mul(pc, t2), 4.16666679e-2f);    // 1/4!
    pc = add(mul(pc, t2), -0.5f);
    const float c0 = add(mul(pc, t2), 1.0f);
    const float s1 = upper ? c0 : s0, c1 = upper ? s0 : c0;  // angle within the quadrant
    switch (q) {
        case 0: sn = s1; cs = c1; break;
        case 1: sn = c1; cs = -s1; break;
        case 2: sn = -s1; cs = -c1; break;
        default: sn = -c1; cs = s1; break;
    }
}

// Gaussian by Box-Muller from two draws.
__device__ __forceinline__ float gauss(uint64_t ha, uint64_t hb) {
    float sn, cs;
    sincos_turn(uint32_t(hb >> 40), sn, cs);
    return mul(sqrt_(mul(-2.0f, ln(uniform_open(ha)))), cs);
}

}  // namespace ic

struct IcArgs {
    cosmos_ic_params p;
    int64_t count;
    int64_t first;  // counter of the first particle (its identity)
    int32_t N;
    float dt;
};

__global__ void k_generate(IcArgs a, float* __restrict__ x, float* __restrict__ y, float* __restrict__ xo,
                           float* __restrict__ yo, float* __restrict__ m) {
    using namespace ic;
    const cosmos_ic_params& p = a.p;
    for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j < a.count; j += int64_t(gridDim.x) * blockDim.x) {
        const uint64_t i = uint64_t(a.first + j);
        float px, py, vx = 0.0f, vy = 0.0f;
        float mass = dvd(p.mass, float(a.count));
        if (p.kind == COSMOS_IC_RING_DISK) {
            // CosmosCuda.cuh:1080-1110 on this handle's N and dt
            const float Nf = float(a.N), dt = a.dt;
            const float n = float(a.count);
            const float w = dvd(p.spin, dt);
            const float R = mul(Nf, p.scale);
            const float rad2 = mul(R, R);
            const float total = add(mul(p.mass, n), p.black_hole ? dvd(mul(n, p.mass), 1000.0f) : 0.0f);
            const float cvx = dvd(p.bulk_vx, dt), cvy = dvd(p.bulk_vy, dt);
            const float cxn = mul(p.center_x, Nf), cyn = mul(p.center_y, Nf);
            const float r = mul(add(0.1f, mul(0.9f, uniform_closed(draw(p.seed, i, 0)))), R);
            float sn, cs;
            sincos_turn(uint32_t(draw(p.seed, i, 1) >> 40), sn, cs);
            const float speed = sqrt_(dvd(mul(mul(4.4e-6f, total), r), rad2));
            px = add(mul(r, cs), cxn);
            py = add(mul(r, sn), cyn);
            const float vecx = sub(px, cxn), vecy = sub(py, cyn);
            float pxo = add(mul(-dt, add(mul(mul(vecy, w), speed), mul(cvx, Nf))), px);
            float pyo = add(mul(-dt, add(mul(mul(-vecx, w), speed), mul(cvy, Nf))), py);
            mass = dvd(p.mass, float(p.total_particles));
            if (p.black_hole && j == a.count - 1) {
                px = cxn;
                py = cyn;
                pxo = sub(px, mul(mul(cvx, Nf), dt));
                pyo = sub(py, mul(mul(cvy, Nf), dt));
                mass = dvd(dvd(mul(n, p.mass), 1000.0f), float(p.total_particles));
            }
            x[j] = px;
            y[j] = py;
            xo[j] = pxo;
            yo[j] = pyo;
            m[j] = mass;
            continue;
        }
        if (p.kind == COSMOS_IC_UNIFORM) {
            px = add(p.center_x, mul(sub(mul(2.0f, uniform_closed(draw(p.seed, i, 0))), 1.0f), p.scale));
            py = add(p.center_y, mul(sub(mul(2.0f, uniform_closed(draw(p.seed, i, 1))), 1.0f), p.scale));
            vx = mul(p.dispersion, gauss(draw(p.seed, i, 2), draw(p.seed, i, 3)));
            vy = mul(p.dispersion, gauss(draw(p.seed, i, 4), draw(p.seed, i, 5)));
        } else {
            float r, frac;  // radius and enclosed mass fraction
            const float s = p.scale;
            if (p.kind == COSMOS_IC_EXP_DISK) {
                // gamma(2) radius, redrawn beyond rmax (at most 6 attempts, then scaled into range)
                r = 0.0f;
                bool ok = false;
                for (uint32_t t = 0; t < 6 && !ok; ++t) {
                    const float u = mul(uniform_open(draw(p.seed, i, 2 * t)), uniform_open(draw(p.seed, i, 2 * t + 1)));
                    r = mul(-s, ic::ln(u));
                    ok = p.rmax <= 0.0f || r < p.rmax;
                }
                if (!ok) r = mul(p.rmax, uniform_closed(draw(p.seed, i, 12)));
                // M(<r) / M = 1 - (1 + r/s) exp(-r/s), normalised by its value at rmax
                const float q = dvd(r, s);
                frac = sub(1.0f, mul(add(1.0f, q), exp_(-q)));
                if (p.rmax > 0.0f) {
                    const float qm = dvd(p.rmax, s);
                    frac = dvd(frac, sub(1.0f, mul(add(1.0f, qm), exp_(-qm))));
                }
            } else {  // PLUMMER, projected: M(<r) / M = r^2 / (r^2 + a^2)
                float u = uniform_open(draw(p.seed, i, 0));
                float umax = 1.0f;
                if (p.rmax > 0.0f) {
                    const float rm2 = mul(p.rmax, p.rmax);
                    umax = dvd(rm2, add(rm2, mul(s, s)));
                    if (u > umax) u = umax;
                }
                r = mul(s, sqrt_(dvd(u, sub(1.0f, u))));
                frac = dvd(u, umax);
            }
            float sn, cs;
            sincos_turn(uint32_t(draw(p.seed, i, 13) >> 40), sn, cs);
            px = add(p.center_x, mul(r, cs));
            py = add(p.center_y, mul(r, sn));
            const float rr = r > 1e-3f ? r : 1e-3f;
            const float vc = sqrt_(dvd(mul(mul(p.g, p.mass), frac), rr));
            vx = mul(mul(-p.spin, vc), sn);
            vy = mul(mul(p.spin, vc), cs);
            if (p.dispersion > 0.0f) {
                const float sd = mul(p.dispersion, vc);
                vx = add(vx, mul(sd, gauss(draw(p.seed, i, 14), draw(p.seed, i, 15))));
                vy = add(vy, mul(sd, gauss(draw(p.seed, i, 14) ^ kGolden, draw(p.seed, i, 15) ^ kGolden)));
            }
        }
        vx = add(vx, p.bulk_vx);
        vy = add(vy, p.bulk_vy);
        if (p.mass_sigma > 0.0f) {
            const uint64_t h = draw(p.seed, i, 11);
            mass = mul(mass, exp_(mul(p.mass_sigma, gauss(h, splitmix(h)))));
        }
        x[j] = px;
        y[j] = py;
        xo[j] = sub(px, mul(vx, a.dt));
        yo[j] = sub(py, mul(vy, a.dt));
        m[j] = mass;
    }
}

cudaError_t launch_generate(const cosmos_ic_params& p, int64_t count, int64_t first, int N, float dt, float* x,
                            float* y, float* xo, float* yo, float* m, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    IcArgs a{p, count, first, N, dt};
    int64_t g = (count + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    k_generate<<<int(g), 256, 0, st>>>(a, x, y, xo, yo, m);
    return cudaGetLastError();
}

}  // namespace cpm
