// CPU restatement of the reference particle-mesh step -- TEST INFRASTRUCTURE ONLY.
//
// This file is the oracle: it restates, on the host, the algorithm of
// CosmosCuda.cuh (tugrul512bit/CosmosSimulationWithCuda) for the step
// deposit -> FFT convolution -> gradient -> gather + integrate, following the
// reference kernels line by line (citations below).  The test suite and
// __graft_entry__.smoke() compare the CUDA path against it, and bench.py times
// it as the CPU baseline.  Nothing in the product library links it or calls it.
//
// Two precisions share one template:
//   * R = double : the FP64 oracle (parity reference for the CUDA path);
//   * R = float  : an FP32 transliteration, the CPU baseline that bench.py times.
// Particle state is FP32 in both (the reference stores x, y, xOld, yOld, m as
// float, CosmosCuda.cuh:857-861); the FP64 variant computes every field and
// every update in double and rounds the new positions to float.
//
// Build: oracle/Makefile (g++ -O3 -fopenmp -ffp-contract=off, shared library).
// -ffp-contract=off keeps results identical on x86-64 and aarch64 hosts: every
// fused multiply-add below is an explicit std::fma.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class R>
using cpx = std::complex<R>;

// Radix-2 iterative Cooley-Tukey FFT, unnormalised, sign -1 = forward
// (e^{-2 pi i jk/n}, the cuFFT CUFFT_FORWARD convention the reference uses at
// CosmosCuda.cuh:1266) and +1 = inverse (CUFFT_INVERSE, :1291).  Twiddles are
// computed in double with std::cos / std::sin and rounded to R.
template <class R>
struct Fft1d {
    int n = 0;
    int logn = 0;
    std::vector<cpx<R>> tw;  // tw[k] = exp(-2 pi i k / n), k < n/2
    std::vector<int> rev;

    explicit Fft1d(int n_) : n(n_) {
        while ((1 << logn) < n) ++logn;
        tw.resize(std::max(1, n / 2));
        for (int k = 0; k < n / 2; ++k) {
            const double a = -2.0 * M_PI * double(k) / double(n);
            tw[k] = cpx<R>(R(std::cos(a)), R(std::sin(a)));
        }
        rev.resize(n);
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < logn; ++b)
                if (i & (1 << b)) r |= 1 << (logn - 1 - b);
            rev[i] = r;
        }
    }

    void run(cpx<R>* a, int sign) const {
        for (int i = 0; i < n; ++i)
            if (i < rev[i]) std::swap(a[i], a[rev[i]]);
        for (int len = 2; len <= n; len <<= 1) {
            const int half = len >> 1;
            const int step = n / len;
            for (int s = 0; s < n; s += len) {
                for (int k = 0; k < half; ++k) {
                    cpx<R> w = tw[k * step];
                    if (sign > 0) w = std::conj(w);
                    const cpx<R> u = a[s + k];
                    const cpx<R> v = a[s + k + half];
                    // explicit complex multiply (no library range checks)
                    const cpx<R> t(v.real() * w.real() - v.imag() * w.imag(),
                                   v.real() * w.imag() + v.imag() * w.real());
                    a[s + k] = u + t;
                    a[s + k + half] = u - t;
                }
            }
        }
    }
};

// 2-D FFT of an N x N row-major complex array: rows, then columns.
template <class R>
void fft2d(const Fft1d<R>& f, cpx<R>* a, int N, int sign) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < N; ++y) f.run(a + size_t(y) * N, sign);
    constexpr int CB = 8;  // columns per block (cache friendliness)
#pragma omp parallel
    {
        std::vector<cpx<R>> col(size_t(N) * CB);
#pragma omp for schedule(static)
        for (int x0 = 0; x0 < N; x0 += CB) {
            const int nb = std::min(CB, N - x0);
            for (int y = 0; y < N; ++y)
                for (int c = 0; c < nb; ++c) col[size_t(c) * N + y] = a[size_t(y) * N + x0 + c];
            for (int c = 0; c < nb; ++c) f.run(col.data() + size_t(c) * N, sign);
            for (int y = 0; y < N; ++y)
                for (int c = 0; c < nb; ++c) a[size_t(y) * N + x0 + c] = col[size_t(c) * N + y];
        }
    }
}

template <class R>
struct PM {
    int N;
    bool cic;
    R dt;
    R gmult;
    Fft1d<R> fft;
    std::vector<cpx<R>> filter;   // FFT of the Green's lattice (filter_d)
    std::vector<cpx<R>> deconv;   // FFT of the mass-assignment kernel (deconvFilter_d)
    std::vector<R> density;       // accumulator_d
    std::vector<cpx<R>> lattice;  // lattice_d
    std::vector<R> potential;     // latticeShifted_d
    std::vector<R> force;         // latticeShiftedForceXY_d, interleaved (fx, fy)

    PM(int N_, bool cic_, double dt_, double g_)
        : N(N_), cic(cic_), dt(R(dt_)), gmult(R(g_)), fft(N_) {
        const size_t NN = size_t(N) * N;
        filter.resize(NN);
        deconv.resize(NN);
        density.assign(NN, R(0));
        lattice.assign(NN, cpx<R>(0, 0));
        potential.assign(NN, R(0));
        force.assign(2 * NN, R(0));
        build_filters();
    }

    // Green's lattice G(i, j) = 1/r with minimum-image distances and 3.0 in
    // the self cell: CosmosCuda.cuh:100-117 (k_generateFilterLattice).
    // Mass-assignment kernel at (N/2, N/2): CosmosCuda.cuh:384-414
    // (k_generateMassAssignmentKernel); both transformed with a forward FFT
    // (:1024-1025, :1271-1284); CIC phase shift by (-0.5, -0.5):
    // CosmosCuda.cuh:427-443 (k_applyPhaseShift, launched at :1026-1028).
    void build_filters() {
        const int h = N / 2;
        for (int j = 0; j < N; ++j) {
            for (int i = 0; i < N; ++i) {
                const int cx = i <= h ? 0 : N;
                const int cy = j <= h ? 0 : N;
                const R dx = R(i - cx);
                const R dy = R(j - cy);
                const R r = std::sqrt(dx * dx + dy * dy);
                filter[size_t(j) * N + i] = cpx<R>(r > R(0.5) ? R(1) / r : R(3), R(0));
                const int ddx = i - h;
                const int ddy = j - h;
                R w = R(0);
                if (!cic) {
                    w = (ddx == 0 && ddy == 0) ? R(1) : R(0);
                } else if ((ddx == 0 || ddx == 1) && (ddy == 0 || ddy == 1)) {
                    const R fx = R(0.5), fy = R(0.5);
                    const R wx = (ddx == 0) ? (R(1) - fx) : fx;
                    const R wy = (ddy == 0) ? (R(1) - fy) : fy;
                    w = wx * wy;
                }
                deconv[size_t(j) * N + i] = cpx<R>(w, R(0));
            }
        }
        fft2d(fft, filter.data(), N, -1);
        fft2d(fft, deconv.data(), N, -1);
        if (cic) {
            const double fx = -0.5, fy = -0.5;
            for (int j = 0; j < N; ++j) {
                for (int i = 0; i < N; ++i) {
                    const int kx = (i <= h) ? i : i - N;
                    const int ky = (j <= h) ? j : j - N;
                    const double ph = -2.0 * M_PI * (double(kx) * fx / N + double(ky) * fy / N);
                    const R c = R(std::cos(ph)), s = R(std::sin(ph));
                    cpx<R>& d = deconv[size_t(j) * N + i];
                    const R re = d.real() * c - d.imag() * s;
                    const R im = d.real() * s + d.imag() * c;
                    d = cpx<R>(re, im);
                }
            }
        }
    }

    // k_clearAccumulator (:315-331) + k_scatterMassOnAccumulator (:446-595).
    // Only the first 4*floor(P/4) particles are processed: the reference walks
    // float4 groups (:454-471).  A particle is deposited only when its cell
    // (int truncation) lies in [1, N-1) on both axes (:495-497).
    void deposit(const float* x, const float* y, const float* m, int64_t P) {
        const size_t NN = size_t(N) * N;
        const int64_t Pq = (P / 4) * 4;
        int nt = 1;
#ifdef _OPENMP
        nt = omp_get_max_threads();
#endif
        const bool private_grids = double(NN) * nt * sizeof(R) <= 2.0e9;
        std::fill(density.begin(), density.end(), R(0));
        if (private_grids && nt > 1) {
            std::vector<std::vector<R>> grids(nt);
#pragma omp parallel
            {
                int t = 0;
#ifdef _OPENMP
                t = omp_get_thread_num();
#endif
                grids[t].assign(NN, R(0));
                R* g = grids[t].data();
#pragma omp for schedule(static)
                for (int64_t p = 0; p < Pq; ++p) deposit_one(g, x[p], y[p], m[p]);
            }
#pragma omp parallel for schedule(static)
            for (int64_t c = 0; c < int64_t(NN); ++c) {
                R s = R(0);
                for (int t = 0; t < nt; ++t) s += grids[t][c];
                density[c] = s;
            }
        } else {
            for (int64_t p = 0; p < Pq; ++p) deposit_one(density.data(), x[p], y[p], m[p]);
        }
    }

    inline void deposit_one(R* acc, float xf, float yf, float mf) const {
        const int xi = int(xf);
        const int yi = int(yf);
        if (!(xi >= 1 && xi < N - 1 && yi >= 1 && yi < N - 1)) return;
        const R fx = R(xf) - R(xi);
        const R fy = R(yf) - R(yi);
        const R mx = R(mf);
        const size_t c = size_t(xi) + size_t(yi) * N;
        if (cic) {
            const R x1 = R(1) - fx, y1 = R(1) - fy;
            acc[c] += (x1 * y1) * mx;           // :508
            acc[c + 1] += (fx * y1) * mx;       // :509
            acc[c + N] += (x1 * fy) * mx;       // :510
            acc[c + 1 + N] += (fx * fy) * mx;   // :511
        } else {
            acc[c] += mx;  // :514
        }
    }

    // k_copyAccumulatorIntoLattice (:596-612), forward FFT (:1265-1270),
    // k_multElementwiseLatticeFilter (:149-173), k_divElementwiseLatticeFilter
    // (:120-148), inverse FFT (:1289-1295), k_shiftLattice (:333-355).
    void potential_from_density() {
        const size_t NN = size_t(N) * N;
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < int64_t(NN); ++c) lattice[c] = cpx<R>(density[c], R(0));
        fft2d(fft, lattice.data(), N, -1);
        const R eps = R(0.001);
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < int64_t(NN); ++c) {
            cpx<R> d1 = lattice[c];
            const cpx<R> g = filter[c];
            d1 = cpx<R>(d1.real() * g.real() - d1.imag() * g.imag(),
                        d1.real() * g.imag() + d1.imag() * g.real());
            const cpx<R> d2 = deconv[c];
            const R den = d2.real() * d2.real() + d2.imag() * d2.imag() + eps;
            const R re = (d1.real() * d2.real() + d1.imag() * d2.imag()) / den;
            const R im = (d1.imag() * d2.real() - d1.real() * d2.imag()) / den;
            lattice[c] = cpx<R>(re, im);
        }
        fft2d(fft, lattice.data(), N, +1);
        const R norm = R(double(N) * double(N));
        const int h = N / 2;
#pragma omp parallel for schedule(static)
        for (int y = 0; y < N; ++y) {
            for (int x = 0; x < N; ++x) {
                const int sx = (x + h) % N, sy = (y + h) % N;
                potential[size_t(sx) + size_t(sy) * N] = lattice[size_t(x) + size_t(y) * N].real() / norm;
            }
        }
    }

    // k_calcGradientLattice (:174-229): 4th-order central difference with
    // out-of-range neighbours replaced by the centre value, times the gravity
    // multiplier, stored as interleaved (fx, fy).
    void gradient() {
#pragma omp parallel for schedule(static)
        for (int cy = 0; cy < N; ++cy) {
            for (int cx = 0; cx < N; ++cx) {
                const size_t idx = size_t(cx) + size_t(cy) * N;
                const R c = potential[idx];
                const R l = cx - 1 >= 0 ? potential[idx - 1] : c;
                const R r = cx + 1 < N ? potential[idx + 1] : c;
                const R t = cy - 1 >= 0 ? potential[idx - N] : c;
                const R b = cy + 1 < N ? potential[idx + N] : c;
                const R ll = cx - 2 >= 0 ? potential[idx - 2] : c;
                const R rr = cx + 2 < N ? potential[idx + 2] : c;
                const R tt = cy - 2 >= 0 ? potential[idx - 2 * N] : c;
                const R bb = cy + 2 < N ? potential[idx + 2 * N] : c;
                const R fx = (-rr + R(8) * r - R(8) * l + ll) / R(12);
                const R fy = (-bb + R(8) * b - R(8) * t + tt) / R(12);
                force[2 * idx] = fx * gmult;
                force[2 * idx + 1] = fy * gmult;
            }
        }
    }

    // k_forceMultiSampling (:231-312): NGP or bilinear force gather, position
    // Verlet update newX = (2x - xOld) + dt*F*dt, wrap into [2, N-2] by N-4,
    // xOld <- pre-step (unwrapped) x.  Inactive particles are left untouched.
    void integrate(float* x, float* y, float* xo, float* yo, int64_t P) const {
        const int64_t Pq = (P / 4) * 4;
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < Pq; ++p) {
            const float px = x[p], py = y[p];
            const int cx = int(px), cy = int(py);
            if (!(cx >= 1 && cx < N - 1 && cy >= 1 && cy < N - 1)) continue;
            const size_t c = size_t(cx) + size_t(cy) * N;
            R Fx, Fy;
            if (cic) {
                const R fx = R(px) - R(cx), fy = R(py) - R(cy);
                const R x1 = R(1) - fx, y1 = R(1) - fy;
                const R* f00 = &force[2 * c];
                const R* f10 = &force[2 * (c + 1)];
                const R* f01 = &force[2 * (c + N)];
                const R* f11 = &force[2 * (c + 1 + N)];
                Fx = f00[0] * x1 * y1 + f10[0] * fx * y1 + f01[0] * x1 * fy + f11[0] * fx * fy;
                Fy = f00[1] * x1 * y1 + f10[1] * fx * y1 + f01[1] * x1 * fy + f11[1] * fx * fy;
            } else {
                Fx = force[2 * c];
                Fy = force[2 * c + 1];
            }
            R nx = R(2) * R(px) - R(xo[p]) + dt * Fx * dt;
            R ny = R(2) * R(py) - R(yo[p]) + dt * Fy * dt;
            const R lo = R(2), hi = R(N) - R(2), span = R(N) - R(4);
            if (nx < lo) nx += span;
            if (ny < lo) ny += span;
            if (nx > hi) nx -= span;
            if (ny > hi) ny -= span;
            xo[p] = px;
            yo[p] = py;
            x[p] = float(nx);
            y[p] = float(ny);
        }
    }
};

// FP32 integrate with the exact operation order of the CUDA integrate kernel
// (cosmos_pm library): bilinear weights w = (1-fx)(1-fy) ... and the update
// fma(dt*F, dt, fma(2, x, -xOld)).  Bit-identical to the device kernel on
// identical inputs, which lets the tests check the gather/update bit-exactly.
void integrate_f32_exact(const float* force, int N, int cic, float dt, float* x, float* y, float* xo,
                         float* yo, int64_t P) {
    const int64_t Pq = (P / 4) * 4;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < Pq; ++p) {
        const float px = x[p], py = y[p];
        const int cx = int(px), cy = int(py);
        if (!(cx >= 1 && cx < N - 1 && cy >= 1 && cy < N - 1)) continue;
        const size_t c = size_t(cx) + size_t(cy) * N;
        float Fx, Fy;
        if (cic) {
            const float fx = px - float(cx), fy = py - float(cy);
            const float x1 = 1.0f - fx, y1 = 1.0f - fy;
            const float w00 = x1 * y1, w10 = fx * y1, w01 = x1 * fy, w11 = fx * fy;
            const float* f00 = &force[2 * c];
            const float* f10 = &force[2 * (c + 1)];
            const float* f01 = &force[2 * (c + N)];
            const float* f11 = &force[2 * (c + 1 + N)];
            Fx = std::fma(f11[0], w11, std::fma(f01[0], w01, std::fma(f10[0], w10, f00[0] * w00)));
            Fy = std::fma(f11[1], w11, std::fma(f01[1], w01, std::fma(f10[1], w10, f00[1] * w00)));
        } else {
            Fx = force[2 * c];
            Fy = force[2 * c + 1];
        }
        float nx = std::fma(dt * Fx, dt, std::fma(2.0f, px, -xo[p]));
        float ny = std::fma(dt * Fy, dt, std::fma(2.0f, py, -yo[p]));
        const float span = float(N) - 4.0f;
        if (nx < 2.0f) nx += span;
        if (ny < 2.0f) ny += span;
        if (nx > float(N) - 2.0f) nx -= span;
        if (ny > float(N) - 2.0f) ny -= span;
        xo[p] = px;
        yo[p] = py;
        x[p] = nx;
        y[p] = ny;
    }
}

struct Handle {
    int fp64;
    PM<double>* d = nullptr;
    PM<float>* f = nullptr;
};

template <class R, class T>
void copy_out(const std::vector<R>& v, T* out) {
    for (size_t i = 0; i < v.size(); ++i) out[i] = T(v[i]);
}
template <class R, class T>
void copy_in(std::vector<R>& v, const T* in) {
    for (size_t i = 0; i < v.size(); ++i) v[i] = R(in[i]);
}

inline uint32_t spread_bits(uint32_t v) {
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

}  // namespace

extern "C" {

void* opm_create(int N, int cic, double dt, double gmult, int fp64) {
    if (N < 8 || (N & (N - 1)) != 0) return nullptr;
    Handle* h = new Handle;
    h->fp64 = fp64;
    if (fp64)
        h->d = new PM<double>(N, cic != 0, dt, gmult);
    else
        h->f = new PM<float>(N, cic != 0, dt, gmult);
    return h;
}

void opm_destroy(void* hp) {
    Handle* h = static_cast<Handle*>(hp);
    if (!h) return;
    delete h->d;
    delete h->f;
    delete h;
}

void opm_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int opm_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void opm_deposit(void* hp, const float* x, const float* y, const float* m, int64_t P) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) h->d->deposit(x, y, m, P); else h->f->deposit(x, y, m, P);
}
void opm_potential(void* hp) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) h->d->potential_from_density(); else h->f->potential_from_density();
}
void opm_gradient(void* hp) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) h->d->gradient(); else h->f->gradient();
}
void opm_integrate(void* hp, float* x, float* y, float* xo, float* yo, int64_t P) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) h->d->integrate(x, y, xo, yo, P); else h->f->integrate(x, y, xo, yo, P);
}

// One full step as the reference worker loop runs it (CosmosCuda.cuh:1337-1341).
void opm_step(void* hp, float* x, float* y, float* xo, float* yo, const float* m, int64_t P, int nsteps) {
    for (int s = 0; s < nsteps; ++s) {
        opm_deposit(hp, x, y, m, P);
        opm_potential(hp);
        opm_gradient(hp);
        opm_integrate(hp, x, y, xo, yo, P);
    }
}

// Field access (as double) and injection, for isolated stage tests.
void opm_get_density(void* hp, double* out) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) copy_out(h->d->density, out); else copy_out(h->f->density, out);
}
void opm_get_potential(void* hp, double* out) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) copy_out(h->d->potential, out); else copy_out(h->f->potential, out);
}
void opm_get_force(void* hp, double* out) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) copy_out(h->d->force, out); else copy_out(h->f->force, out);
}
void opm_set_density(void* hp, const double* in) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) copy_in(h->d->density, in); else copy_in(h->f->density, in);
}
void opm_set_potential(void* hp, const double* in) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) copy_in(h->d->potential, in); else copy_in(h->f->potential, in);
}
void opm_set_force(void* hp, const double* in) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->fp64) copy_in(h->d->force, in); else copy_in(h->f->force, in);
}
// Filter spectra (re, im interleaved), for cross-checks of the filter build.
void opm_get_filters(void* hp, double* filt, double* deconv) {
    Handle* h = static_cast<Handle*>(hp);
    const size_t NN = h->fp64 ? h->d->filter.size() : h->f->filter.size();
    for (size_t i = 0; i < NN; ++i) {
        if (h->fp64) {
            filt[2 * i] = h->d->filter[i].real(); filt[2 * i + 1] = h->d->filter[i].imag();
            deconv[2 * i] = h->d->deconv[i].real(); deconv[2 * i + 1] = h->d->deconv[i].imag();
        } else {
            filt[2 * i] = h->f->filter[i].real(); filt[2 * i + 1] = h->f->filter[i].imag();
            deconv[2 * i] = h->f->deconv[i].real(); deconv[2 * i + 1] = h->f->deconv[i].imag();
        }
    }
}

void opm_integrate_f32_exact(const float* force, int N, int cic, float dt, float* x, float* y, float* xo,
                             float* yo, int64_t P) {
    integrate_f32_exact(force, N, cic, dt, x, y, xo, yo, P);
}

// Sort keys of the cosmos_pm library, restated: Morton code of the cell
// (int-truncated x, y) shifted right by 2*granularity bits, so that particles
// group by (2^g x 2^g)-cell tiles in Z order; particles outside the active
// window [1, N-1)^2 get the key (N >> g)^2, one past every tile key, which
// sorts them last.
void opm_sort_keys(const float* x, const float* y, int64_t P, int N, int gran, uint32_t* keys) {
    const uint32_t tiles_per_axis = uint32_t(N) >> gran;
    const uint32_t inactive = tiles_per_axis * tiles_per_axis;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < P; ++p) {
        const int cx = int(x[p]), cy = int(y[p]);
        if (cx >= 1 && cx < N - 1 && cy >= 1 && cy < N - 1)
            keys[p] = spread_bits(uint32_t(cx) >> gran) | (spread_bits(uint32_t(cy) >> gran) << 1);
        else
            keys[p] = inactive;
    }
}

// Stable sort permutation of the keys: perm[i] = index of the i-th smallest.
void opm_stable_sort_perm(const uint32_t* keys, int64_t P, uint32_t* perm) {
    std::vector<uint32_t> idx(P);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [keys](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    std::memcpy(perm, idx.data(), size_t(P) * sizeof(uint32_t));
}

}  // extern "C"
