// host.cpp -- host-side pieces of the path: initial conditions, the
// reference's crosscheck metric, and norm-wise force error statistics.
//
// Initial conditions:
//   nbgb_ic_reference      the reference driver's own bodies: seedRandom /
//                          nbodyRandom / randomUnitBodies
//                          (src/nbody_util.cpp:81-144), same LCG and
//                          rejection order, so the same seed gives the same
//                          bodies as `nbody --seed`.
//   nbgb_ic_uniform_ball   uniform in a ball, masses m_lo..m_hi (scaled by 1/N)
//   nbgb_ic_plummer        Plummer sphere (G = M = a = 1), Aarseth, Henon &
//                          Wielen (1974): radii by inverting the cumulative
//                          mass, speeds by von Neumann rejection on
//                          q^2 (1 - q^2)^(7/2), isotropic directions, centre of
//                          mass moved to rest at the origin; truncated at 99.9%
//                          of the mass.
// All generators are deterministic in (seed, N) and portable: a splitmix64
// stream, binary64 arithmetic with no contraction-sensitive expressions that
// matter for equality tests, results rounded to binary32 at the end.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "nbody_gb300.h"

namespace {

struct SplitMix {
    uint64_t s;
    explicit SplitMix(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // uniform in [0, 1)
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double lo, double hi) { return lo + (hi - lo) * u01(); }
};

// The reference's LCG: x' = (214013 x + 2531011) mod 2^31, max() = 2^31 - 1.
struct RefLcg {
    uint32_t x;
    explicit RefLcg(uint32_t seed) : x(seed % (1u << 31)) {}
    float uniform(float lo, float hi) {
        x = (uint32_t)(((uint64_t)214013u * x + 2531011u) % (1ull << 31));
        volatile float r = (float)x / (float)((1u << 31) - 1u);
        volatile float a = (1.0f - r) * lo;
        volatile float b = r * hi;
        return a + b;
    }
};

void unit_ball_point(SplitMix &g, double &x, double &y, double &z) {
    for (;;) {
        x = g.uniform(-1, 1);
        y = g.uniform(-1, 1);
        z = g.uniform(-1, 1);
        if (x * x + y * y + z * z <= 1.0)
            return;
    }
}

void isotropic(SplitMix &g, double r, double &x, double &y, double &z) {
    const double u = g.uniform(-1.0, 1.0);
    const double ph = 2.0 * M_PI * g.u01();
    const double s = std::sqrt(std::max(0.0, 1.0 - u * u));
    x = r * s * std::cos(ph);
    y = r * s * std::sin(ph);
    z = r * u;
}

}  // namespace

extern "C" {

NBGB_API int nbgb_ic_reference(float *posMass, float *velInvMass, size_t N, float scale,
                               float velscale, unsigned seed) {
    if (!posMass || !velInvMass)
        return NBGB_ERR_INVALID_ARGUMENT;
    RefLcg g(seed);
    const float pscale = scale * ((float)N / 1024.0f);
    const float vscale = scale * velscale;
    for (size_t i = 0; i < N; i++) {
        float p[3], v[3];
        for (int c = 0; c < 3; c++)
            p[c] = g.uniform(-1.0f, 1.0f);
        volatile float l2 = p[0] * p[0];
        l2 = l2 + p[1] * p[1];
        l2 = l2 + p[2] * p[2];
        if (l2 > 1.0f) {
            i--;
            continue;
        }
        for (int c = 0; c < 3; c++)
            v[c] = g.uniform(-1.0f, 1.0f);
        volatile float k2 = v[0] * v[0];
        k2 = k2 + v[1] * v[1];
        k2 = k2 + v[2] * v[2];
        if (k2 > 1.0f) {
            i--;
            continue;
        }
        for (int c = 0; c < 3; c++) {
            posMass[4 * i + c] = p[c] * pscale;
            velInvMass[4 * i + c] = v[c] * vscale;
        }
        posMass[4 * i + 3] = g.uniform(0.5f, 1.0f);
        velInvMass[4 * i + 3] = 1.0f / posMass[4 * i + 3];
    }
    return NBGB_OK;
}

// Uniform ball of radius `radius`; mass_i = U[m_lo, m_hi] / N (m_lo == m_hi:
// equal masses); zero velocities; velInvMass.w = 1/m (may be NULL).
NBGB_API int nbgb_ic_uniform_ball(float *posMass, float *velInvMass, size_t N, double radius,
                                  double m_lo, double m_hi, unsigned long long seed) {
    if (!posMass)
        return NBGB_ERR_INVALID_ARGUMENT;
    SplitMix g(seed * 0x2545F4914F6CDD1Dull + 1);
    for (size_t i = 0; i < N; i++) {
        double x, y, z;
        unit_ball_point(g, x, y, z);
        const double m = (m_lo == m_hi ? m_lo : g.uniform(m_lo, m_hi)) / (double)N;
        posMass[4 * i + 0] = (float)(x * radius);
        posMass[4 * i + 1] = (float)(y * radius);
        posMass[4 * i + 2] = (float)(z * radius);
        posMass[4 * i + 3] = (float)m;
        if (velInvMass) {
            velInvMass[4 * i + 0] = velInvMass[4 * i + 1] = velInvMass[4 * i + 2] = 0.0f;
            velInvMass[4 * i + 3] = 1.0f / posMass[4 * i + 3];
        }
    }
    return NBGB_OK;
}

// Plummer sphere.  Outputs FP64 pos3/vel3 (double[N][3]) and/or FP32 float4
// posMass / velInvMass (any may be NULL).  Equal masses 1/N.
NBGB_API int nbgb_ic_plummer(double *pos3, double *vel3, float *posMass, float *velInvMass,
                             size_t N, unsigned long long seed) {
    if (N == 0)
        return NBGB_OK;
    SplitMix g(seed * 0x9E3779B97F4A7C15ull + 7);
    std::vector<double> p(3 * N), v(3 * N);
    const double m = 1.0 / (double)N;
    for (size_t i = 0; i < N; i++) {
        double x1;
        do {
            x1 = g.u01();
        } while (x1 <= 0.0 || x1 > 0.999);
        const double r = 1.0 / std::sqrt(std::pow(x1, -2.0 / 3.0) - 1.0);
        isotropic(g, r, p[3 * i], p[3 * i + 1], p[3 * i + 2]);
        double q;
        for (;;) {
            const double x4 = g.u01(), x5 = g.u01();
            const double gq = x4 * x4 * std::pow(1.0 - x4 * x4, 3.5);
            if (0.1 * x5 < gq) {
                q = x4;
                break;
            }
        }
        const double ve = std::sqrt(2.0) * std::pow(1.0 + r * r, -0.25);
        isotropic(g, q * ve, v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    }
    double cp[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
    for (size_t i = 0; i < N; i++)
        for (int c = 0; c < 3; c++) {
            cp[c] += p[3 * i + c];
            cv[c] += v[3 * i + c];
        }
    for (int c = 0; c < 3; c++) {
        cp[c] /= (double)N;
        cv[c] /= (double)N;
    }
    for (size_t i = 0; i < N; i++)
        for (int c = 0; c < 3; c++) {
            p[3 * i + c] -= cp[c];
            v[3 * i + c] -= cv[c];
        }
    for (size_t i = 0; i < N; i++) {
        for (int c = 0; c < 3; c++) {
            if (pos3)
                pos3[3 * i + c] = p[3 * i + c];
            if (vel3)
                vel3[3 * i + c] = v[3 * i + c];
            if (posMass)
                posMass[4 * i + c] = (float)p[3 * i + c];
            if (velInvMass)
                velInvMass[4 * i + c] = (float)v[3 * i + c];
        }
        if (posMass)
            posMass[4 * i + 3] = (float)m;
        if (velInvMass)
            velInvMass[4 * i + 3] = (float)(1.0 / m);
    }
    return NBGB_OK;
}

// FP64 all-pairs force (and potential, self pair excluded) on the host for
// the listed target bodies against all N sources -- the library's accuracy
// yardstick for its own FP32 results (the reference's analogue is its CPU
// crosscheck golden, src/nbody.cu:313-325).  Sources are the FP32 bodies
// widened exactly; eps2 should be the binary32 value the GPU used.  Spread
// over the host's hardware threads.  force3: double[n_targets][3]; phi may
// be NULL.
NBGB_API int nbgb_force_f64_host(const float *posMass, size_t N, double eps2,
                                 const long long *idx, size_t n_targets, double *force3,
                                 double *phi) {
    if (!posMass || !force3 || (n_targets && !idx))
        return NBGB_ERR_INVALID_ARGUMENT;
    for (size_t t = 0; t < n_targets; t++)
        if (idx[t] < 0 || (size_t)idx[t] >= N)
            return NBGB_ERR_INVALID_ARGUMENT;
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (;;) {
            const size_t t = next.fetch_add(1);
            if (t >= n_targets)
                return;
            const size_t i = (size_t)idx[t];
            const double x0 = posMass[4 * i], y0 = posMass[4 * i + 1], z0 = posMass[4 * i + 2];
            double ax = 0, ay = 0, az = 0, p = 0;
            for (size_t j = 0; j < N; j++) {
                const double dx = (double)posMass[4 * j] - x0;
                const double dy = (double)posMass[4 * j + 1] - y0;
                const double dz = (double)posMass[4 * j + 2] - z0;
                const double m = posMass[4 * j + 3];
                const double inv = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz + eps2);
                const double s = m * inv * inv * inv;
                ax += dx * s;
                ay += dy * s;
                az += dz * s;
                if (j != i)
                    p -= m * inv;
            }
            force3[3 * t] = ax;
            force3[3 * t + 1] = ay;
            force3[3 * t + 2] = az;
            if (phi)
                phi[t] = p;
        }
    };
    const unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 256u));
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < nt; k++)
        pool.emplace_back(work);
    work();
    for (auto &th : pool)
        th.join();
    return NBGB_OK;
}

// The reference crosscheck: max over bodies and x,y,z of relError(a, b) =
// |a - b| / b with b signed (src/nbody.cu:120-125, 406-418).  float4 arrays.
NBGB_API float nbgb_crosscheck_max_rel_error(const float *force, const float *golden, size_t N) {
    float mx = 0.0f;
    for (size_t i = 0; i < N; i++)
        for (int c = 0; c < 3; c++) {
            const float a = force[4 * i + c], b = golden[4 * i + c];
            const float e = (a == b) ? 0.0f : std::fabs(a - b) / b;
            if (e > mx)
                mx = e;
        }
    return mx;
}

// Norm-wise per-body relative error |F_i - T_i| / |T_i| of float4 forces
// against FP64 truth (double[N][3]); max and RMS over bodies.  idx (may be
// NULL) maps row t of truth to body idx[t] of force.
NBGB_API int nbgb_force_error_stats(const float *force, const double *truth3,
                                    const long long *idx, size_t n_rows, double *max_rel,
                                    double *rms_rel) {
    if (!force || !truth3)
        return NBGB_ERR_INVALID_ARGUMENT;
    double mx = 0.0, ss = 0.0;
    for (size_t t = 0; t < n_rows; t++) {
        const size_t i = idx ? (size_t)idx[t] : t;
        double num = 0.0, den = 0.0;
        for (int c = 0; c < 3; c++) {
            const double d = (double)force[4 * i + c] - truth3[3 * t + c];
            num += d * d;
            den += truth3[3 * t + c] * truth3[3 * t + c];
        }
        const double rel = den > 0 ? std::sqrt(num / den) : std::sqrt(num);
        mx = rel > mx ? rel : mx;
        ss += rel * rel;
    }
    if (max_rel)
        *max_rel = mx;
    if (rms_rel)
        *rms_rel = n_rows ? std::sqrt(ss / (double)n_rows) : 0.0;
    return NBGB_OK;
}

}  // extern "C"
