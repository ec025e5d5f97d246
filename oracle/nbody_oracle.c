/*
 * nbody_oracle.c -- CPU restatement of the reference's all-pairs force path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline leg of bench.py load it.
 * The GB300 library never links, loads or calls it.
 *
 * Parity is pinned: tests/golden/ holds forces produced by the reference's
 * own CPU_AOS / CPU_SOA objects (compiled from the reference sources by
 * oracle/Makefile into oracle/_ref/), and tests/test_oracle.py checks this
 * restatement against them.
 *
 * The same source is compiled twice (oracle/Makefile):
 *   liborc_ieee.so  -O2 -ffp-contract=off, no fast-math: every float op is a
 *                   single IEEE-754 binary32 operation in source order.  This
 *                   build defines the exact semantics that the GPU's
 *                   reference-mode integrator reproduces bit for bit.
 *   liborc_fast.so  -O3 -ffast-math -fopenmp: the reference's own build flags
 *                   (meson.build:33-51; on aarch64 also
 *                   -mlow-precision-recip-sqrt, meson.build:53-58).  This is
 *                   the timed CPU baseline ("port") when the reference's own
 *                   objects are not available.
 *
 * Every function cites the reference file:line it restates.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* Pair interaction: src/bodybodyInteraction.cuh:40-65.                      */
/* On the host the reference's rsqrtf is 1.0f/sqrtf (src/chCUDA.h:143-146).  */
/* ------------------------------------------------------------------------ */
static inline void orc_body_body(float *fx, float *fy, float *fz,
                                 float x0, float y0, float z0,
                                 float x1, float y1, float z1, float m1,
                                 float eps2)
{
    float dx = x1 - x0;
    float dy = y1 - y0;
    float dz = z1 - z0;
    float d2 = dx * dx + dy * dy + dz * dz;
    d2 += eps2;
    float inv = 1.0f / sqrtf(d2);
    float inv3 = inv * inv * inv;
    float s = m1 * inv3;
    *fx = dx * s;
    *fy = dy * s;
    *fz = dz * s;
}

/* ------------------------------------------------------------------------ */
/* CPU_AOS: src/nbody_CPU_AOS.cpp:51-98.  float4 {x,y,z,m} in, float4 out   */
/* (.w untouched).  Unlike the reference this accepts any N >= 0; callers    */
/* that want the reference's N%1024 contract pad with zero-mass bodies.     */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_forces_aos(float *force, const float *posMass, float eps2, size_t N)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(guided)
#endif
    for (long long ii = 0; ii < (long long)N; ii++) {
        size_t i = (size_t)ii;
        const float myX = posMass[4 * i + 0];
        const float myY = posMass[4 * i + 1];
        const float myZ = posMass[4 * i + 2];
        float acx = 0, acy = 0, acz = 0;
#if defined(_OPENMP) && defined(ORC_FAST)
#pragma omp simd reduction(+ : acx, acy, acz)
#endif
        for (size_t j = 0; j < N; j++) {
            float fx, fy, fz;
            orc_body_body(&fx, &fy, &fz, myX, myY, myZ,
                          posMass[4 * j + 0], posMass[4 * j + 1],
                          posMass[4 * j + 2], posMass[4 * j + 3], eps2);
            acx += fx;
            acy += fy;
            acz += fz;
        }
        force[4 * i + 0] = acx;
        force[4 * i + 1] = acy;
        force[4 * i + 2] = acz;
    }
}

/* CPU_AOS's per-target loop (src/nbody_CPU_AOS.cpp:60-95) for a list of    */
/* targets only: row t of force (float4) is body idx[t] against all N        */
/* sources, summed exactly as orc_forces_aos sums it.  Lets a large system   */
/* be checked on a sample of its bodies.                                     */
ORC_EXPORT void orc_forces_aos_idx(float *force, const float *posMass, float eps2, size_t N,
                                   const long long *idx, size_t n_targets)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(guided)
#endif
    for (long long tt = 0; tt < (long long)n_targets; tt++) {
        size_t i = (size_t)idx[tt];
        const float myX = posMass[4 * i + 0];
        const float myY = posMass[4 * i + 1];
        const float myZ = posMass[4 * i + 2];
        float acx = 0, acy = 0, acz = 0;
#if defined(_OPENMP) && defined(ORC_FAST)
#pragma omp simd reduction(+ : acx, acy, acz)
#endif
        for (size_t j = 0; j < N; j++) {
            float fx, fy, fz;
            orc_body_body(&fx, &fy, &fz, myX, myY, myZ,
                          posMass[4 * j + 0], posMass[4 * j + 1],
                          posMass[4 * j + 2], posMass[4 * j + 3], eps2);
            acx += fx;
            acy += fy;
            acz += fz;
        }
        force[4 * tt + 0] = acx;
        force[4 * tt + 1] = acy;
        force[4 * tt + 2] = acz;
        force[4 * tt + 3] = 0.0f;
    }
}

/* ------------------------------------------------------------------------ */
/* CPU_SOA: src/nbody_CPU_SOA.cpp:53-105.  pos[3][N], mass[N], force[3][N].  */
/* This is the reference's timed CPU path.  i_begin/i_end restrict the       */
/* target bodies (all N sources are always summed) so a bounded sample of a  */
/* large system can be timed.                                                 */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_forces_soa(float *fx_out, float *fy_out, float *fz_out,
                               const float *px, const float *py, const float *pz,
                               const float *mass, float eps2, size_t N,
                               size_t i_begin, size_t i_end)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(guided)
#endif
    for (long long ii = (long long)i_begin; ii < (long long)i_end; ii++) {
        size_t i = (size_t)ii;
        const float myX = px[i], myY = py[i], myZ = pz[i];
        float acx = 0, acy = 0, acz = 0;
#if defined(_OPENMP) && defined(ORC_FAST)
#pragma omp simd reduction(+ : acx, acy, acz)
#endif
        for (size_t j = 0; j < N; j++) {
            float fx, fy, fz;
            orc_body_body(&fx, &fy, &fz, myX, myY, myZ, px[j], py[j], pz[j],
                          mass[j], eps2);
            acx += fx;
            acy += fy;
            acz += fz;
        }
        fx_out[i] = acx;
        fy_out[i] = acy;
        fz_out[i] = acz;
    }
}

/* ------------------------------------------------------------------------ */
/* FP64 all-pairs sum (no reference counterpart: the accuracy yardstick).    */
/* Sources are the float4 bodies widened exactly to double; target bodies   */
/* are the listed indices (idx == NULL means 0..n_targets-1).                */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_forces_f64(double *force3, const float *posMass, double eps2,
                               size_t N, const long long *idx, size_t n_targets)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(guided)
#endif
    for (long long tt = 0; tt < (long long)n_targets; tt++) {
        size_t i = idx ? (size_t)idx[tt] : (size_t)tt;
        const double x0 = posMass[4 * i + 0];
        const double y0 = posMass[4 * i + 1];
        const double z0 = posMass[4 * i + 2];
        double ax = 0, ay = 0, az = 0;
        for (size_t j = 0; j < N; j++) {
            double dx = (double)posMass[4 * j + 0] - x0;
            double dy = (double)posMass[4 * j + 1] - y0;
            double dz = (double)posMass[4 * j + 2] - z0;
            double d2 = dx * dx + dy * dy + dz * dz + eps2;
            double inv = 1.0 / sqrt(d2);
            double s = (double)posMass[4 * j + 3] * inv * inv * inv;
            ax += dx * s;
            ay += dy * s;
            az += dz * s;
        }
        force3[3 * tt + 0] = ax;
        force3[3 * tt + 1] = ay;
        force3[3 * tt + 2] = az;
    }
}

/* FP64 potential per target: phi_i = -sum_{j != i} m_j / sqrt(r^2 + eps^2).  */
ORC_EXPORT void orc_potential_f64(double *phi, const float *posMass, double eps2,
                                  size_t N, const long long *idx, size_t n_targets)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(guided)
#endif
    for (long long tt = 0; tt < (long long)n_targets; tt++) {
        size_t i = idx ? (size_t)idx[tt] : (size_t)tt;
        const double x0 = posMass[4 * i + 0];
        const double y0 = posMass[4 * i + 1];
        const double z0 = posMass[4 * i + 2];
        double p = 0;
        for (size_t j = 0; j < N; j++) {
            if (j == i)
                continue;
            double dx = (double)posMass[4 * j + 0] - x0;
            double dy = (double)posMass[4 * j + 1] - y0;
            double dz = (double)posMass[4 * j + 2] - z0;
            p -= (double)posMass[4 * j + 3] / sqrt(dx * dx + dy * dy + dz * dz + eps2);
        }
        phi[tt] = p;
    }
}

/* ------------------------------------------------------------------------ */
/* Integrator: integrateOne, src/nbody.cu:158-182, applied per body as in    */
/* integrateGravitation_SOA (src/nbody.cu:186-236).  Arrays are float4 AOS:  */
/* posMass {x,y,z,m}, velInvMass {vx,vy,vz,1/m}, force {fx,fy,fz,-}.  Only   */
/* xyz of posMass and velInvMass are written, as in the reference.           */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_integrate(float *posMass, float *velInvMass, const float *force,
                              float dt, float damping, size_t N)
{
    for (size_t i = 0; i < N; i++) {
        float invMass = velInvMass[4 * i + 3];
        for (int c = 0; c < 3; c++) {
            float v = velInvMass[4 * i + c];
            v += (force[4 * i + c] * invMass) * dt;
            v *= damping;
            velInvMass[4 * i + c] = v;
        }
        for (int c = 0; c < 3; c++)
            posMass[4 * i + c] += velInvMass[4 * i + c] * dt;
    }
}

/* The same step as the reference binary computes it when built with its    */
/* own flags (meson.build:33-38: -O3 -ffast-math -march=native): GCC then    */
/* contracts the position update pos += vel * dt into one fused multiply-add */
/* and leaves the velocity update as written.  This form is checked bit for  */
/* bit against the reference's compiled integrateGravitation_SOA            */
/* (oracle/ref_shim.cpp) on this machine.                                    */
ORC_EXPORT void orc_integrate_contracted(float *posMass, float *velInvMass, const float *force,
                                         float dt, float damping, size_t N)
{
    for (size_t i = 0; i < N; i++) {
        float invMass = velInvMass[4 * i + 3];
        for (int c = 0; c < 3; c++) {
            float v = velInvMass[4 * i + c];
            v += (force[4 * i + c] * invMass) * dt;
            v *= damping;
            velInvMass[4 * i + c] = v;
        }
        for (int c = 0; c < 3; c++)
            posMass[4 * i + c] = fmaf(velInvMass[4 * i + c], dt, posMass[4 * i + c]);
    }
}

/* ------------------------------------------------------------------------ */
/* Crosscheck metric: relError (src/nbody.cu:120-125) maxed over x,y,z of    */
/* every body (src/nbody.cu:406-418).  The denominator is signed, so only    */
/* components whose golden value is positive can raise the maximum.         */
/* ------------------------------------------------------------------------ */
ORC_EXPORT float orc_max_rel_error(const float *force, const float *golden, size_t N)
{
    float mx = 0.0f;
    for (size_t i = 0; i < 4 * N; i++) {
        if ((i + 1) % 4 == 0)
            continue;
        float a = force[i], b = golden[i];
        float err = (a == b) ? 0.0f : fabsf(a - b) / b;
        if (err > mx)
            mx = err;
    }
    return mx;
}

/* ------------------------------------------------------------------------ */
/* Reference initial conditions: seedRandom / nbodyRandom / randomUnitBodies */
/* (src/nbody_util.cpp:81-144).  The generator is std::minstd-style LCG      */
/* x' = (214013 x + 2531011) mod 2^31 with max() = 2^31 - 1.                 */
/* ------------------------------------------------------------------------ */
typedef struct { uint32_t x; } orc_lcg;

static uint32_t orc_lcg_next(orc_lcg *g)
{
    g->x = (uint32_t)(((uint64_t)214013u * g->x + 2531011u) % (1ull << 31));
    return g->x;
}

static float orc_lcg_uniform(orc_lcg *g, float lo, float hi)
{
    uint32_t v = orc_lcg_next(g);
    float r = (float)v / (float)((1u << 31) - 1u);
    return (1.0f - r) * lo + r * hi;
}

ORC_EXPORT void orc_random_unit_bodies(float *pos, float *vel, size_t N,
                                       float gscale, float velscale, uint32_t seed)
{
    /* std::linear_congruential_engine::seed(s): x = s mod m, and 0 -> 1
       only when the increment is 0 (it is not, so 0 stays 0). */
    orc_lcg g = { seed % (1u << 31) };
    const float scale = gscale * ((float)N / 1024.0f);
    const float vscale = gscale * velscale;
    for (size_t i = 0; i < N; i++) {
        float p[3], v[3];
        p[0] = orc_lcg_uniform(&g, -1.0f, 1.0f);
        p[1] = orc_lcg_uniform(&g, -1.0f, 1.0f);
        p[2] = orc_lcg_uniform(&g, -1.0f, 1.0f);
        if (p[0] * p[0] + p[1] * p[1] + p[2] * p[2] > 1) {
            i--;
            continue;
        }
        v[0] = orc_lcg_uniform(&g, -1.0f, 1.0f);
        v[1] = orc_lcg_uniform(&g, -1.0f, 1.0f);
        v[2] = orc_lcg_uniform(&g, -1.0f, 1.0f);
        if (v[0] * v[0] + v[1] * v[1] + v[2] * v[2] > 1) {
            i--;
            continue;
        }
        pos[4 * i + 0] = p[0] * scale;
        pos[4 * i + 1] = p[1] * scale;
        pos[4 * i + 2] = p[2] * scale;
        pos[4 * i + 3] = orc_lcg_uniform(&g, 0.5f, 1.0f);
        vel[4 * i + 0] = v[0] * vscale;
        vel[4 * i + 1] = v[1] * vscale;
        vel[4 * i + 2] = v[2] * vscale;
        vel[4 * i + 3] = 1.0f / pos[4 * i + 3];
    }
}

/* ------------------------------------------------------------------------ */
/* Plummer sphere (G = M = a = 1) exactly as the GB300 library's              */
/* nbgb_ic_plummer generates it (that generator has no reference            */
/* counterpart: the reference only draws its LCG ball).  Restated here so    */
/* the CPU baseline can build its inputs without loading the GB300 library;  */
/* the tests check that both produce the same bytes.  Steps: a splitmix64    */
/* stream seeded with seed * 0x9E3779B97F4A7C15 + 7; per body a mass         */
/* fraction x1 in (0, 0.999] gives r = (x1^(-2/3) - 1)^(-1/2); an isotropic  */
/* direction (u uniform in [-1, 1), phi = 2 pi U[0,1)); a speed fraction q   */
/* by von Neumann rejection on q^2 (1 - q^2)^(7/2) < 0.1 U; speed            */
/* q sqrt(2) (1 + r^2)^(-1/4) in another isotropic direction; then the       */
/* centre of mass and its velocity are moved to zero.  Binary64 throughout   */
/* (built without contraction), rounded to binary32 only for posMass.        */
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t s; } orc_splitmix;

static uint64_t orc_sm_next(orc_splitmix *g)
{
    uint64_t z = (g->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double orc_sm_u01(orc_splitmix *g)
{
    return (double)(orc_sm_next(g) >> 11) * (1.0 / 9007199254740992.0);
}

static double orc_sm_uniform(orc_splitmix *g, double lo, double hi)
{
    return lo + (hi - lo) * orc_sm_u01(g);
}

static void orc_isotropic(orc_splitmix *g, double r, double *out)
{
    const double u = orc_sm_uniform(g, -1.0, 1.0);
    const double ph = 2.0 * 3.14159265358979323846 * orc_sm_u01(g);
    const double s = sqrt(fmax(0.0, 1.0 - u * u));
    out[0] = r * s * cos(ph);
    out[1] = r * s * sin(ph);
    out[2] = r * u;
}

ORC_EXPORT void orc_ic_plummer(double *pos3, double *vel3, float *posMass, size_t N,
                               uint64_t seed)
{
    orc_splitmix g = { seed * 0x9E3779B97F4A7C15ull + 7 };
    double cp[3] = { 0, 0, 0 }, cv[3] = { 0, 0, 0 };
    if (N == 0)
        return;
    for (size_t i = 0; i < N; i++) {
        double x1;
        do {
            x1 = orc_sm_u01(&g);
        } while (x1 <= 0.0 || x1 > 0.999);
        const double r = 1.0 / sqrt(pow(x1, -2.0 / 3.0) - 1.0);
        orc_isotropic(&g, r, pos3 + 3 * i);
        double q;
        for (;;) {
            const double x4 = orc_sm_u01(&g), x5 = orc_sm_u01(&g);
            const double gq = x4 * x4 * pow(1.0 - x4 * x4, 3.5);
            if (0.1 * x5 < gq) {
                q = x4;
                break;
            }
        }
        const double ve = sqrt(2.0) * pow(1.0 + r * r, -0.25);
        orc_isotropic(&g, q * ve, vel3 + 3 * i);
    }
    for (size_t i = 0; i < N; i++)
        for (int c = 0; c < 3; c++) {
            cp[c] += pos3[3 * i + c];
            cv[c] += vel3[3 * i + c];
        }
    for (int c = 0; c < 3; c++) {
        cp[c] /= (double)N;
        cv[c] /= (double)N;
    }
    for (size_t i = 0; i < N; i++) {
        for (int c = 0; c < 3; c++) {
            pos3[3 * i + c] -= cp[c];
            vel3[3 * i + c] -= cv[c];
            posMass[4 * i + c] = (float)pos3[3 * i + c];
        }
        posMass[4 * i + 3] = (float)(1.0 / (double)N);
    }
}

ORC_EXPORT int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
