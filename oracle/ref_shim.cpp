// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.  Exposes the reference driver's
// own integrator, integrateGravitation_SOA (src/nbody.cu:186-236, applying
// integrateOne, src/nbody.cu:158-182), which the driver keeps static.  This
// translation unit compiles the reference's nbody.cu in place (included from
// the reference checkout by path, never copied) with the reference's flags,
// its main() renamed, and adds one extern "C" entry that calls the static
// function.  Built by `make -C oracle ref` into oracle/_ref/ (git-ignored).
#define main nbody_reference_driver_main
#include "nbody.cu"
#undef main

extern "C" void ref_integrate_soa(float *x, float *y, float *z, float *invMass, float *vx,
                                  float *vy, float *vz, float *fx, float *fy, float *fz,
                                  float dt, float damping, size_t N) {
    float *pos[3] = {x, y, z};
    float *vel[3] = {vx, vy, vz};
    float *force[3] = {fx, fy, fz};
    integrateGravitation_SOA(pos, invMass, vel, force, dt, damping, N);
}
