// system.cu -- a GPU-resident simulation: the reference's per-step
// orchestration (src/nbody.cu:293-470: force pass, then integrate) without
// the host round trip.
//
// The reference copies posMass host->device, runs the force algorithm,
// copies forces back and integrates on one host thread every step
// (src/nbody.cu:351-371, 420-441).  Here state stays in HBM: a step is one
// force launch plus one integrate launch that also writes the next step's
// j-stream, captured once into a CUDA graph and replayed.
//
// Integrators:
//   NBGB_INTEGRATOR_REFERENCE        integrateOne (src/nbody.cu:158-182),
//                                    FP32, damping, invMass from
//                                    velInvMass.w, each operation rounded
//   NBGB_INTEGRATOR_REFERENCE_FUSED  the same with x = fma(v, dt, x), as the
//                                    reference binary computes it
//   NBGB_INTEGRATOR_KDK64            FP64 kick-drift-kick leapfrog, a = F,
//                                    no damping
//
// Timing mode brackets every force launch and every integrate launch with
// CUDA events on the system's stream (the step then runs eagerly).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "nbgb_internal.h"
#include "nbody_gb300.h"

using nbgb::ForcePlan;

struct nbgb_system {
    size_t n = 0;
    int integrator = 0;
    float eps2 = 0.f, dt = 0.f, damping = 1.f;
    int device = 0;
    cudaStream_t stream = nullptr;
    ForcePlan plan;
    // device state
    float4 *pm = nullptr;     // posMass {x,y,z,m} (FP32, what the force pass reads)
    float4 *vel = nullptr;    // velInvMass {vx,vy,vz,1/m} (reference integrator)
    float4 *force = nullptr;  // force / acceleration {fx,fy,fz,0}
    double *x64 = nullptr;    // KDK: px,py,pz,vx,vy,vz (6 components, ld apart)
    size_t ld = 0;            // KDK: leading dimension of x64 (n rounded up to 64)
    float *mass = nullptr;    // KDK: m
    void *ws = nullptr;
    size_t ws_bytes = 0;
    bool js_valid = false;     // j-stream in ws matches pm
    bool accel_valid = false;  // KDK: force holds a(x) for the current x
    bool v_lag = false;        // KDK: velocities trail by half a step (closing kick pending)
    bool use_graph = true;
    cudaGraphExec_t graph = nullptr;
    // reference integrators: the force launch also integrates (fused
    // epilogue) and writes the next step's j-stream into the other of two
    // buffers (the workspace's and js2); js_cur names the one to read
    float4 *js2 = nullptr;
    size_t js2_bytes = 0;
    bool js2_ready = false;  // js2 holds the plan's zero-mass padding
    int js_cur = 0;
    cudaGraphExec_t graph2 = nullptr;  // the step body starting from buffer 1
    // optional per-launch timing of the force kernel (bypasses the graph)
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed_once = false;
    // integrate launches: [0,1] reference integrate or kick+drift, [2,3] the
    // closing half kick (KDK)
    cudaEvent_t iev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool itimed = false, htimed = false;
    // force algorithm: 0 one-sided (planned kernel), 1 Newton's third law
    int algorithm = 0;
    void *ws_n3 = nullptr;
    size_t ws_n3_bytes = 0;
    // diagnostics (allocated on first use)
    ForcePlan diag_plan;
    void *diag_ws = nullptr;
    float4 *phi = nullptr;
    double *diag_scratch = nullptr;
    double *diag_out = nullptr;
    int status = NBGB_OK;
};

namespace {

float4 *js_of(nbgb_system *s) { return (float4 *)((char *)s->ws + s->plan.off_js); }
float4 *js_cur_ptr(nbgb_system *s) { return s->js_cur ? s->js2 : js_of(s); }
float4 *js_next_ptr(nbgb_system *s) { return s->js_cur ? js_of(s) : s->js2; }

void drop_graphs(nbgb_system *s) {
    if (s->graph)
        cudaGraphExecDestroy(s->graph);
    if (s->graph2)
        cudaGraphExecDestroy(s->graph2);
    s->graph = s->graph2 = nullptr;
}
unsigned *cnt_of(nbgb_system *s) {
    return nbgb::split_blocks(s->plan) ? (unsigned *)((char *)s->ws + s->plan.off_cnt) : nullptr;
}
int ncnt_of(nbgb_system *s) { return nbgb::split_blocks(s->plan); }
int npad_of(nbgb_system *s) { return s->plan.ntiles * s->plan.tile_bodies; }

double *comp(nbgb_system *s, int c) { return s->x64 + (size_t)c * s->ld; }

bool reference_integrator(int integrator) {
    return integrator == NBGB_INTEGRATOR_REFERENCE || integrator == NBGB_INTEGRATOR_REFERENCE_FUSED;
}

// Event pair k (0: integrate / kick+drift, 1: half kick) around a launch.
int mark(nbgb_system *s, int ev) {
    if (s->timing && cudaEventRecord(s->iev[ev], s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    return NBGB_OK;
}

int ensure_jstream(nbgb_system *s) {
    if (s->js_valid)
        return NBGB_OK;
    int rc = s->js_cur ? nbgb::launch_pack(s->plan, s->pm, s->ws, s->stream, s->js2)
                       : nbgb::launch_pack(s->plan, s->pm, s->ws, s->stream);
    if (rc == NBGB_OK)
        s->js_valid = true;
    return rc;
}

size_t js_bytes(const nbgb::ForcePlan &pl) {
    return (size_t)pl.ntiles * pl.tile_bodies * 16 * (size_t)pl.js_vpb;
}

// Reference integrators: the second j-stream buffer, allocated with the
// system and whenever the plan changes (never inside a step, so steps can be
// captured by the caller), large enough for the plan.
int alloc_js2(nbgb_system *s) {
    const size_t bytes = js_bytes(s->plan);
    s->js2_ready = false;
    if (s->js2 && s->js2_bytes >= bytes)
        return NBGB_OK;
    cudaFree(s->js2);
    s->js2 = nullptr;
    s->js2_bytes = 0;
    if (cudaMalloc(&s->js2, bytes) != cudaSuccess) {
        s->js2 = nullptr;
        return NBGB_ERR_NO_MEMORY;
    }
    s->js2_bytes = bytes;
    return NBGB_OK;
}

// Packed once per plan so its zero-mass padding is in place (the fused
// integrate writes the real bodies' entries every step).
int ensure_js2(nbgb_system *s) {
    if (s->js2_ready)
        return NBGB_OK;
    if (!s->js2 || s->js2_bytes < js_bytes(s->plan))
        return NBGB_ERR_INVALID_ARGUMENT;
    int rc = nbgb::launch_pack(s->plan, s->pm, s->ws, s->stream, s->js2);
    if (rc == NBGB_OK)
        s->js2_ready = true;
    return rc;
}

int force_pass(nbgb_system *s) {
    if (s->algorithm == 1)
        return nbgb_force_newton3((float *)s->force, (const float *)s->pm, s->eps2, s->n,
                                  s->ws_n3, s->ws_n3_bytes, s->stream);
    int rc = ensure_jstream(s);
    if (rc != NBGB_OK)
        return rc;
    return nbgb::launch_force(s->plan, s->force, s->pm, js_cur_ptr(s), s->eps2, s->ws, s->stream);
}

// The force launch of a step, bracketed by events when timing is on; fi:
// the reference integrator fused into it (one-sided kernel only).
int timed_force(nbgb_system *s, const nbgb::FusedIntegrate *fi = nullptr) {
    if (s->timing && cudaEventRecord(s->ev0, s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    int rc = s->algorithm == 1
                 ? nbgb_force_newton3((float *)s->force, (const float *)s->pm, s->eps2, s->n,
                                      s->ws_n3, s->ws_n3_bytes, s->stream)
                 : nbgb::launch_force(s->plan, s->force, s->pm, js_cur_ptr(s), s->eps2, s->ws,
                                      s->stream, fi);
    if (rc == NBGB_OK && s->timing) {
        if (cudaEventRecord(s->ev1, s->stream) != cudaSuccess)
            return NBGB_ERR_CUDA;
        s->timed_once = true;
    }
    return rc;
}

// One reference step: force(x) then integrate (writes x' and its j-stream).
// With the one-sided kernel both happen in one launch: the force kernel's
// epilogue integrates each body once its force is final and writes the next
// step's j-stream into the other buffer, which then becomes current.  With
// the Newton-3 kernel the integrate is its own launch.
int ref_step_body(nbgb_system *s) {
    const int fused_drift = s->integrator == NBGB_INTEGRATOR_REFERENCE_FUSED ? 1 : 0;
    if (s->algorithm == 0) {
        nbgb::FusedIntegrate fi;
        fi.pm = s->pm;
        fi.vel = s->vel;
        fi.js = js_next_ptr(s);
        fi.dt = s->dt;
        fi.damping = s->damping;
        fi.fused_drift = fused_drift;
        int rc = timed_force(s, &fi);
        if (rc == NBGB_OK)
            s->js_cur ^= 1;
        return rc;
    }
    int rc = timed_force(s);
    if (rc == NBGB_OK)
        rc = mark(s, 0);
    if (rc == NBGB_OK)
        rc = nbgb::launch_integrate_reference(
            s->pm, s->vel, s->force, s->dt, s->damping, s->n, fused_drift, js_cur_ptr(s),
            s->plan.js_vpb, s->plan.js_log, npad_of(s), cnt_of(s), ncnt_of(s), s->stream);
    if (rc == NBGB_OK && (rc = mark(s, 1)) == NBGB_OK && s->timing)
        s->itimed = true;
    return rc;
}

// One fused leapfrog body: v += a*kick; x += v*dt; a = F(x).
int kdk_body(nbgb_system *s, double kick) {
    int rc = mark(s, 0);
    if (rc == NBGB_OK)
        rc = nbgb::launch_kick_drift(s->x64, s->ld, s->mass, s->force, kick, (double)s->dt, s->n,
                                     s->pm, js_of(s), s->plan.js_vpb, s->plan.js_log, npad_of(s),
                                     cnt_of(s), ncnt_of(s), s->stream);
    if (rc == NBGB_OK && (rc = mark(s, 1)) == NBGB_OK && s->timing)
        s->itimed = true;
    if (rc != NBGB_OK)
        return rc;
    return timed_force(s);
}

int half_kick(nbgb_system *s) {
    int rc = mark(s, 2);
    if (rc == NBGB_OK)
        rc = nbgb::launch_half_kick(s->x64, s->ld, s->force, 0.5 * (double)s->dt, s->n, s->stream);
    if (rc == NBGB_OK && (rc = mark(s, 3)) == NBGB_OK && s->timing)
        s->htimed = true;
    return rc;
}

// KDK: a step leaves the velocities half a step behind the positions; the
// closing half kick is applied only when something reads or replaces the
// velocities, and otherwise merges into the next step's opening kick (one
// kick of dt instead of two of dt/2).  The steady-state loop is then one
// integrate launch and one force launch per step.
int sync_velocities(nbgb_system *s) {
    if (s->integrator != NBGB_INTEGRATOR_KDK64 || !s->v_lag)
        return NBGB_OK;
    int rc = half_kick(s);
    if (rc == NBGB_OK)
        s->v_lag = false;
    return rc;
}

// Masses below zero (or NaN) have no logarithm: a system whose plan takes
// some source pairs in the log domain moves to an rsqrt-only plan (growing
// its workspace if needed) when such masses are set.  m: n masses, stride
// floats apart (host memory).
int fit_plan_to_masses(nbgb_system *s, const float *m, size_t stride) {
    if (!s->plan.js_log)
        return NBGB_OK;
    bool all_nonneg = true;
    for (size_t i = 0; i < s->n && all_nonneg; i++)
        all_nonneg = m[i * stride] >= 0.f;
    if (all_nonneg)
        return NBGB_OK;
    nbgb::ForcePlan pl;
    int rc = nbgb::plan_force_rsqrt(s->n, pl);
    if (rc != NBGB_OK)
        return rc;
    if (cudaStreamSynchronize(s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    if (pl.workspace_bytes > s->ws_bytes) {
        void *ws = nullptr;
        if (cudaMalloc(&ws, pl.workspace_bytes) != cudaSuccess)
            return NBGB_ERR_NO_MEMORY;
        cudaFree(s->ws);
        s->ws = ws;
        s->ws_bytes = pl.workspace_bytes;
    }
    // split counters start at zero
    if (cudaMemsetAsync(s->ws, 0, s->ws_bytes, s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    drop_graphs(s);
    s->plan = pl;
    s->js_cur = 0;
    if (reference_integrator(s->integrator) && (rc = alloc_js2(s)) != NBGB_OK)
        return rc;  // repacked for the new plan at the next step
    return NBGB_OK;
}

int check_device_status() {
    unsigned bits = 0;
    if (nbgb::read_and_clear_status(&bits) != NBGB_OK)
        return NBGB_ERR_CUDA;
    return bits ? NBGB_ERR_DEVICE : NBGB_OK;
}

void free_all(nbgb_system *s) {
    drop_graphs(s);
    if (s->ev0)
        cudaEventDestroy(s->ev0);
    if (s->ev1)
        cudaEventDestroy(s->ev1);
    for (cudaEvent_t e : s->iev)
        if (e)
            cudaEventDestroy(e);
    cudaFree(s->pm);
    cudaFree(s->vel);
    cudaFree(s->force);
    cudaFree(s->x64);
    cudaFree(s->mass);
    cudaFree(s->ws);
    cudaFree(s->js2);
    cudaFree(s->diag_ws);
    cudaFree(s->ws_n3);
    cudaFree(s->phi);
    cudaFree(s->diag_scratch);
    cudaFree(s->diag_out);
    if (s->stream)
        cudaStreamDestroy(s->stream);
}

// The reference step with the integrate fused into the force launch, which
// alternates between the two j-stream buffers.
bool alternates(const nbgb_system *s) {
    return reference_integrator(s->integrator) && s->algorithm == 0;
}

// Steps per captured graph.  Kernels inside one graph start back to back;
// a graph holding one step (one or two kernels) launches no faster than the
// kernels themselves.  Even, so that an alternating sequence ends on the
// j-stream buffer it started from.
constexpr int kGraphSteps = 8;

// Capture kGraphSteps step bodies into one graph (reference: force with the
// fused integrate, or force then integrate; KDK: full kick + drift + force).
int capture_step(nbgb_system *s, cudaGraphExec_t *out) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return NBGB_ERR_CUDA;
    int rc = NBGB_OK;
    for (int k = 0; k < kGraphSteps && rc == NBGB_OK; k++)
        rc = reference_integrator(s->integrator) ? ref_step_body(s)
                                                 : kdk_body(s, (double)s->dt);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (rc != NBGB_OK || e != cudaSuccess) {
        if (g)
            cudaGraphDestroy(g);
        return NBGB_ERR_CUDA;
    }
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    return e == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

// An alternating step sequence needs one graph per starting buffer: graph
// starts by reading buffer 0, graph2 buffer 1.
int build_graph(nbgb_system *s) {
    if (s->graph)
        return NBGB_OK;
    if (!alternates(s))
        return capture_step(s, &s->graph);
    const int cur = s->js_cur;
    s->js_cur = 0;
    int rc = capture_step(s, &s->graph);
    s->js_cur = 1;
    if (rc == NBGB_OK)
        rc = capture_step(s, &s->graph2);
    s->js_cur = cur;  // capturing toggled it (an even number of times)
    if (rc != NBGB_OK)
        drop_graphs(s);
    return rc;
}

cudaGraphExec_t step_graph(nbgb_system *s) {
    return alternates(s) && s->js_cur ? s->graph2 : s->graph;
}

}  // namespace

extern "C" {

NBGB_API nbgb_system *nbgb_system_create(size_t N, int integrator, float softeningSquared, float dt,
                                         float damping) {
    if (N == 0 || N > nbgb::kMaxBodies)
        return nullptr;
    if (!reference_integrator(integrator) && integrator != NBGB_INTEGRATOR_KDK64)
        return nullptr;
    nbgb_system *s = new (std::nothrow) nbgb_system();
    if (!s)
        return nullptr;
    s->n = N;
    s->integrator = integrator;
    s->eps2 = softeningSquared;
    s->dt = dt;
    s->damping = damping;
    cudaGetDevice(&s->device);
    bool ok = nbgb::plan_force(N, -1, -1, s->plan) == NBGB_OK;
    ok = ok && cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMalloc(&s->pm, N * 16) == cudaSuccess;
    ok = ok && cudaMalloc(&s->force, N * 16) == cudaSuccess;
    ok = ok && cudaMalloc(&s->ws, s->plan.workspace_bytes) == cudaSuccess;
    s->ws_bytes = s->plan.workspace_bytes;
    if (reference_integrator(integrator)) {
        ok = ok && cudaMalloc(&s->vel, N * 16) == cudaSuccess;
        ok = ok && alloc_js2(s) == NBGB_OK;
    } else {
        s->ld = (N + 63) / 64 * 64;
        ok = ok && cudaMalloc(&s->x64, s->ld * 6 * sizeof(double)) == cudaSuccess;
        // padding entries stay zero (the pair kernels read and rewrite them)
        ok = ok && cudaMemsetAsync(s->x64, 0, s->ld * 6 * sizeof(double), s->stream) == cudaSuccess;
        ok = ok && cudaMalloc(&s->mass, N * sizeof(float)) == cudaSuccess;
    }
    ok = ok && cudaMemsetAsync(s->force, 0, N * 16, s->stream) == cudaSuccess;
    // counters start at zero; every force launch leaves them at zero
    ok = ok && cudaMemsetAsync(s->ws, 0, s->plan.workspace_bytes, s->stream) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(s->stream) == cudaSuccess;
    if (!ok) {
        free_all(s);
        delete s;
        return nullptr;
    }
    return s;
}

NBGB_API void nbgb_system_destroy(nbgb_system *s) {
    if (!s)
        return;
    cudaStreamSynchronize(s->stream);
    free_all(s);
    delete s;
}

NBGB_API int nbgb_system_set_graph(nbgb_system *s, int enable) {
    if (!s)
        return NBGB_ERR_INVALID_ARGUMENT;
    s->use_graph = enable != 0;
    return NBGB_OK;
}

// Host arrays, float4 AOS: posMass {x,y,z,m}, velInvMass {vx,vy,vz,1/m}.
// For the KDK integrator velInvMass.w is ignored and positions/velocities
// are widened to FP64.
NBGB_API int nbgb_system_set_state(nbgb_system *s, const float *posMass, const float *velInvMass) {
    if (!s || !posMass || !velInvMass)
        return NBGB_ERR_INVALID_ARGUMENT;
    const size_t n = s->n;
    int rc = fit_plan_to_masses(s, posMass + 3, 4);
    if (rc != NBGB_OK)
        return rc;
    if (cudaMemcpyAsync(s->pm, posMass, n * 16, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    if (reference_integrator(s->integrator)) {
        if (cudaMemcpyAsync(s->vel, velInvMass, n * 16, cudaMemcpyHostToDevice, s->stream) !=
            cudaSuccess)
            return NBGB_ERR_CUDA;
    } else {
        const size_t ld = s->ld;
        std::vector<double> h(ld * 6, 0.0);
        std::vector<float> m(n);
        for (size_t i = 0; i < n; i++) {
            for (int c = 0; c < 3; c++) {
                h[c * ld + i] = posMass[4 * i + c];
                h[(3 + c) * ld + i] = velInvMass[4 * i + c];
            }
            m[i] = posMass[4 * i + 3];
        }
        if (cudaMemcpyAsync(s->x64, h.data(), ld * 6 * sizeof(double), cudaMemcpyHostToDevice,
                            s->stream) != cudaSuccess ||
            cudaMemcpyAsync(s->mass, m.data(), n * sizeof(float), cudaMemcpyHostToDevice,
                            s->stream) != cudaSuccess ||
            cudaStreamSynchronize(s->stream) != cudaSuccess)
            return NBGB_ERR_CUDA;
    }
    s->js_valid = false;
    s->accel_valid = false;
    s->v_lag = false;
    return NBGB_OK;
}

// FP64 state in (KDK only): x, v as double[N][3] (AOS), mass float[N].
NBGB_API int nbgb_system_set_state64(nbgb_system *s, const double *pos3, const double *vel3,
                                     const float *mass) {
    if (!s || !pos3 || !vel3 || !mass || s->integrator != NBGB_INTEGRATOR_KDK64)
        return NBGB_ERR_INVALID_ARGUMENT;
    const size_t n = s->n;
    int rc = fit_plan_to_masses(s, mass, 1);
    if (rc != NBGB_OK)
        return rc;
    const size_t ld = s->ld;
    std::vector<double> h(ld * 6, 0.0);
    std::vector<float> pm(n * 4);
    for (size_t i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) {
            h[c * ld + i] = pos3[3 * i + c];
            h[(3 + c) * ld + i] = vel3[3 * i + c];
            pm[4 * i + c] = (float)pos3[3 * i + c];
        }
        pm[4 * i + 3] = mass[i];
    }
    if (cudaMemcpyAsync(s->x64, h.data(), ld * 6 * sizeof(double), cudaMemcpyHostToDevice,
                        s->stream) != cudaSuccess ||
        cudaMemcpyAsync(s->mass, mass, n * sizeof(float), cudaMemcpyHostToDevice, s->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(s->pm, pm.data(), n * 16, cudaMemcpyHostToDevice, s->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    s->js_valid = false;
    s->accel_valid = false;
    s->v_lag = false;
    return NBGB_OK;
}

NBGB_API int nbgb_system_step(nbgb_system *s, int nsteps) {
    if (!s || nsteps < 0)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (nsteps == 0)
        return NBGB_OK;
    int rc = alternates(s) ? ensure_js2(s) : NBGB_OK;
    if (rc == NBGB_OK)
        rc = ensure_jstream(s);
    if (rc != NBGB_OK)
        return rc;
    // whole graphs of kGraphSteps steps, the rest launched directly
    const bool graph = s->use_graph && !s->timing;
    if (reference_integrator(s->integrator)) {
        int k = 0;
        if (graph && nsteps >= kGraphSteps) {
            if ((rc = build_graph(s)) != NBGB_OK)
                return rc;
            for (; k + kGraphSteps <= nsteps; k += kGraphSteps)
                if (cudaGraphLaunch(step_graph(s), s->stream) != cudaSuccess)
                    return NBGB_ERR_CUDA;
        }
        for (; k < nsteps; k++)
            if ((rc = ref_step_body(s)) != NBGB_OK)
                return rc;
        return NBGB_OK;
    }
    // KDK: the opening kick is a half kick when the velocities are in step
    // with the positions, a full one when the previous call's closing half
    // kick is still pending; the call ends with its closing half kick
    // pending (sync_velocities).
    if (!s->accel_valid) {
        if ((rc = force_pass(s)) != NBGB_OK)
            return rc;
        s->accel_valid = true;
    }
    const double first = s->v_lag ? (double)s->dt : 0.5 * (double)s->dt;
    if ((rc = kdk_body(s, first)) != NBGB_OK)  // opening kick + drift + force
        return rc;
    s->v_lag = true;
    int k = 1;
    if (graph && nsteps - 1 >= kGraphSteps) {
        if ((rc = build_graph(s)) != NBGB_OK)
            return rc;
        for (; k + kGraphSteps <= nsteps; k += kGraphSteps)
            if (cudaGraphLaunch(s->graph, s->stream) != cudaSuccess)
                return NBGB_ERR_CUDA;
    }
    for (; k < nsteps; k++)
        if ((rc = kdk_body(s, (double)s->dt)) != NBGB_OK)
            return rc;
    return NBGB_OK;
}

// KDK: apply a pending closing half kick now (the getters and diagnostics do
// it themselves); no-op otherwise.
NBGB_API int nbgb_system_sync_velocities(nbgb_system *s) {
    if (!s)
        return NBGB_ERR_INVALID_ARGUMENT;
    return sync_velocities(s);
}

// Force algorithm of the step loop: 0 the one-sided kernel (default), 1 the
// Newton's-third-law variant (allocates its workspace on first selection).
NBGB_API int nbgb_system_set_force_algorithm(nbgb_system *s, int algorithm) {
    if (!s || algorithm < 0 || algorithm > 1)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (algorithm == 1 && !s->ws_n3) {
        s->ws_n3_bytes = nbgb_force_newton3_workspace_bytes(s->n);
        if (!s->ws_n3_bytes || cudaMalloc(&s->ws_n3, s->ws_n3_bytes) != cudaSuccess) {
            s->ws_n3 = nullptr;
            return NBGB_ERR_NO_MEMORY;
        }
    }
    // the pending closing kick belongs to the old algorithm's accelerations
    int rc = sync_velocities(s);
    if (rc != NBGB_OK)
        return rc;
    drop_graphs(s);
    s->algorithm = algorithm;
    s->accel_valid = false;
    return NBGB_OK;
}

// Timing mode: every force launch is bracketed by CUDA events on the
// system's stream (steps run eagerly, not from the graph).
NBGB_API int nbgb_system_set_timing(nbgb_system *s, int enable) {
    if (!s)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (enable && !s->ev0) {
        if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess)
            return NBGB_ERR_CUDA;
        for (cudaEvent_t &e : s->iev)
            if (cudaEventCreate(&e) != cudaSuccess)
                return NBGB_ERR_CUDA;
    }
    s->timing = enable != 0;
    s->timed_once = false;
    s->itimed = s->htimed = false;
    return NBGB_OK;
}

// Milliseconds of the most recent timed integrate launches (waits for them):
// step_ms the reference integrate or the FP64 kick+drift, half_kick_ms the
// closing FP64 half kick (0 when none ran, e.g. reference integrators).  A
// reference step on the one-sided kernel integrates inside the force launch
// and times no separate integrate.
NBGB_API int nbgb_system_last_integrate_ms(nbgb_system *s, float *step_ms, float *half_kick_ms) {
    if (!s || !s->timing || !s->itimed)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (step_ms && (cudaEventSynchronize(s->iev[1]) != cudaSuccess ||
                    cudaEventElapsedTime(step_ms, s->iev[0], s->iev[1]) != cudaSuccess))
        return NBGB_ERR_CUDA;
    if (half_kick_ms) {
        *half_kick_ms = 0.f;
        if (s->htimed && (cudaEventSynchronize(s->iev[3]) != cudaSuccess ||
                          cudaEventElapsedTime(half_kick_ms, s->iev[2], s->iev[3]) != cudaSuccess))
            return NBGB_ERR_CUDA;
    }
    return NBGB_OK;
}

// Milliseconds of the most recent timed force launch (waits for it).
NBGB_API int nbgb_system_last_force_ms(nbgb_system *s, float *ms) {
    if (!s || !ms || !s->timing || !s->timed_once)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (cudaEventSynchronize(s->ev1) != cudaSuccess ||
        cudaEventElapsedTime(ms, s->ev0, s->ev1) != cudaSuccess)
        return NBGB_ERR_CUDA;
    return NBGB_OK;
}

NBGB_API int nbgb_system_synchronize(nbgb_system *s) {
    if (!s)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (cudaStreamSynchronize(s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    return check_device_status();
}

NBGB_API int nbgb_system_get_state(nbgb_system *s, float *posMass, float *velInvMass) {
    if (!s)
        return NBGB_ERR_INVALID_ARGUMENT;
    const size_t n = s->n;
    if (velInvMass) {
        int rc = sync_velocities(s);
        if (rc != NBGB_OK)
            return rc;
    }
    if (posMass &&
        cudaMemcpyAsync(posMass, s->pm, n * 16, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    if (velInvMass) {
        if (reference_integrator(s->integrator)) {
            if (cudaMemcpyAsync(velInvMass, s->vel, n * 16, cudaMemcpyDeviceToHost, s->stream) !=
                cudaSuccess)
                return NBGB_ERR_CUDA;
        } else {
            const size_t ld = s->ld;
            std::vector<double> h(ld * 3);
            std::vector<float> m(n);
            if (cudaMemcpyAsync(h.data(), comp(s, 3), ld * 3 * sizeof(double),
                                cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
                cudaMemcpyAsync(m.data(), s->mass, n * sizeof(float), cudaMemcpyDeviceToHost,
                                s->stream) != cudaSuccess ||
                cudaStreamSynchronize(s->stream) != cudaSuccess)
                return NBGB_ERR_CUDA;
            for (size_t i = 0; i < n; i++) {
                for (int c = 0; c < 3; c++)
                    velInvMass[4 * i + c] = (float)h[c * ld + i];
                velInvMass[4 * i + 3] = 1.0f / m[i];
            }
        }
    }
    if (cudaStreamSynchronize(s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    return check_device_status();
}

NBGB_API int nbgb_system_get_state64(nbgb_system *s, double *pos3, double *vel3) {
    if (!s || s->integrator != NBGB_INTEGRATOR_KDK64)
        return NBGB_ERR_INVALID_ARGUMENT;
    const size_t n = s->n, ld = s->ld;
    if (vel3) {
        int rc = sync_velocities(s);
        if (rc != NBGB_OK)
            return rc;
    }
    std::vector<double> h(ld * 6);
    if (cudaMemcpyAsync(h.data(), s->x64, ld * 6 * sizeof(double), cudaMemcpyDeviceToHost,
                        s->stream) != cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    for (size_t i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            if (pos3)
                pos3[3 * i + c] = h[c * ld + i];
            if (vel3)
                vel3[3 * i + c] = h[(3 + c) * ld + i];
        }
    return check_device_status();
}

// Forces of the last force pass (reference: F(x) before the integrate; KDK:
// a(x) at the current positions), float4 AOS.
NBGB_API int nbgb_system_get_force(nbgb_system *s, float *force) {
    if (!s || !force)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (cudaMemcpyAsync(force, s->force, s->n * 16, cudaMemcpyDeviceToHost, s->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    return check_device_status();
}

// Conserved quantities at the current state, FP64: out[0] kinetic energy,
// out[1] potential energy (softened, self pairs excluded), out[2..4] linear
// momentum, out[5..7] angular momentum.  One force+potential pass (an extra
// all-pairs evaluation) plus FP64 reductions; synchronises.
NBGB_API int nbgb_system_diagnostics(nbgb_system *s, double *out) {
    if (!s || !out)
        return NBGB_ERR_INVALID_ARGUMENT;
    const size_t n = s->n;
    int sync_rc = sync_velocities(s);  // kinetic energy and momenta need v(t)
    if (sync_rc != NBGB_OK)
        return sync_rc;
    if (!s->diag_ws) {
        int rc = nbgb::plan_force(n, nbgb::kPotentialConfig, -1, s->diag_plan);
        if (rc != NBGB_OK)
            return rc;
        if (cudaMalloc(&s->diag_ws, s->diag_plan.workspace_bytes) != cudaSuccess ||
            cudaMalloc(&s->phi, n * 16) != cudaSuccess ||
            cudaMalloc(&s->diag_scratch, nbgb::diag_scratch_bytes()) != cudaSuccess ||
            cudaMalloc(&s->diag_out, 8 * sizeof(double)) != cudaSuccess)
            return NBGB_ERR_NO_MEMORY;
    }
    int rc = nbgb::launch_pack(s->diag_plan, s->pm, s->diag_ws, s->stream);
    if (rc == NBGB_OK)
        rc = nbgb::launch_force(s->diag_plan, s->phi, s->pm, nullptr, s->eps2, s->diag_ws,
                                s->stream);
    if (rc == NBGB_OK)
        rc = nbgb::launch_diagnostics((int)n, s->x64, s->ld, s->mass, s->pm, s->vel, s->phi,
                                      s->diag_scratch, s->diag_out, s->stream);
    if (rc != NBGB_OK)
        return rc;
    if (cudaMemcpyAsync(out, s->diag_out, 8 * sizeof(double), cudaMemcpyDeviceToHost,
                        s->stream) != cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    return check_device_status();
}

// Device pointers for callers that manage copies themselves.
NBGB_API void *nbgb_system_device_posmass(nbgb_system *s) { return s ? s->pm : nullptr; }
NBGB_API void *nbgb_system_device_force(nbgb_system *s) { return s ? s->force : nullptr; }
NBGB_API void *nbgb_system_stream(nbgb_system *s) { return s ? s->stream : nullptr; }
// Force plan of the one-sided kernel: config / nsplit as for nbgb_force_ex
// (-1, -1: the planner's choice again).  For tuning and tests.  The
// potential configuration is refused; log-domain configurations need masses
// >= 0.  KDK: a pending closing half kick is applied first and the next step
// starts with a force pass under the new plan.
NBGB_API int nbgb_system_set_plan(nbgb_system *s, int config, int nsplit) {
    if (!s || config == nbgb::kPotentialConfig)
        return NBGB_ERR_INVALID_ARGUMENT;
    nbgb::ForcePlan pl;
    int rc = nbgb::plan_force(s->n, config, nsplit, pl);
    if (rc != NBGB_OK)
        return rc;
    if ((rc = sync_velocities(s)) != NBGB_OK)
        return rc;
    if (cudaStreamSynchronize(s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    if (pl.workspace_bytes > s->ws_bytes) {
        void *ws = nullptr;
        if (cudaMalloc(&ws, pl.workspace_bytes) != cudaSuccess)
            return NBGB_ERR_NO_MEMORY;
        cudaFree(s->ws);
        s->ws = ws;
        s->ws_bytes = pl.workspace_bytes;
    }
    // split counters start at zero
    if (cudaMemsetAsync(s->ws, 0, s->ws_bytes, s->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    drop_graphs(s);
    s->plan = pl;
    s->js_cur = 0;
    s->js_valid = false;  // repacked in the new layout at the next step
    s->accel_valid = false;
    if (reference_integrator(s->integrator) && (rc = alloc_js2(s)) != NBGB_OK)
        return rc;
    return NBGB_OK;
}

NBGB_API int nbgb_system_plan(nbgb_system *s, int *config, int *nsplit) {
    if (!s)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (config)
        *config = s->plan.config;
    if (nsplit)
        *nsplit = s->plan.nsplit;
    return NBGB_OK;
}

}  // extern "C"
