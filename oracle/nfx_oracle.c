/*
 * nfx_oracle — CPU restatement of noFluidX3D's explicit tetra-mesh time step.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY. The product (nofluidx3d_gb300) never links, loads or calls
 * this library; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do, and only
 * as the checker or as the timed CPU baseline.
 *
 * Parity pin: ora_*_f64 is checked against the reference's own OpenCL C kernels compiled for the
 * host (oracle/build_ref.py -> oracle/_ref/) and against golden vectors generated from them
 * (tests/golden/). The reference ships no tests or golden vectors of its own.
 *
 * The kernels are in oracle_body.h, included once per precision:
 *   _f64 : double, as the reference ships (nofluidx3d/kernels/typedefs.h:1-7)
 *   _f32 : float, the same scheme with single-precision typedefs
 * ora_run_par_* runs the same step with OpenMP over work-items and atomic force adds, which is
 * how an OpenCL CPU runtime executes the reference; it is used only to time the CPU baseline.
 *
 * Build: cc -O2 -fPIC -shared -fopenmp -ffp-contract=off nfx_oracle.c -lm (see oracle/build.py).
 * -ffp-contract=off keeps x86-64 and aarch64 results identical (no fused multiply-add).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { ORA_MODEL_MR = 0, ORA_MODEL_SVK = 1, ORA_MODEL_SVKK = 2, ORA_MODEL_VP = 3 };
enum { ORA_SUBSTRATE = 0, ORA_PLANE = 1, ORA_SPHERE = 2, ORA_SPHERE_INTEGRAL = 3 };

typedef struct {
    int kind;      /* ORA_SUBSTRATE / ORA_PLANE / ORA_SPHERE / ORA_SPHERE_INTEGRAL */
    double k;      /* penalty constant (def_FORCE_CONST) */
    double radius; /* sphere radius */
    double p0;     /* position at t = 0 (wall height or sphere centre height) */
    double v;      /* descent per step */
    double tmove;  /* time after which the indenter stops (Simulation.py:117-132, :173-183) */
} ora_contact;

typedef struct {
    long np, nt;
    const unsigned* tets; /* 4*nt, SoA */
    const void* edge;     /* 9*nt real, SoA */
    const void* vol;      /* nt real */
    int model;
    double E, nu, mr;     /* Tetra(E, nu, mooneyRivlinRatio) */
    int n_contacts;
    ora_contact contacts[4];
    double xi;            /* velocity-Verlet damping */
    int fix_top_bottom;
    int record_contact;   /* contact whose force is recorded, -1 for none */
    int integrator;       /* 0: VelocityVerlet (unit mass), 1: VelocityVerlet2 (lumped masses) */
    const void* masses;   /* np real, lumped nodal masses (integrator 1) */
} ora_problem;

typedef struct {
    void* points;   /* 3*np real */
    void* vel;      /* 3*np real */
    void* force;    /* 3*np real */
    void* fold;     /* 3*np real */
    void* acc;      /* nt real (VP accumulated plastic strain) */
    void* Fp;       /* 9*nt real (VP plastic deformation tensor) */
    void* vonMises; /* nt real */
    void* pressure; /* nt real */
    void* vp_par;   /* 8 real */
} ora_state;
typedef ora_state* ora_state_p;

/* wallFunc / sphereFunc of nofluidx3d/Simulation.py:117-132 and :173-183 in lattice units. */
static double ora_contact_pos(const ora_contact* c, double t) {
    if (c->kind == ORA_SUBSTRATE) return c->p0;
    if (t <= c->tmove) return c->p0 - c->v * t;
    return c->p0 - c->v * c->tmove;
}

/* One row of simdata.dat: time, indentation = f(0) - f(t), force (Simulation.py:142-153, :194-212). */
static void ora_curve_row(const ora_problem* P, long t, double force, double* row) {
    row[0] = (double)t;
    row[1] = 0.0;
    if (P->record_contact >= 0 && P->record_contact < P->n_contacts) {
        const ora_contact* c = &P->contacts[P->record_contact];
        row[1] = ora_contact_pos(c, 0.0) - ora_contact_pos(c, (double)t);
    }
    row[2] = force;
}

#define real double
#define SFX _f64
#define SQRT sqrt
#define POW pow
#define FMAX fmax
#define FABS fabs
#define EXP exp
#include "oracle_body.h"
#undef real
#undef SFX
#undef SQRT
#undef POW
#undef FMAX
#undef FABS
#undef EXP

#define real float
#define SFX _f32
#define SQRT sqrtf
#define POW powf
#define FMAX fmaxf
#define FABS fabsf
#define EXP expf
#include "oracle_body.h"
#undef real
#undef SFX
#undef SQRT
#undef POW
#undef FMAX
#undef FABS
#undef EXP

/* ------------------------------------------------------------------------------------------ */
/* OpenMP step (CPU baseline timing). Element work-items run in parallel with atomic adds, the  */
/* node work-items in parallel; ordering of the adds is therefore not fixed.                  */
/* ------------------------------------------------------------------------------------------ */
#define PAR_STEP(real, SFX)                                                                         \
    static void ora_step_par##SFX(const ora_problem* P, ora_state_p S, long t) {                    \
        const long np = P->np, nt = P->nt;                                                          \
        real* x = (real*)S->points;                                                                 \
        real* f = (real*)S->force;                                                                  \
        _Pragma("omp parallel for schedule(static)")                                               \
        for (long e = 0; e < nt; e++) {                                                             \
            ora_v3##SFX fo[4];                                                                      \
            if (P->model == ORA_MODEL_VP)                                                           \
                vp_one##SFX(e, np, nt, x, P->tets, (const real*)P->edge, (const real*)S->vp_par,   \
                            (real*)S->acc, (real*)S->Fp, (real*)S->vonMises, (real*)S->pressure, fo); \
            else                                                                                    \
                tet_force_one##SFX(e, np, nt, x, P->tets, (const real*)P->edge, (const real*)P->vol, \
                                   P->model, (real)P->E, (real)P->nu, (real)P->mr, fo);             \
            for (int k = 0; k < 4; k++) {                                                           \
                const long n = P->tets[k * nt + e];                                                 \
                _Pragma("omp atomic") f[n] += fo[k].x;                                              \
                _Pragma("omp atomic") f[np + n] += fo[k].y;                                         \
                _Pragma("omp atomic") f[2 * np + n] += fo[k].z;                                     \
            }                                                                                       \
        }                                                                                           \
        for (int c = 0; c < P->n_contacts; c++) {                                                   \
            const ora_contact* C = &P->contacts[c];                                                 \
            const real pos = (real)ora_contact_pos(C, (double)t);                                   \
            _Pragma("omp parallel for schedule(static)")                                           \
            for (long i = 0; i < np; i++) {                                                         \
                if (C->kind == ORA_SUBSTRATE) substrate_node##SFX(i, np, x, pos, (real)C->k, f);   \
                else if (C->kind == ORA_PLANE) plane_node##SFX(i, np, x, pos, (real)C->k, f);      \
                else sphere_node##SFX(i, np, x, (real)C->radius, pos, (real)C->k, f);              \
            }                                                                                       \
        }                                                                                           \
        _Pragma("omp parallel for schedule(static)")                                               \
        for (long i = 0; i < np; i++)                                                               \
            vv_node##SFX(i, np, x, (real*)S->vel, f, (real*)S->fold, (real)P->xi, P->fix_top_bottom); \
    }                                                                                               \
    long ora_run_par##SFX(const ora_problem* P, ora_state_p S, long t0, long nsteps, int threads) {  \
        int serial = P->integrator != 0; /* the parallel step covers the timed workloads only */    \
        for (int c = 0; c < P->n_contacts; c++) serial |= P->contacts[c].kind == ORA_SPHERE_INTEGRAL; \
        if (threads > 0) omp_set_num_threads(threads);                                              \
        for (long s = 0; s < nsteps; s++) {                                                         \
            if (serial) ora_step##SFX(P, S, t0 + s);                                                \
            else ora_step_par##SFX(P, S, t0 + s);                                                   \
        }                                                                                           \
        return nsteps;                                                                              \
    }

#ifdef _OPENMP
PAR_STEP(double, _f64)
PAR_STEP(float, _f32)
int ora_max_threads(void) { return omp_get_max_threads(); }
#else
long ora_run_par_f64(const ora_problem* P, ora_state_p S, long t0, long nsteps, int threads) {
    (void)threads;
    for (long s = 0; s < nsteps; s++) ora_step_f64(P, S, t0 + s);
    return nsteps;
}
long ora_run_par_f32(const ora_problem* P, ora_state_p S, long t0, long nsteps, int threads) {
    (void)threads;
    for (long s = 0; s < nsteps; s++) ora_step_f32(P, S, t0 + s);
    return nsteps;
}
int ora_max_threads(void) { return 1; }
#endif
