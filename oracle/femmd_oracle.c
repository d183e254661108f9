/*
 * femmd_oracle.c -- TEST INFRASTRUCTURE: the oracle.  Not product code.
 *
 * A single-file, plain-C CPU restatement of the femmd2D timestep of the
 * reference project valeraml/femmd_old (directory femmd2D/src): cell binning,
 * Verlet neighbour list, Lennard-Jones pair forces, harmonic bonds, FEA
 * triangle elasticity (both material laws of the reference) and the
 * kick-drift-kick leapfrog with the reference's half-skin rebuild rule.
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may
 * load it, and only to check results (or as the timed CPU baseline); the CUDA
 * product never links or calls it.
 *
 * Arithmetic families
 *   FP32 "reference" semantics: the same IEEE single-precision operations in
 *     the same order as the reference's CPU path (float overloads of floor,
 *     sqrt and log, which is what the reference's host build resolves to).
 *     This family is pinned bit-for-bit against golden vectors produced by the
 *     reference itself, compiled from its own sources (oracle/Makefile ->
 *     oracle/_ref/ref_harness, fixtures in tests/golden/).
 *   FP32 "exact-image" semantics (image_mode = 1): identical except that a
 *     coordinate difference taken across the periodic boundary is rounded
 *     once from its exact value (TwoSum error term), instead of twice.  The
 *     neighbour/cutoff decisions still use the reference's float values.
 *   own-log (log_mode = 1): the natural log used by the neo-Hookean law is the
 *     fdlibm-style reduction log(x) = k ln2 + log(m), m in [sqrt(1/2), sqrt(2)),
 *     s = f/(2+f), log(m) = f - s (f - R(s^2)) with Taylor coefficients of
 *     2 atanh(s), evaluated without FMA so that the CUDA kernels reproduce it
 *     bit for bit.  log_mode = 0 calls the C library logf like the reference.
 *   FP64 restatement (orc_forces_f64): the same force formulas in double on
 *     the same float inputs, with the discrete decisions (image shifts, cutoff
 *     test, neighbour set) taken from the float path.
 *
 * Build with -ffp-contract=off (no FMA contraction; x86-64 baseline codegen of
 * the reference has none, aarch64 gcc would otherwise fuse).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { NOPBC = 0, XPBC = 1, XYPBC = 2 };

typedef struct {
    int offset, nv, nt, tetOffset;
    float mass, rho;
    float cmx, cmy, cvx, cvy;
} orc_cluster;

typedef struct orc {
    /* Particles (src/particles.h:48-96) */
    int N, cap;
    float *px, *py, *vx, *vy, *ax, *ay, *fx, *fy, *mass, *sigma, *vv;
    int *type, *excl, *cluster;
    /* FeaElements (src/feaElements.h:24-55); refPos/unfoldedPos kept for all N */
    float *refx, *refy, *unfx, *unfy;
    int ntri, tricap;
    int *tri;     /* 3 per triangle, global particle indices */
    float *xm;    /* 9 per triangle, inverse of [1 X Y] (src/particles.cpp:340-352) */
    float *refVol;
    int ncl, clcap;
    orc_cluster *cl;
    int nexcl; /* number of exclusion groups created */
    /* Bonds (src/bonds.h:11-39) */
    int nb, bcap;
    int *bond;
    float *r0;
    /* MDSystem / Interactions parameters */
    float Lx, Ly, density, dt;
    int pbc, numTypes, steps;
    float *eps, *rc, *us;
    float rCutMax;
    int bondForces, feaForces;
    float kBond, E, nu, lambda, mu, Cxxxx, Cxxyy, Cxyxy;
    int fea_law, bond_k_mode, image_mode, log_mode, threads;
    int bond_mode; /* 0: every triangle edge (reference), 1: boundary edges, 2: none */
    /* NeighborList (src/nn.h:21-77); cells and list kept as CSR */
    float skin, nnRadius, nnRadiusSq, dispHi;
    int ncx, ncy, ncells, nn_ready;
    int totalUpdates, initialUpdate, initialSteps, totalSteps;
    int *cellStart, *cellIds, *cellOf;
    int *nbrStart, *nbrList;
    long long nbrCap;
    /* per-step scalars (src/md3dsystem.h:45-53) */
    float potEnergy, virial, feaVirial, kinEneSum, vvMax;
    /* scratch for threaded pair loop */
    float *ui, *wi;
    /* per-elastomer material (own E, nu) and moving harmonic walls */
    float *clE, *clNu;
    int *clOwn, clMatCap;
    int wallOn;
    float wallK, wallY0, wallV;
    /* Interactions::kWall, gravity (src/interactions.h:14-18) */
    float kWall, gravity;
    int gravityForce;
    /* Interactions::kArea, areaForces (src/interactions.h:14,20) */
    float kArea;
    int areaForces;
} orc;

/* ---------------------------------------------------------------- helpers */

static void *xrealloc(void *p, size_t n) {
    void *q = realloc(p, n ? n : 1);
    if (!q) abort();
    return q;
}

#define GROW(ptr, type, cnt) ptr = (type *)xrealloc(ptr, sizeof(type) * (size_t)(cnt))

static void ensure_particles(orc *s, int need) {
    if (need <= s->cap) return;
    int c = s->cap ? s->cap : 64;
    while (c < need) c *= 2;
    GROW(s->px, float, c); GROW(s->py, float, c); GROW(s->vx, float, c); GROW(s->vy, float, c);
    GROW(s->ax, float, c); GROW(s->ay, float, c); GROW(s->fx, float, c); GROW(s->fy, float, c);
    GROW(s->mass, float, c); GROW(s->sigma, float, c); GROW(s->vv, float, c);
    GROW(s->type, int, c); GROW(s->excl, int, c); GROW(s->cluster, int, c);
    GROW(s->refx, float, c); GROW(s->refy, float, c); GROW(s->unfx, float, c); GROW(s->unfy, float, c);
    GROW(s->cellOf, int, c); GROW(s->ui, float, c); GROW(s->wi, float, c);
    s->cap = c;
}

/* TwoSum error of s = a + b (Knuth): a + b == s + err exactly. */
static float two_sum_err(float a, float b, float s) {
    float bb = s - a;
    float t = s - bb;
    return (a - t) + (b - bb);
}

/* minImage (src/def.h:91-93) for one axis.  Returns the reference value in
 * *ref and, in exact-image mode, the once-rounded difference in *out. */
static void image_axis(float a, float b, float L, int wraps, int exact, float *ref, float *out) {
    float d = a - b;
    if (wraps) {
        if (d >= 0.5f * L) {
            float r = d - L;
            *ref = r;
            *out = exact ? r + two_sum_err(a, -b, d) : r;
            return;
        } else if (d < -0.5f * L) {
            float r = d + L;
            *ref = r;
            *out = exact ? r + two_sum_err(a, -b, d) : r;
            return;
        }
    }
    *ref = d;
    *out = d;
}

/* a - b + k L, rounded once from the exact value in exact mode (used by the
 * triangle unwrap, src/interactions.cpp:554-568, exact-image mode). */
static float diff_shift(float a, float b, int k, float L) {
    float d = a - b;
    if (k == 0) return d;
    float e = two_sum_err(a, -b, d);
    float t = d + (float)k * L;
    return t + e;
}

/* pbcCalc (src/def.h:112) */
static float wrap_coord(float r, float L) { return r - floorf(r / L) * L; }

static float own_logf(float x) {
    /* fdlibm-style argument reduction; Taylor coefficients of 2 atanh(s). */
    union { float f; uint32_t u; } v;
    v.f = x;
    if (!(x > 0.0f) || x != x || x == INFINITY) return logf(x); /* NaN/-inf/inf paths */
    int k = 0;
    if (v.u < 0x00800000u) { /* subnormal: scale up */
        v.f = x * 16777216.0f;
        k = -24;
    }
    k += (int)((v.u >> 23) & 0xff) - 127;
    v.u = (v.u & 0x007fffffu) | 0x3f800000u; /* m in [1,2) */
    float m = v.f;
    if (m > 1.41421356f) { m = m * 0.5f; k += 1; }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float R = z * (0.6666666666666666f + z * (0.4f + z * (0.2857142857142857f + z * 0.2222222222222222f)));
    float lm = f - s * (f - R);
    const float ln2_hi = 0.693145751953125f;     /* 16 significant bits */
    const float ln2_lo = 1.428606765330187e-06f; /* ln2 - ln2_hi */
    float fk = (float)k;
    return (fk * ln2_lo + lm) + fk * ln2_hi;
}

static float fea_log(const orc *s, float x) { return s->log_mode ? own_logf(x) : logf(x); }

/* ------------------------------------------------------- system lifecycle */

orc *orc_create(void) {
    orc *s = (orc *)calloc(1, sizeof(orc));
    s->threads = 1;
    return s;
}

static void free_all(orc *s) {
    free(s->px); free(s->py); free(s->vx); free(s->vy); free(s->ax); free(s->ay);
    free(s->fx); free(s->fy); free(s->mass); free(s->sigma); free(s->vv);
    free(s->type); free(s->excl); free(s->cluster); free(s->refx); free(s->refy);
    free(s->unfx); free(s->unfy); free(s->tri); free(s->xm); free(s->refVol); free(s->cl);
    free(s->bond); free(s->r0); free(s->eps); free(s->rc); free(s->us);
    free(s->cellStart); free(s->cellIds); free(s->cellOf); free(s->nbrStart); free(s->nbrList);
    free(s->ui); free(s->wi);
    free(s->clE); free(s->clNu); free(s->clOwn);
}

void orc_destroy(orc *s) {
    if (!s) return;
    free_all(s);
    free(s);
}

/* Interactions::setElasticConstants (src/interactions.cpp:43-50) */
static void lame(float E, float nu, float *mu, float *lambda) {
    *lambda = E * nu / ((1.0f - 2.0f * nu) * (1.0f + nu));
    *mu = E / (2.0f * (1.0f + nu));
}

static void set_elastic_constants(orc *s) {
    lame(s->E, s->nu, &s->mu, &s->lambda);
    s->Cxxxx = s->lambda + 2.0f * s->mu;
    s->Cxxyy = s->lambda;
    s->Cxyxy = s->mu;
}

/* Interactions::setPairForce (src/interactions.cpp:65-79) */
int orc_set_pair_potential(orc *s, const double *eps, const double *rc, const double *us, int n2) {
    int nt = s->numTypes;
    if (n2 < nt * nt) return 1;
    GROW(s->eps, float, nt * nt); GROW(s->rc, float, nt * nt); GROW(s->us, float, nt * nt);
    s->rCutMax = 0.0f;
    for (int i = 0; i < nt * nt; i++) {
        s->eps[i] = (float)eps[i];
        s->rc[i] = (float)rc[i];
        if (s->rc[i] > s->rCutMax) s->rCutMax = s->rc[i];
        s->us[i] = (float)us[i];
    }
    return 0;
}

/* MDSystem::init (src/md3dsystem.cpp:49-80) + Interactions::init
 * (src/interactions.cpp:11-30): WCA defaults, E=0, nu=0.3, kBond=0. */
void orc_init(orc *s, double Lx, double Ly) {
    int th = s->threads;
    int fl = s->fea_law, bm = s->bond_k_mode, im = s->image_mode, lm = s->log_mode, bd = s->bond_mode;
    free_all(s);
    memset(s, 0, sizeof(orc));
    s->threads = th;
    s->fea_law = fl; s->bond_k_mode = bm; s->image_mode = im; s->log_mode = lm; s->bond_mode = bd;
    s->dt = 0.005f;
    s->pbc = XYPBC;
    s->Lx = (float)Lx;
    s->Ly = (float)Ly;
    s->numTypes = 1;
    s->skin = 0.4f; /* NeighborList() default, src/nn.h:63 */
    s->initialUpdate = 1;
    s->nu = 0.3f;
    s->kWall = 10.0f; /* Interactions::init, src/interactions.cpp:22 */
    set_elastic_constants(s);
    double eps = 1.0, rc = pow(2.0, 1.0 / 6.0), us = 1.0;
    orc_set_pair_potential(s, &eps, &rc, &us, 1);
}

void orc_set_box(orc *s, double Lx, double Ly) { s->Lx = (float)Lx; s->Ly = (float)Ly; }
void orc_set_pbc(orc *s, int p) { s->pbc = (p == 0) ? NOPBC : (p == 1) ? XPBC : XYPBC; }
void orc_set_dt(orc *s, double dt) { s->dt = (float)dt; }
void orc_set_num_types(orc *s, int n) { s->numTypes = n; }
void orc_set_skin(orc *s, double sk) { s->skin = (float)sk; }
void orc_set_threads(orc *s, int t) { s->threads = t < 1 ? 1 : t; }
void orc_set_elastomer_bonds(orc *s, int mode) { s->bond_mode = mode; }
void orc_set_modes(orc *s, int fea_law, int bond_k_mode, int image_mode, int log_mode) {
    s->fea_law = fea_law; s->bond_k_mode = bond_k_mode; s->image_mode = image_mode; s->log_mode = log_mode;
}

/* DukSystemSetKBond (src/interface.cpp:455-465) */
void orc_set_kbond(orc *s, double k) {
    if (k > 0) { s->kBond = (float)k; s->bondForces = 1; } else s->bondForces = 0;
}
/* DukSystemSetYoungsModulus (src/interface.cpp:479-490) */
void orc_set_youngs_modulus(orc *s, double E) {
    if (E > 0) { s->E = (float)E; s->feaForces = 1; } else s->feaForces = 0;
    set_elastic_constants(s);
}
void orc_set_nu(orc *s, double nu) { s->nu = (float)nu; set_elastic_constants(s); }

/* Own (E, nu) of elastomer e (neo-Hookean law); no counterpart in the
 * reference, which has one global E. */
int orc_set_elastomer_material(orc *s, int e, double E, double nu) {
    if (e < 0 || e >= s->ncl) return 1;
    if (s->clMatCap < s->ncl) {
        s->clE = (float *)xrealloc(s->clE, sizeof(float) * (size_t)s->ncl);
        s->clNu = (float *)xrealloc(s->clNu, sizeof(float) * (size_t)s->ncl);
        s->clOwn = (int *)xrealloc(s->clOwn, sizeof(int) * (size_t)s->ncl);
        for (int k = s->clMatCap; k < s->ncl; k++) { s->clE[k] = 0; s->clNu[k] = 0; s->clOwn[k] = 0; }
        s->clMatCap = s->ncl;
    }
    s->clE[e] = (float)E; s->clNu[e] = (float)nu; s->clOwn[e] = 1;
    return 0;
}

/* Moving harmonic walls: bottom at y = 0, top at y0 - v (n dt) for the
 * positions of step n; contact range 2^(1/6) sigma_i (the range of
 * calcTopBottomWallForces, src/interactions.cpp:242-270); force k * overlap. */
void orc_set_moving_wall(orc *s, double k, double y0, double v) {
    s->wallOn = k > 0;
    s->wallK = s->wallOn ? (float)k : 0.0f;
    s->wallY0 = (float)y0;
    s->wallV = (float)v;
}

static float wall_range(void) { return (float)pow(2.0, 1.0 / 6.0); }
static float wall_y(const orc *s) { return s->wallY0 - s->wallV * ((float)s->steps * s->dt); }

/* Lame constants of triangle t: its elastomer's own, or the global ones. */
static void tri_lame(const orc *s, int t, float *mu, float *lambda) {
    *mu = s->mu; *lambda = s->lambda;
    if (!s->clOwn) return;
    int e = s->cluster[s->tri[3 * t]];
    if (e >= 0 && e < s->clMatCap && s->clOwn[e]) lame(s->clE[e], s->clNu[e], mu, lambda);
}

/* DukSystemSetGravity (src/interface.cpp:443-453) */
void orc_set_gravity(orc *s, double g) {
    if (g > 0) { s->gravity = (float)g; s->gravityForce = 1; } else s->gravityForce = 0;
}

/* DukSystemSetKArea (src/interface.cpp:466-476) */
void orc_set_karea(orc *s, double k) {
    if (k > 0) { s->kArea = (float)k; s->areaForces = 1; } else s->areaForces = 0;
}

/* ljwallforce (src/interactionsCuda.cu:31-40), float operations as written
 * (zi6 is zi^9 there) */
static float ljwallforce(float zi, float sigma, float *fz) {
    zi = sigma / zi;
    float zi3 = zi * zi * zi;
    float zi6 = zi3 * zi3 * zi3;
    float u = 4.0f * zi6 * (zi6 - 1.0f) + 1.0f;
    float fcVal = 48.0f * zi6 * (zi6 - 0.5f) / zi;
    *fz = fabsf(fcVal);
    return u;
}

/* The reference's fixed walls, first in calcForces (src/interactions.cpp:
 * 83-93): calcWallForces (NOPBC, :176-236: LJ wall on each side) and
 * calcTopBottomWallForces (XPBC, :238-286: f = kWall * distance within the
 * contact range).  The moving walls replace them when set. */
static void ref_wall_forces(orc *s) {
    if (s->wallOn || s->pbc == XYPBC) return;
    float rc = (float)pow(2.0, 1.0 / 6.0);
    for (int i = 0; i < s->N; i++) {
        float s0 = s->sigma[i], f;
        if (s->pbc == NOPBC) {
            if ((s->Ly - s->py[i]) < s0 * rc) {
                float yi = s->Ly - s->py[i];
                float u = ljwallforce(yi, s0, &f);
                s->fy[i] += -f;
                s->potEnergy += u;
            } else if (s->py[i] < s0 * rc) {
                float yi = s->py[i];
                float u = ljwallforce(yi, s0, &f);
                s->fy[i] += f;
                s->potEnergy += u;
            }
            if ((s->Lx - s->px[i]) < s0 * rc) {
                float xi = s->Lx - s->px[i];
                float u = ljwallforce(xi, s0, &f);
                s->fx[i] += -f;
                s->potEnergy += u;
            } else if (s->px[i] < s0 * rc) {
                float xi = s->px[i];
                float u = ljwallforce(xi, s0, &f);
                s->fx[i] += f;
                s->potEnergy += u;
            }
        } else {
            if ((s->Ly - s->py[i]) < s0 * rc) {
                float yi = s->Ly - s->py[i];
                f = s->kWall * yi;
                float u = (float)(0.5 * s->kWall * yi * yi);
                s->fy[i] += -f;
                s->potEnergy += u;
            } else if (s->py[i] < s0 * rc) {
                float yi = s->py[i];
                f = s->kWall * yi;
                float u = (float)(0.5 * s->kWall * yi * yi);
                s->fy[i] += f;
                s->potEnergy += u;
            }
        }
    }
}

/* calcGravityForces (src/interactions.cpp:111-126) */
static void gravity_forces(orc *s) {
    if (!s->gravityForce || !(s->gravity > 0)) return;
    for (int i = 0; i < s->N; i++) s->fy[i] -= s->mass[i] * s->gravity;
}

/* wall forces of every particle, after the pair forces */
static void wall_forces(orc *s) {
    if (!s->wallOn) return;
    float yw = wall_y(s), range = wall_range();
    for (int i = 0; i < s->N; i++) {
        float dl = range * s->sigma[i];
        float ht = (s->py[i] + dl) - yw;
        if (ht > 0.0f) { s->fy[i] -= s->wallK * ht; s->potEnergy += 0.5f * s->wallK * ht * ht; }
        float hb = dl - s->py[i];
        if (hb > 0.0f) { s->fy[i] += s->wallK * hb; s->potEnergy += 0.5f * s->wallK * hb * hb; }
    }
}

/* forces of the particles on the top and bottom walls at the current positions */
void orc_wall_forces(const orc *s, double *top, double *bottom) {
    *top = *bottom = 0;
    if (!s->wallOn) return;
    float yw = wall_y(s), range = wall_range();
    for (int i = 0; i < s->N; i++) {
        float dl = range * s->sigma[i];
        float ht = (s->py[i] + dl) - yw, hb = dl - s->py[i];
        if (ht > 0.0f) *top += (double)(s->wallK * ht);
        if (hb > 0.0f) *bottom += (double)(s->wallK * hb);
    }
}

/* Particles::addParticle (src/particles.cpp:201-231) */
int orc_add_particle(orc *s, double x, double y, double vx, double vy, double m, double sig, int typ) {
    int pid = s->N;
    ensure_particles(s, pid + 1);
    s->N += 1;
    s->density = (float)s->N / (s->Lx * s->Ly);
    s->px[pid] = (float)x; s->py[pid] = (float)y;
    s->vx[pid] = (float)vx; s->vy[pid] = (float)vy;
    s->ax[pid] = s->ay[pid] = s->fx[pid] = s->fy[pid] = 0.0f;
    s->vv[pid] = 0.0f;
    s->mass[pid] = (float)m;
    s->type[pid] = typ;
    s->sigma[pid] = (float)sig;
    s->excl[pid] = -1;
    s->cluster[pid] = -1;
    s->refx[pid] = s->refy[pid] = 0.0f;
    s->unfx[pid] = s->unfy[pid] = 0.0f;
    return pid;
}

/* n calls of addParticle with per-particle arguments */
int orc_add_particles(orc *s, int n, const double *x, const double *y, const double *vx, const double *vy,
                      const double *m, const double *sig, const int *typ) {
    ensure_particles(s, s->N + n);
    for (int k = 0; k < n; k++) orc_add_particle(s, x[k], y[k], vx[k], vy[k], m[k], sig[k], typ[k]);
    return 0;
}

/* Bonds::createBond (src/bonds.cpp:14-29): rest length from current
 * positions, no minimum image. */
int orc_create_bond(orc *s, int i, int j) {
    if (i < 0 || j < 0 || i >= s->N || j >= s->N) return 1;
    if (s->nb + 1 > s->bcap) {
        s->bcap = s->bcap ? 2 * s->bcap : 256;
        GROW(s->bond, int, 2 * s->bcap);
        GROW(s->r0, float, s->bcap);
    }
    s->bond[2 * s->nb] = i;
    s->bond[2 * s->nb + 1] = j;
    float dx = s->px[i] - s->px[j];
    float dy = s->py[i] - s->py[j];
    s->r0[s->nb] = sqrtf(dx * dx + dy * dy);
    s->nb += 1;
    return 0;
}

/* invertMatrix (src/def.h:154-179) */
static int invert3(const float *m, float *out) {
    float inv[9], det;
    det = -m[2] * m[4] * m[6] + m[1] * m[5] * m[6] + m[2] * m[3] * m[7] - m[0] * m[5] * m[7] - m[1] * m[3] * m[8] + m[0] * m[4] * m[8];
    if (det == 0) return 0;
    inv[0] = -m[5] * m[7] + m[4] * m[8];
    inv[1] = m[2] * m[7] - m[1] * m[8];
    inv[2] = -m[2] * m[4] + m[1] * m[5];
    inv[3] = m[5] * m[6] - m[3] * m[8];
    inv[4] = -m[2] * m[6] + m[0] * m[8];
    inv[5] = m[2] * m[3] - m[0] * m[5];
    inv[6] = -m[4] * m[6] + m[3] * m[7];
    inv[7] = m[1] * m[6] - m[0] * m[7];
    inv[8] = -m[1] * m[3] + m[0] * m[4];
    det = 1.0f / det;
    for (int i = 0; i < 9; i++) out[i] = inv[i] * det;
    return 1;
}

/* Particles::addElastomer (src/particles.cpp:295-385).  Returns 0 on success,
 * 2 when the reference's same-mesh / elastomers-first constraint is broken. */
int orc_add_elastomer(orc *s, const float *vert, int nv, const int *tet, int nt, double x, double y,
                      int typ, int g, double sig, double M, int exclude) {
    (void)g;
    int offset = s->N;
    if (s->ncl > 0 && (s->cl[0].nv != nv || s->cl[0].nt != nt)) return 2;
    if (offset != s->ncl * nv) return 2;
    int exclusionGroupId = s->nexcl++;
    if (s->ncl + 1 > s->clcap) {
        s->clcap = s->clcap ? 2 * s->clcap : 16;
        GROW(s->cl, orc_cluster, s->clcap);
    }
    int ci = s->ncl++;
    memset(&s->cl[ci], 0, sizeof(orc_cluster));
    s->cl[ci].offset = offset; s->cl[ci].nv = nv; s->cl[ci].nt = nt;
    float fx0 = (float)x, fy0 = (float)y;
    for (int i = 0; i < nv; i++) {
        float x1 = vert[2 * i] + fx0;
        float y1 = vert[2 * i + 1] + fy0;
        int pid = orc_add_particle(s, x1, y1, 0.0, 0.0, 0.0, sig, typ);
        s->refx[pid] = s->px[pid]; s->refy[pid] = s->py[pid];
        s->unfx[pid] = s->px[pid]; s->unfy[pid] = s->py[pid];
        if (s->pbc == XYPBC) { s->px[pid] = wrap_coord(s->px[pid], s->Lx); s->py[pid] = wrap_coord(s->py[pid], s->Ly); }
        else if (s->pbc == XPBC) { s->px[pid] = wrap_coord(s->px[pid], s->Lx); }
        if (exclude) s->excl[pid] = exclusionGroupId;
        s->cluster[pid] = ci;
    }
    float totVol = 0.0f;
    int tetOffset = ci * nt;
    s->cl[ci].tetOffset = tetOffset;
    if (tetOffset + nt > s->tricap) {
        int c = s->tricap ? s->tricap : 256;
        while (c < tetOffset + nt) c *= 2;
        GROW(s->tri, int, 3 * c); GROW(s->xm, float, 9 * c); GROW(s->refVol, float, c);
        s->tricap = c;
    }
    for (int i = 0; i < nt; i++) {
        int i0 = tet[3 * i] + offset - 1;
        int i1 = tet[3 * i + 1] + offset - 1;
        int i2 = tet[3 * i + 2] + offset - 1;
        int t = i + tetOffset;
        s->tri[3 * t] = i0; s->tri[3 * t + 1] = i1; s->tri[3 * t + 2] = i2;
        if (s->bond_mode == 0) {
            orc_create_bond(s, i0, i1);
            orc_create_bond(s, i0, i2);
            orc_create_bond(s, i1, i2);
        }
        float aa[9], rxv[3], ryv[3];
        for (int j = 0; j < 3; j++) {
            int ip = s->tri[3 * t + j];
            aa[3 * j] = 1.0f; aa[3 * j + 1] = s->refx[ip]; aa[3 * j + 2] = s->refy[ip];
            rxv[j] = s->refx[ip]; ryv[j] = s->refy[ip];
        }
        if (!invert3(aa, &s->xm[9 * t])) memset(&s->xm[9 * t], 0, 9 * sizeof(float));
        float vol = (float)(0.5 * (double)((ryv[2] - ryv[0]) * (rxv[1] - rxv[0]) - (ryv[1] - ryv[0]) * (rxv[2] - rxv[0])));
        s->refVol[t] = vol;
        totVol += vol;
    }
    s->ntri = tetOffset + nt;
    if (s->bond_mode == 1) {
        /* boundary edges only: edges of exactly one triangle, created in
         * triangle order with the per-triangle edge order of the reference */
        long long *keys = (long long *)malloc(sizeof(long long) * 3 * (size_t)nt);
        for (int i = 0; i < nt; i++) {
            const int *q = &tet[3 * i];
            int e[3][2] = {{q[0], q[1]}, {q[0], q[2]}, {q[1], q[2]}};
            for (int k = 0; k < 3; k++) {
                long long a = e[k][0] < e[k][1] ? e[k][0] : e[k][1], b = e[k][0] < e[k][1] ? e[k][1] : e[k][0];
                keys[3 * i + k] = a * 4294967296LL + b;
            }
        }
        for (int i = 0; i < nt; i++) {
            const int *q = &tet[3 * i];
            int e[3][2] = {{q[0], q[1]}, {q[0], q[2]}, {q[1], q[2]}};
            for (int k = 0; k < 3; k++) {
                int cnt = 0;
                for (int m = 0; m < 3 * nt; m++) cnt += keys[m] == keys[3 * i + k];
                if (cnt == 1) orc_create_bond(s, e[k][0] + offset - 1, e[k][1] + offset - 1);
            }
        }
        free(keys);
    }
    s->cl[ci].mass = (float)M;
    s->cl[ci].rho = s->cl[ci].mass / totVol;
    for (int it = 0; it < nt; it++) {
        for (int j = 0; j < 3; j++) {
            int ip = s->tri[3 * (it + tetOffset) + j];
            /* mass[ip] += rho*refVol[itet]/3.0 -- note refVol indexed by the
             * local triangle index, as in the reference (src/particles.cpp:364) */
            float prod = s->cl[ci].rho * s->refVol[it];
            s->mass[ip] = (float)((double)s->mass[ip] + (double)prod / 3.0);
        }
    }
    return 0;
}

/* ----------------------------------------------------- cells & neighbours */

/* cellId (src/nnCuda.cu:9-17); out-of-range rows/columns (only possible on a
 * non-periodic axis, undefined behaviour in the reference) are clamped. */
static int cell_id(const orc *s, float x, float y) {
    int ix = (int)(x * (float)s->ncx / s->Lx);
    if (ix == s->ncx) ix -= 1;
    int iy = (int)(y * (float)s->ncy / s->Ly);
    if (iy == s->ncy) iy -= 1;
    if (ix < 0) ix = 0; if (ix >= s->ncx) ix = s->ncx - 1;
    if (iy < 0) iy = 0; if (iy >= s->ncy) iy = s->ncy - 1;
    return ix + iy * s->ncx;
}

/* NeighborList::init(s, rc) (src/nn.cpp:200-227); capacities are not needed
 * since the oracle keeps CSR arrays. */
int orc_init_neighbor_list(orc *s) {
    float rc = s->rCutMax;
    s->nnRadius = rc + s->skin;
    s->nnRadiusSq = s->nnRadius * s->nnRadius;
    s->ncx = (int)floorf(s->Lx / s->nnRadius);
    s->ncy = (int)floorf(s->Ly / s->nnRadius);
    if (s->ncx < 1 || s->ncy < 1) return 1;
    s->ncells = s->ncx * s->ncy;
    s->dispHi = 0.0f;
    s->totalUpdates = 0;
    s->initialUpdate = 1;
    GROW(s->cellStart, int, s->ncells + 1);
    GROW(s->cellIds, int, s->N > 0 ? s->N : 1);
    GROW(s->nbrStart, int, s->N + 1);
    if (s->nbrCap < 1024) { s->nbrCap = 1024; GROW(s->nbrList, int, s->nbrCap); }
    s->nn_ready = 1;
    return 0;
}

/* updateCellsCPU (src/nn.cpp:8-20): ascending particle id inside a cell. */
static void update_cells(orc *s) {
    int nc = s->ncells;
    memset(s->cellStart, 0, sizeof(int) * (size_t)(nc + 1));
    for (int i = 0; i < s->N; i++) {
        int c = cell_id(s, s->px[i], s->py[i]);
        s->cellOf[i] = c;
        s->cellStart[c + 1]++;
    }
    for (int c = 0; c < nc; c++) s->cellStart[c + 1] += s->cellStart[c];
    int *fill = (int *)malloc(sizeof(int) * (size_t)nc);
    memcpy(fill, s->cellStart, sizeof(int) * (size_t)nc);
    for (int i = 0; i < s->N; i++) s->cellIds[fill[s->cellOf[i]]++] = i;
    free(fill);
}

/* buildNNCPUSerial (src/nn.cpp:22-62) with applyCellBC (src/nnCuda.cu:26-36),
 * which wraps both axes whatever the boundary type. */
static void build_list(orc *s) {
    long long k = 0;
    int wx = (s->pbc == XYPBC || s->pbc == XPBC), wy = (s->pbc == XYPBC);
    for (int pi = 0; pi < s->N; pi++) {
        s->nbrStart[pi] = (int)k;
        int c = s->cellOf[pi];
        int cy0 = c / s->ncx, cx0 = c - cy0 * s->ncx;
        int gi = s->excl[pi];
        for (int cx = -1; cx <= 1; cx++) {
            for (int cy = -1; cy <= 1; cy++) {
                int nx = cx0 + cx, ny = cy0 + cy;
                if (nx < 0) nx = s->ncx - 1; else if (nx == s->ncx) nx = 0;
                if (ny < 0) ny = s->ncy - 1; else if (ny == s->ncy) ny = 0;
                int nc = nx + ny * s->ncx;
                for (int q = s->cellStart[nc]; q < s->cellStart[nc + 1]; q++) {
                    int pj = s->cellIds[q];
                    int gj = s->excl[pj];
                    if (pi != pj && (gi == -1 || gj == -1 || gi != gj)) {
                        float dxr, dyr, dxo, dyo;
                        image_axis(s->px[pi], s->px[pj], s->Lx, wx, 0, &dxr, &dxo);
                        image_axis(s->py[pi], s->py[pj], s->Ly, wy, 0, &dyr, &dyo);
                        float dr2 = dxr * dxr + dyr * dyr;
                        if (dr2 <= s->nnRadiusSq) {
                            if (k >= s->nbrCap) { s->nbrCap *= 2; GROW(s->nbrList, int, s->nbrCap); }
                            s->nbrList[k++] = pj;
                        }
                    }
                }
            }
        }
    }
    s->nbrStart[s->N] = (int)k;
}

void orc_build_nn(orc *s) {
    update_cells(s);
    build_list(s);
}

/* NeighborList::update (src/nn.cpp:114-134) */
void orc_update_nn(orc *s, int restart) {
    if (restart) s->initialUpdate = 1;
    if ((double)s->dispHi > 0.5 * (double)s->skin) {
        s->totalUpdates++;
        s->totalSteps = s->steps - s->initialSteps;
        s->dispHi = 0.0f;
        orc_build_nn(s);
    }
    if (s->initialUpdate) {
        s->totalUpdates = 1;
        s->totalSteps = 0;
        s->initialSteps = s->steps;
        s->initialUpdate = 0;
        s->dispHi = 0.0f;
        orc_build_nn(s);
    }
}

/* ------------------------------------------------------------ FP32 forces */

static void zero_curr_vals(orc *s) {
    s->vvMax = s->kinEneSum = s->potEnergy = 0.0f;
    s->virial = s->feaVirial = 0.0f;
}

/* Integrator::zeroStuff (src/integrator.cpp:146-162) */
void orc_zero_stuff(orc *s) {
    zero_curr_vals(s);
    for (int i = 0; i < s->N; i++) { s->ax[i] = s->ay[i] = 0.0f; s->fx[i] = s->fy[i] = 0.0f; }
}

/* calcBondForcesCPU (src/interactions.cpp:143-173); k = kBond, or E/r0 as in
 * computeBondForcesGPU (src/interactionsCuda.cu:238) when bond_k_mode == 1. */
static void bond_forces(orc *s) {
    int wx = (s->pbc == XYPBC || s->pbc == XPBC), wy = (s->pbc == XYPBC);
    for (int l = 0; l < s->nb; l++) {
        int i = s->bond[2 * l], j = s->bond[2 * l + 1];
        float r0 = s->r0[l];
        float dxr, dyr, dx, dy;
        image_axis(s->px[i], s->px[j], s->Lx, wx, s->image_mode, &dxr, &dx);
        image_axis(s->py[i], s->py[j], s->Ly, wy, s->image_mode, &dyr, &dy);
        float r = sqrtf(dx * dx + dy * dy);
        float deltar = r - r0;
        float k = s->bond_k_mode ? s->E / r0 : s->kBond;
        float kdr = -k * deltar / r;
        float fx = kdr * dx, fy = kdr * dy;
        s->fx[i] += fx; s->fy[i] += fy;
        s->fx[j] -= fx; s->fy[j] -= fy;
        float vir = k * deltar * deltar;
        float u = 0.5f * vir;
        s->potEnergy += u;
    }
}

/* FeaElements::unfoldPos (src/feaElements.cpp:86-151): per-cluster unwrap and
 * centre of mass; feeds feaVirial only. */
static void unfold_pos(orc *s) {
    for (int ei = 0; ei < s->ncl; ei++) {
        float xmin = 100000, xmax = -100000, ymin = 100000, ymax = -100000, xc = 0, yc = 0;
        int off = s->cl[ei].offset, n = s->cl[ei].nv;
        for (int p = 0; p < n; p++) {
            int q = p + off;
            s->unfx[q] = s->px[q]; s->unfy[q] = s->py[q];
            xc += s->unfx[q]; yc += s->unfy[q];
            if (s->unfx[q] < xmin) xmin = s->unfx[q];
            if (xmax < s->unfx[q]) xmax = s->unfx[q];
            if (s->unfy[q] < ymin) ymin = s->unfy[q];
            if (ymax < s->unfy[q]) ymax = s->unfy[q];
        }
        if (xmax - xmin > s->Lx / 2.0f) {
            xc = 0;
            for (int p = 0; p < n; p++) {
                int q = p + off;
                if (s->unfx[q] > s->Lx / 2.0f) s->unfx[q] -= s->Lx;
                xc += s->unfx[q];
            }
            if (xc / (float)n < 0) for (int p = 0; p < n; p++) s->unfx[p + off] += s->Lx;
        }
        if (ymax - ymin > s->Ly / 2.0f) {
            yc = 0;
            for (int p = 0; p < n; p++) {
                int q = p + off;
                if (s->unfy[q] > s->Ly / 2.0f) s->unfy[q] -= s->Ly;
                yc += s->unfy[q];
            }
            if (yc / (float)n < 0) for (int p = 0; p < n; p++) s->unfy[p + off] += s->Ly;
        }
        float vxc = 0, vyc = 0;
        xc = yc = 0;
        for (int p = 0; p < n; p++) {
            int q = p + off;
            float mp = s->mass[q];
            xc += mp * s->unfx[q]; yc += mp * s->unfy[q];
            vxc += mp * s->vx[q]; vyc += mp * s->vy[q];
        }
        s->cl[ei].cmx = xc / s->cl[ei].mass; s->cl[ei].cmy = yc / s->cl[ei].mass;
        s->cl[ei].cvx = vxc / s->cl[ei].mass; s->cl[ei].cvy = vyc / s->cl[ei].mass;
    }
}

/* Per-triangle nodal forces of the neo-Hookean law, calcFeaForcesCPU2
 * (src/interactions.cpp:532-689).  Writes f[6] and the energy pe*vol0. */
static float tri_neo_hookean(const orc *s, int t, float *f) {
    int p0 = s->tri[3 * t], p1 = s->tri[3 * t + 1], p2 = s->tri[3 * t + 2];
    float x0 = s->px[p0], y0 = s->py[p0], x1 = s->px[p1], y1 = s->py[p1], x2 = s->px[p2], y2 = s->py[p2];
    float L = s->Lx, Ly = s->Ly;
    int k1x = 0, k2x = 0, k1y = 0, k2y = 0;
    float dx01 = x0 - x1, dx02 = x0 - x2, dy01 = y0 - y1, dy02 = y0 - y2;
    if (dx01 > L / 2.0f) k1x += 1;
    if (dx01 < -L / 2.0f) k1x -= 1;
    if (dx02 > L / 2.0f) k2x += 1;
    if (dx02 < -L / 2.0f) k2x -= 1;
    if (dy01 > Ly / 2.0f) k1y += 1;
    if (dy01 < -Ly / 2.0f) k1y -= 1;
    if (dy02 > Ly / 2.0f) k2y += 1;
    if (dy02 < -Ly / 2.0f) k2y -= 1;
    float Ds00, Ds10, Ds01, Ds11;
    if (s->image_mode) {
        Ds00 = diff_shift(x0, x2, -k2x, L);
        Ds10 = diff_shift(y0, y2, -k2y, Ly);
        Ds01 = diff_shift(x1, x2, k1x - k2x, L);
        Ds11 = diff_shift(y1, y2, k1y - k2y, Ly);
    } else {
        float r1x = x1, r2x = x2, r1y = y1, r2y = y2;
        if (k1x > 0) r1x += L; if (k1x < 0) r1x -= L;
        if (k2x > 0) r2x += L; if (k2x < 0) r2x -= L;
        if (k1y > 0) r1y += Ly; if (k1y < 0) r1y -= Ly;
        if (k2y > 0) r2y += Ly; if (k2y < 0) r2y -= Ly;
        Ds00 = x0 - r2x; Ds10 = y0 - r2y; Ds01 = r1x - r2x; Ds11 = r1y - r2y;
    }
    float X0 = s->refx[p0], Y0 = s->refy[p0], X1 = s->refx[p1], Y1 = s->refy[p1], X2 = s->refx[p2], Y2 = s->refy[p2];
    float Dm00 = X0 - X2, Dm10 = Y0 - Y2, Dm01 = X1 - X2, Dm11 = Y1 - Y2;
    float detDm = Dm00 * Dm11 - Dm01 * Dm10;
    float vol0 = detDm / 2.0f;
    float Bm00 = Dm11 / detDm, Bm10 = -Dm10 / detDm, Bm01 = -Dm01 / detDm, Bm11 = Dm00 / detDm;
    float F00 = Ds00 * Bm00 + Ds01 * Bm10;
    float F10 = Ds10 * Bm00 + Ds11 * Bm10;
    float F01 = Ds00 * Bm01 + Ds01 * Bm11;
    float F11 = Ds10 * Bm01 + Ds11 * Bm11;
    float detF = F00 * F11 - F01 * F10;
    float logJ = fea_log(s, detF);
    float mu, lambda;
    tri_lame(s, t, &mu, &lambda);
    float llogJ = lambda * logJ;
    float iF00 = F11 / detF, iF10 = -F10 / detF, iF01 = -F01 / detF, iF11 = F00 / detF;
    float P00 = mu * (F00 - iF00) + llogJ * iF00;
    float P10 = mu * (F10 - iF01) + llogJ * iF01;
    float P01 = mu * (F01 - iF10) + llogJ * iF10;
    float P11 = mu * (F11 - iF11) + llogJ * iF11;
    float I1 = F00 * F00 + F10 * F10 + F01 * F01 + F11 * F11;
    float pe = (float)(0.5 * (double)mu * (double)(I1 - 2.0f) - (double)(mu * logJ) +
                       0.5 * (double)lambda * (double)logJ * (double)logJ);
    float nv0 = -vol0;
    float H00 = nv0 * (P00 * Bm00 + P01 * Bm01);
    float H10 = nv0 * (P10 * Bm00 + P11 * Bm01);
    float H01 = nv0 * (P00 * Bm10 + P01 * Bm11);
    float H11 = nv0 * (P10 * Bm10 + P11 * Bm11);
    f[0] = H00; f[1] = H10; f[2] = H01; f[3] = H11;
    f[4] = -f[0] - f[2]; f[5] = -f[1] - f[3];
    return pe * vol0;
}

/* Green strain / linear C law of computeFeaForcesGPU
 * (src/interactionsCuda.cu:312-451), float arithmetic as on the device. */
static float tri_green(const orc *s, int t, float *f) {
    int p[3] = {s->tri[3 * t], s->tri[3 * t + 1], s->tri[3 * t + 2]};
    float rx[3], ry[3], X[3], Y[3];
    for (int i = 0; i < 3; i++) { rx[i] = s->px[p[i]]; ry[i] = s->py[p[i]]; X[i] = s->refx[p[i]]; Y[i] = s->refy[p[i]]; }
    float L = s->Lx, Ly = s->Ly;
    float dx01 = rx[0] - rx[1];
    if (dx01 > L / 2.0f) rx[1] += L;
    if (dx01 < -L / 2.0f) rx[1] -= L;
    float dx02 = rx[0] - rx[2];
    if (dx02 > L / 2.0f) rx[2] += L;
    if (dx02 < -L / 2.0f) rx[2] -= L;
    float dy01 = ry[0] - ry[1];
    if (dy01 > Ly / 2.0f) ry[1] += Ly;
    if (dy01 < -Ly / 2.0f) ry[1] -= Ly;
    float dy02 = ry[0] - ry[2];
    if (dy02 > Ly / 2.0f) ry[2] += Ly;
    if (dy02 < -Ly / 2.0f) ry[2] -= Ly;
    float tetVol = 0.5f * ((Y[2] - Y[0]) * (X[1] - X[0]) - (Y[1] - Y[0]) * (X[2] - X[0]));
    tetVol = fabsf(tetVol);
    float aa[9], mm[9], ux[3], uy[3], a[3], b[3];
    for (int i = 0; i < 3; i++) {
        aa[3 * i] = 1.0f; aa[3 * i + 1] = X[i]; aa[3 * i + 2] = Y[i];
        ux[i] = rx[i] - X[i]; uy[i] = ry[i] - Y[i];
        a[i] = b[i] = 0.0f;
    }
    if (!invert3(aa, mm)) memset(mm, 0, sizeof(mm));
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            a[i] = a[i] + mm[3 * i + j] * ux[j];
            b[i] = b[i] + mm[3 * i + j] * uy[j];
        }
    float e00 = a[1] + 0.5f * (a[1] * a[1] + b[1] * b[1]);
    float e11 = b[2] + 0.5f * (a[2] * a[2] + b[2] * b[2]);
    float e01 = 0.5f * (a[2] + b[1] + a[1] * a[2] + b[1] * b[2]);
    float c1 = s->Cxxxx, c2 = s->Cxxyy, c3 = s->Cxyxy;
    float pesum = c1 * (e00 * e00 + e11 * e11) + 2.0f * c2 * (e00 * e11) + 4.0f * c3 * (e01 * e01);
    float eneVal = pesum * tetVol;
    for (int i = 0; i < 3; i++) {
        float m1 = mm[3 + i], m2 = mm[6 + i];
        float fxs = -2.0f * c1 * e00 * m1 * (1.0f + a[1]) - 2.0f * c1 * e11 * m2 * a[2] - 2.0f * c2 * e00 * m2 * a[2] -
                    2.0f * c2 * e11 * m1 * (1.0f + a[1]) - 4.0f * c3 * e01 * m2 * (1.0f + a[1]) - 4.0f * c3 * e01 * m1 * a[2];
        float fys = -2.0f * c1 * e00 * m1 * b[1] - 2.0f * c1 * e11 * m2 * (1.0f + b[2]) - 2.0f * c2 * e00 * m2 * (1.0f + b[2]) -
                    2.0f * c2 * e11 * m1 * b[1] - 4.0f * c3 * e01 * m1 * (1.0f + b[2]) - 4.0f * c3 * e01 * m2 * b[1];
        f[2 * i] = fxs * tetVol;
        f[2 * i + 1] = fys * tetVol;
    }
    return eneVal;
}

static void fea_forces(orc *s);

/* Interactions::calcFeaForcesCPU1 (src/interactions.cpp:411-530), the
 * reference's CPU twin of the GPU kernel's Green-strain / linear-C law, alone
 * after Integrator::zeroStuff: FEA forces and energy only, with the
 * reference's own mix of precisions -- positions, strains, energy and the
 * scatter in float; the half-box tests against box / 2.0, the area's and
 * e01's halving and the nodal force sums (-2.0 * Cxxxx * ...) in double,
 * rounded to float once.  xm and the reference positions are the setup
 * arrays (src/particles.cpp:340-352); FeaElements::offset is 0
 * (src/feaElements.cpp:9). */
void orc_fea_cpu1(orc *s) {
    orc_zero_stuff(s);
    const float Lx = s->Lx, Ly = s->Ly;
    for (int t = 0; t < s->ntri; t++) {
        int p[3];
        float rx[3], ry[3], X[3], Y[3];
        for (int i = 0; i < 3; i++) {
            p[i] = s->tri[3 * t + i];
            rx[i] = s->px[p[i]]; ry[i] = s->py[p[i]];
            X[i] = s->refx[p[i]]; Y[i] = s->refy[p[i]];
        }
        const float dx01 = rx[0] - rx[1];
        if (dx01 > (double)Lx / 2.0) rx[1] += Lx;
        if (dx01 < -(double)Lx / 2.0) rx[1] -= Lx;
        const float dx02 = rx[0] - rx[2];
        if (dx02 > (double)Lx / 2.0) rx[2] += Lx;
        if (dx02 < -(double)Lx / 2.0) rx[2] -= Lx;
        const float dy01 = ry[0] - ry[1];
        if (dy01 > (double)Ly / 2.0) ry[1] += Ly;
        if (dy01 < -(double)Ly / 2.0) ry[1] -= Ly;
        const float dy02 = ry[0] - ry[2];
        if (dy02 > (double)Ly / 2.0) ry[2] += Ly;
        if (dy02 < -(double)Ly / 2.0) ry[2] -= Ly;
        float vol = (float)(0.5 * (double)((Y[2] - Y[0]) * (X[1] - X[0]) - (Y[1] - Y[0]) * (X[2] - X[0])));
        vol = fabsf(vol);
        const float *m = s->xm + 9 * (size_t)t;
        float ux[3], uy[3], a[3], b[3];
        for (int i = 0; i < 3; i++) { ux[i] = rx[i] - X[i]; uy[i] = ry[i] - Y[i]; a[i] = b[i] = 0.0f; }
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) {
                a[i] = a[i] + m[3 * i + j] * ux[j];
                b[i] = b[i] + m[3 * i + j] * uy[j];
            }
        const float e00 = a[1] + 0.5f * (a[1] * a[1] + b[1] * b[1]);
        const float e11 = b[2] + 0.5f * (a[2] * a[2] + b[2] * b[2]);
        const float e01 = (float)(0.5 * (double)(a[2] + b[1] + a[1] * a[2] + b[1] * b[2]));
        const float c1 = s->Cxxxx, c2 = s->Cxxyy, c3 = s->Cxyxy;
        const float pesum = c1 * (e00 * e00 + e11 * e11) + 2.0f * c2 * (e00 * e11) + 4.0f * c3 * (e01 * e01);
        s->potEnergy += pesum * vol;
        for (int i = 0; i < 3; i++) {
            const int j = p[i];
            const double m1 = m[3 + i], m2 = m[6 + i];
            const float fxsum = (float)(-2.0 * c1 * e00 * m1 * (1.0 + a[1]) - 2.0 * c1 * e11 * m2 * a[2]
                                        - 2.0 * c2 * e00 * m2 * a[2] - 2.0 * c2 * e11 * m1 * (1.0 + a[1])
                                        - 4.0 * c3 * e01 * m2 * (1.0 + a[1]) - 4.0 * c3 * e01 * m1 * a[2]);
            const float fysum = (float)(-2.0 * c1 * e00 * m1 * b[1] - 2.0 * c1 * e11 * m2 * (1.0 + b[2])
                                        - 2.0 * c2 * e00 * m2 * (1.0 + b[2]) - 2.0 * c2 * e11 * m1 * b[1]
                                        - 4.0 * c3 * e01 * m1 * (1.0 + b[2]) - 4.0 * c3 * e01 * m2 * b[1]);
            s->fx[j] += fxsum * vol;
            s->fy[j] += fysum * vol;
        }
    }
}

/* The FEA forces and energy alone, after zeroStuff, by the law in use (the
 * float law of the GPU kernel for fea_law 1), for comparison with
 * orc_fea_cpu1. */
void orc_fea_only(orc *s) {
    orc_zero_stuff(s);
    fea_forces(s);
}

static void fea_forces(orc *s) {
    if (s->ncl > 0) unfold_pos(s);
    for (int t = 0; t < s->ntri; t++) {
        float f[6];
        float e = s->fea_law ? tri_green(s, t, f) : tri_neo_hookean(s, t, f);
        for (int i = 0; i < 3; i++) {
            int j = s->tri[3 * t + i];
            s->fx[j] += f[2 * i];
            s->fy[j] += f[2 * i + 1];
            s->feaVirial += f[2 * i] * s->unfx[j] + f[2 * i + 1] * s->unfy[j];
        }
        s->potEnergy += e;
    }
}

/* pairForce/ljforce (src/interactionsCuda.cu:43-100) for one ordered pair.
 * Returns 1 when inside the cutoff. */
static int lj_pair(const orc *s, int i, int j, float *fxo, float *fyo, float *u, float *vir) {
    int wx = (s->pbc == XYPBC || s->pbc == XPBC), wy = (s->pbc == XYPBC);
    int ti = s->type[i], tj = s->type[j], nt = s->numTypes;
    float eij = s->eps[ti * nt + tj], rcij = s->rc[ti * nt + tj], usij = s->us[ti * nt + tj];
    float sij = (s->sigma[i] + s->sigma[j]) / 2.0f;
    float dxr, dyr, dx, dy;
    image_axis(s->px[i], s->px[j], s->Lx, wx, s->image_mode, &dxr, &dx);
    image_axis(s->py[i], s->py[j], s->Ly, wy, s->image_mode, &dyr, &dy);
    float dr2r = dxr * dxr + dyr * dyr;
    float rcut2 = rcij * rcij * sij * sij;
    if (!(dr2r < rcut2)) return 0;
    float dr2 = dx * dx + dy * dy;
    float c = 48.0f * eij / (sij * sij);
    float dr2i = sij * sij / dr2;
    float dr6i = dr2i * dr2i * dr2i;
    float fc = c * dr6i * (dr6i - 0.5f) * dr2i;
    *fxo = fc * dx;
    *fyo = fc * dy;
    *vir = fc * dr2;
    *u = 4.0f * eij * dr6i * (dr6i - 1.0f) + usij;
    return 1;
}

/* calcPairForcesNN (src/interactions.cpp:347-389), one thread: potential
 * energy and virial accumulate in global pair order as in the reference. */
static void lj_forces(orc *s) {
    if (s->threads <= 1) {
        for (int pi = 0; pi < s->N; pi++) {
            for (int q = s->nbrStart[pi]; q < s->nbrStart[pi + 1]; q++) {
                float fx, fy, u, vir;
                if (lj_pair(s, pi, s->nbrList[q], &fx, &fy, &u, &vir)) {
                    s->fx[pi] += fx; s->fy[pi] += fy;
                    s->potEnergy += u * 0.5f;
                    s->virial += vir * 0.5f;
                } else {
                    s->potEnergy += 0.0f * 0.5f;
                    s->virial += 0.0f * 0.5f;
                }
            }
        }
        return;
    }
    /* threaded timing path: forces identical, energy summed per particle */
#pragma omp parallel for schedule(static) num_threads(s->threads)
    for (int pi = 0; pi < s->N; pi++) {
        float ue = 0.0f, we = 0.0f, fxa = s->fx[pi], fya = s->fy[pi];
        for (int q = s->nbrStart[pi]; q < s->nbrStart[pi + 1]; q++) {
            float fx, fy, u, vir;
            if (lj_pair(s, pi, s->nbrList[q], &fx, &fy, &u, &vir)) {
                fxa += fx; fya += fy; ue += u * 0.5f; we += vir * 0.5f;
            }
        }
        s->fx[pi] = fxa; s->fy[pi] = fya; s->ui[pi] = ue; s->wi[pi] = we;
    }
    for (int pi = 0; pi < s->N; pi++) { s->potEnergy += s->ui[pi]; s->virial += s->wi[pi]; }
}

/* calcAreaForcesCPU (src/interactions.cpp:696-750).  Triangle by triangle
 * in list order, each reading the positions the earlier ones left: r1 and r2
 * moved to r0's side by the half-box rule on both axes (whatever the
 * periodicity), the reference area A0 and the current area A (float products,
 * halved in double), c = -kArea (A - A0) / (2 A0) formed in double and
 * rounded to float, and the vertices displaced -- positions, not forces -- by
 * f1 = c (y2 - y0, -(x2 - x0)), f2 = c (-(y1 - y0), x1 - x0), f0 = -f1 - f2.
 * The energy 1/2 kArea (A - A0)^2 is added in double to the float sum. */
static void area_springs(orc *s) {
    const float Lx = s->Lx, Ly = s->Ly;
    for (int t = 0; t < s->ntri; t++) {
        const int *v = s->tri + 3 * t;
        float rx[3], ry[3], qx[3], qy[3];
        for (int k = 0; k < 3; k++) {
            rx[k] = s->px[v[k]]; ry[k] = s->py[v[k]];
            qx[k] = s->refx[v[k]]; qy[k] = s->refy[v[k]];
        }
        float dx01 = rx[0] - rx[1], dx02 = rx[0] - rx[2];
        if (dx01 > Lx / 2.0) rx[1] += Lx;
        if (dx01 < -Lx / 2.0) rx[1] -= Lx;
        if (dx02 > Lx / 2.0) rx[2] += Lx;
        if (dx02 < -Lx / 2.0) rx[2] -= Lx;
        float dy01 = ry[0] - ry[1], dy02 = ry[0] - ry[2];
        if (dy01 > Ly / 2.0) ry[1] += Ly;
        if (dy01 < -Ly / 2.0) ry[1] -= Ly;
        if (dy02 > Ly / 2.0) ry[2] += Ly;
        if (dy02 < -Ly / 2.0) ry[2] -= Ly;
        float pa = (qy[2] - qy[0]) * (qx[1] - qx[0]), pb = (qy[1] - qy[0]) * (qx[2] - qx[0]);
        float A0 = (float)(0.5 * (float)(pa - pb));
        pa = (ry[2] - ry[0]) * (rx[1] - rx[0]);
        pb = (ry[1] - ry[0]) * (rx[2] - rx[0]);
        float A = (float)(0.5 * (float)(pa - pb));
        float dA = A - A0;
        float c = (float)(-0.5 * (double)s->kArea * (double)dA / (double)A0);
        s->potEnergy = (float)((double)s->potEnergy + 0.5 * (double)s->kArea * (double)dA * (double)dA);
        float f1x = c * (ry[2] - ry[0]), f1y = -c * (rx[2] - rx[0]);
        float f2x = -c * (ry[1] - ry[0]), f2y = c * (rx[1] - rx[0]);
        float fxs[3] = {-f1x - f2x, f1x, f2x}, fys[3] = {-f1y - f2y, f1y, f2y};
        for (int k = 0; k < 3; k++) {
            s->px[v[k]] += fxs[k];
            s->py[v[k]] += fys[k];
        }
    }
}

/* Interactions::calcForces (src/interactions.cpp:83-109): the fixed walls
 * of NOPBC / XPBC boxes, gravity, bonds, FEA, area springs (which move the
 * positions the pair forces then see), pairs, then the moving harmonic walls
 * (no counterpart in the reference). */
void orc_calc_forces(orc *s) {
    ref_wall_forces(s);
    gravity_forces(s);
    if (s->bondForces) bond_forces(s);
    if (s->feaForces) fea_forces(s);
    if (s->areaForces) area_springs(s);
    lj_forces(s);
    wall_forces(s);
}

/* ------------------------------------------------------------ integrator */

static void leapfrog1(orc *s) {
    float dt = s->dt, hdt = 0.5f * dt;
    for (int i = 0; i < s->N; i++) {
        s->vx[i] += hdt * s->ax[i];
        s->vy[i] += hdt * s->ay[i];
        s->px[i] += dt * s->vx[i];
        s->py[i] += dt * s->vy[i];
    }
}

static void apply_pbc(orc *s) {
    for (int i = 0; i < s->N; i++) {
        if (s->pbc == XYPBC) { s->px[i] = wrap_coord(s->px[i], s->Lx); s->py[i] = wrap_coord(s->py[i], s->Ly); }
        else if (s->pbc == XPBC) s->px[i] = wrap_coord(s->px[i], s->Lx);
    }
}

static void update_acc(orc *s) {
    for (int i = 0; i < s->N; i++) { s->ax[i] = s->fx[i] / s->mass[i]; s->ay[i] = s->fy[i] / s->mass[i]; }
}

static void leapfrog2(orc *s) {
    float hdt = 0.5f * s->dt;
    for (int i = 0; i < s->N; i++) { s->vx[i] += hdt * s->ax[i]; s->vy[i] += hdt * s->ay[i]; }
}

/* MDSystem::evalProps (src/md3dsystem.cpp:151-179), CPU branch */
static void eval_props(orc *s) {
    for (int i = 0; i < s->N; i++) {
        s->vv[i] = s->vx[i] * s->vx[i] + s->vy[i] * s->vy[i];
        if (s->vvMax < s->vv[i]) s->vvMax = s->vv[i];
        float kin = s->mass[i] * s->vv[i];
        s->kinEneSum += kin;
    }
    s->dispHi += sqrtf(s->vvMax) * s->dt;
}

/* Integrator::doStep (src/integrator.cpp:8-29) */
void orc_do_step(orc *s) {
    s->steps += 1;
    zero_curr_vals(s);
    leapfrog1(s);
    apply_pbc(s);
    orc_zero_stuff(s);
    orc_update_nn(s, 0);
    orc_calc_forces(s);
    update_acc(s);
    leapfrog2(s);
    eval_props(s);
}

/* Integrator::run (src/integrator.cpp:31-57) */
void orc_run(orc *s, int steps) {
    orc_update_nn(s, 1);
    orc_zero_stuff(s);
    orc_calc_forces(s);
    update_acc(s);
    for (int i = 0; i < steps; i++) orc_do_step(s);
}

/* ------------------------------------------------------- FP64 restatement */

static void image_axis_d(float a, float b, float L, int wraps, double *out) {
    float d = a - b;
    double e = (double)a - (double)b;
    if (wraps) {
        if (d >= 0.5f * L) e -= (double)L;
        else if (d < -0.5f * L) e += (double)L;
    }
    *out = e;
}

/* Condition scales: for every float expression the sum of the magnitudes of
 * its operands, propagated through the formula.  |fp32 - fp64| of a correctly
 * evaluated expression is bounded by a small multiple of eps_f32 times this
 * scale, whatever cancellation the result suffers. */

static double tri_neo_hookean_d(const orc *s, int t, double *f, double *cf, double *cu) {
    int p0 = s->tri[3 * t], p1 = s->tri[3 * t + 1], p2 = s->tri[3 * t + 2];
    float L = s->Lx, Ly = s->Ly;
    float dx01 = s->px[p0] - s->px[p1], dx02 = s->px[p0] - s->px[p2];
    float dy01 = s->py[p0] - s->py[p1], dy02 = s->py[p0] - s->py[p2];
    double r1x = s->px[p1], r2x = s->px[p2], r1y = s->py[p1], r2y = s->py[p2];
    if (dx01 > L / 2.0f) r1x += L; if (dx01 < -L / 2.0f) r1x -= L;
    if (dx02 > L / 2.0f) r2x += L; if (dx02 < -L / 2.0f) r2x -= L;
    if (dy01 > Ly / 2.0f) r1y += Ly; if (dy01 < -Ly / 2.0f) r1y -= Ly;
    if (dy02 > Ly / 2.0f) r2y += Ly; if (dy02 < -Ly / 2.0f) r2y -= Ly;
    double Ds00 = (double)s->px[p0] - r2x, Ds10 = (double)s->py[p0] - r2y, Ds01 = r1x - r2x, Ds11 = r1y - r2y;
    double Dm00 = (double)s->refx[p0] - s->refx[p2], Dm10 = (double)s->refy[p0] - s->refy[p2];
    double Dm01 = (double)s->refx[p1] - s->refx[p2], Dm11 = (double)s->refy[p1] - s->refy[p2];
    double det = Dm00 * Dm11 - Dm01 * Dm10, vol0 = det / 2;
    double B00 = Dm11 / det, B10 = -Dm10 / det, B01 = -Dm01 / det, B11 = Dm00 / det;
    double F00 = Ds00 * B00 + Ds01 * B10, F10 = Ds10 * B00 + Ds11 * B10;
    double F01 = Ds00 * B01 + Ds01 * B11, F11 = Ds10 * B01 + Ds11 * B11;
    double J = F00 * F11 - F01 * F10, lJ = log(J);
    float muf, lamf;
    tri_lame(s, t, &muf, &lamf);
    double lam = lamf, mu = muf;
    double i00 = F11 / J, i10 = -F10 / J, i01 = -F01 / J, i11 = F00 / J;
    double P00 = mu * (F00 - i00) + lam * lJ * i00, P10 = mu * (F10 - i01) + lam * lJ * i01;
    double P01 = mu * (F01 - i10) + lam * lJ * i10, P11 = mu * (F11 - i11) + lam * lJ * i11;
    double I1 = F00 * F00 + F10 * F10 + F01 * F01 + F11 * F11;
    double pe = 0.5 * mu * (I1 - 2) - mu * lJ + 0.5 * lam * lJ * lJ;
    f[0] = -vol0 * (P00 * B00 + P01 * B01);
    f[1] = -vol0 * (P10 * B00 + P11 * B01);
    f[2] = -vol0 * (P00 * B10 + P01 * B11);
    f[3] = -vol0 * (P10 * B10 + P11 * B11);
    f[4] = -f[0] - f[2]; f[5] = -f[1] - f[3];
    /* condition: |F| entries carry |Ds||Bm| (the entries are differences of
     * positions, each with magnitude |x|); P carries mu(|F|+|F^-T|)+|lam lnJ||F^-T| */
    double aF00 = fabs(Ds00) * fabs(B00) + fabs(Ds01) * fabs(B10), aF10 = fabs(Ds10) * fabs(B00) + fabs(Ds11) * fabs(B10);
    double aF01 = fabs(Ds00) * fabs(B01) + fabs(Ds01) * fabs(B11), aF11 = fabs(Ds10) * fabs(B01) + fabs(Ds11) * fabs(B11);
    double al = fabs(lam * lJ) + mu;
    double c00 = mu * aF00 + al * fabs(i00), c10 = mu * aF10 + al * fabs(i01);
    double c01 = mu * aF01 + al * fabs(i10), c11 = mu * aF11 + al * fabs(i11);
    double av = fabs(vol0);
    double h00 = av * (c00 * fabs(B00) + c01 * fabs(B01)), h10 = av * (c10 * fabs(B00) + c11 * fabs(B01));
    double h01 = av * (c00 * fabs(B10) + c01 * fabs(B11)), h11 = av * (c10 * fabs(B10) + c11 * fabs(B11));
    cf[0] = sqrt(h00 * h00 + h10 * h10);
    cf[1] = sqrt(h01 * h01 + h11 * h11);
    cf[2] = cf[0] + cf[1];
    *cu = av * (0.5 * mu * (aF00 * aF00 + aF10 * aF10 + aF01 * aF01 + aF11 * aF11 + 2) + mu * fabs(lJ) + 0.5 * fabs(lam) * lJ * lJ);
    return pe * vol0;
}

static double tri_green_d(const orc *s, int t, double *f, double *cf, double *cu) {
    int p[3] = {s->tri[3 * t], s->tri[3 * t + 1], s->tri[3 * t + 2]};
    float L = s->Lx, Ly = s->Ly;
    double rx[3], ry[3], X[3], Y[3];
    for (int i = 0; i < 3; i++) { rx[i] = s->px[p[i]]; ry[i] = s->py[p[i]]; X[i] = s->refx[p[i]]; Y[i] = s->refy[p[i]]; }
    float dx01 = s->px[p[0]] - s->px[p[1]], dx02 = s->px[p[0]] - s->px[p[2]];
    float dy01 = s->py[p[0]] - s->py[p[1]], dy02 = s->py[p[0]] - s->py[p[2]];
    if (dx01 > L / 2.0f) rx[1] += L; if (dx01 < -L / 2.0f) rx[1] -= L;
    if (dx02 > L / 2.0f) rx[2] += L; if (dx02 < -L / 2.0f) rx[2] -= L;
    if (dy01 > Ly / 2.0f) ry[1] += Ly; if (dy01 < -Ly / 2.0f) ry[1] -= Ly;
    if (dy02 > Ly / 2.0f) ry[2] += Ly; if (dy02 < -Ly / 2.0f) ry[2] -= Ly;
    double vol = fabs(0.5 * ((Y[2] - Y[0]) * (X[1] - X[0]) - (Y[1] - Y[0]) * (X[2] - X[0])));
    double det = (X[1] - X[0]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[1] - Y[0]);
    double gx[3] = {(Y[1] - Y[2]) / det, (Y[2] - Y[0]) / det, (Y[0] - Y[1]) / det};
    double gy[3] = {(X[2] - X[1]) / det, (X[0] - X[2]) / det, (X[1] - X[0]) / det};
    double a1 = 0, a2 = 0, b1 = 0, b2 = 0, A1 = 0, A2 = 0, B1 = 0, B2 = 0;
    for (int j = 0; j < 3; j++) {
        double ux = rx[j] - X[j], uy = ry[j] - Y[j];
        double Ux = fabs(rx[j]) + fabs(X[j]), Uy = fabs(ry[j]) + fabs(Y[j]);
        a1 += gx[j] * ux; a2 += gy[j] * ux; b1 += gx[j] * uy; b2 += gy[j] * uy;
        A1 += fabs(gx[j]) * Ux; A2 += fabs(gy[j]) * Ux; B1 += fabs(gx[j]) * Uy; B2 += fabs(gy[j]) * Uy;
    }
    double e00 = a1 + 0.5 * (a1 * a1 + b1 * b1), e11 = b2 + 0.5 * (a2 * a2 + b2 * b2);
    double e01 = 0.5 * (a2 + b1 + a1 * a2 + b1 * b2);
    double E00 = A1 + 0.5 * (A1 * A1 + B1 * B1), E11 = B2 + 0.5 * (A2 * A2 + B2 * B2);
    double E01 = 0.5 * (A2 + B1 + A1 * A2 + B1 * B2);
    double c1 = s->Cxxxx, c2 = s->Cxxyy, c3 = s->Cxyxy, k1 = fabs(c1), k2 = fabs(c2), k3 = fabs(c3);
    double pes = c1 * (e00 * e00 + e11 * e11) + 2 * c2 * e00 * e11 + 4 * c3 * e01 * e01;
    for (int i = 0; i < 3; i++) {
        double m1 = gx[i], m2 = gy[i], n1 = fabs(m1), n2 = fabs(m2);
        double fxs = -2 * c1 * e00 * m1 * (1 + a1) - 2 * c1 * e11 * m2 * a2 - 2 * c2 * e00 * m2 * a2 - 2 * c2 * e11 * m1 * (1 + a1) -
                     4 * c3 * e01 * m2 * (1 + a1) - 4 * c3 * e01 * m1 * a2;
        double fys = -2 * c1 * e00 * m1 * b1 - 2 * c1 * e11 * m2 * (1 + b2) - 2 * c2 * e00 * m2 * (1 + b2) - 2 * c2 * e11 * m1 * b1 -
                     4 * c3 * e01 * m1 * (1 + b2) - 4 * c3 * e01 * m2 * b1;
        double cx = 2 * k1 * E00 * n1 * (1 + A1) + 2 * k1 * E11 * n2 * A2 + 2 * k2 * E00 * n2 * A2 + 2 * k2 * E11 * n1 * (1 + A1) +
                    4 * k3 * E01 * n2 * (1 + A1) + 4 * k3 * E01 * n1 * A2;
        double cy = 2 * k1 * E00 * n1 * B1 + 2 * k1 * E11 * n2 * (1 + B2) + 2 * k2 * E00 * n2 * (1 + B2) + 2 * k2 * E11 * n1 * B1 +
                    4 * k3 * E01 * n1 * (1 + B2) + 4 * k3 * E01 * n2 * B1;
        f[2 * i] = fxs * vol;
        f[2 * i + 1] = fys * vol;
        cf[i] = sqrt(cx * cx + cy * cy) * vol;
    }
    *cu = vol * (k1 * (E00 * E00 + E11 * E11) + 2 * k2 * E00 * E11 + 4 * k3 * E01 * E01);
    return pes * vol;
}

/* FP64 forces on the current positions and neighbour list.
 * fx, fy: forces; cond: per-particle condition scale of the float force (sum
 * over contributions of their operand magnitudes); ui: per-particle potential
 * energy (bond energy on the bond's first particle, triangle energy 1/3 per
 * vertex, LJ 1/2 per ordered pair); out[0..3] = U, W, condition scales of U
 * and W. */
void orc_forces_f64(const orc *s, double *fx, double *fy, double *cond, double *ui, double *out) {
    int N = s->N;
    int wx = (s->pbc == XYPBC || s->pbc == XPBC), wy = (s->pbc == XYPBC);
    double U = 0, W = 0, Uc = 0, Wc = 0;
    for (int i = 0; i < N; i++) fx[i] = fy[i] = cond[i] = ui[i] = 0;
    if (!s->wallOn && s->pbc != XYPBC) {
        /* the reference's fixed walls; contact decisions from the float path.
         * Condition: the LJ wall force varies like d^-19 with the float
         * distance d = L - y, so its scale carries 20 (L + |y|) / d. */
        float rc = (float)pow(2.0, 1.0 / 6.0);
        for (int i = 0; i < N; i++) {
            float s0 = s->sigma[i];
            double sd = s0;
            for (int ax = 0; ax < (s->pbc == NOPBC ? 2 : 1); ax++) {
                float p = ax == 0 ? s->py[i] : s->px[i], L = ax == 0 ? s->Ly : s->Lx;
                double *fa = ax == 0 ? fy : fx;
                double d = 0, sign = 0;
                if ((L - p) < s0 * rc) { d = (double)L - p; sign = -1; }
                else if (p < s0 * rc) { d = p; sign = 1; }
                if (sign == 0) continue;
                double f, u;
                if (s->pbc == NOPBC) {
                    double z = sd / d, z3 = z * z * z, z6 = z3 * z3 * z3;
                    u = 4 * z6 * (z6 - 1) + 1;
                    f = fabs(48 * z6 * (z6 - 0.5) / z);
                    cond[i] += f * (1 + 20 * ((double)L + fabs((double)p)) / d);
                    Uc += fabs(u) * (1 + 20 * ((double)L + fabs((double)p)) / d);
                } else {
                    f = (double)s->kWall * d;
                    u = 0.5 * s->kWall * d * d;
                    cond[i] += fabs((double)s->kWall) * ((double)L + fabs((double)p));
                    Uc += u;
                }
                fa[i] += sign * f;
                ui[i] += u;
                U += u;
            }
        }
    }
    if (s->gravityForce && s->gravity > 0)
        for (int i = 0; i < N; i++) { fy[i] -= (double)s->mass[i] * s->gravity; cond[i] += fabs((double)s->mass[i] * s->gravity); }
    if (s->bondForces) {
        for (int l = 0; l < s->nb; l++) {
            int i = s->bond[2 * l], j = s->bond[2 * l + 1];
            double dx, dy;
            image_axis_d(s->px[i], s->px[j], s->Lx, wx, &dx);
            image_axis_d(s->py[i], s->py[j], s->Ly, wy, &dy);
            double r = sqrt(dx * dx + dy * dy), r0 = s->r0[l], dl = r - r0;
            double k = s->bond_k_mode ? (double)s->E / r0 : (double)s->kBond;
            double kdr = -k * dl / r, f1 = kdr * dx, f2 = kdr * dy;
            fx[i] += f1; fy[i] += f2; fx[j] -= f1; fy[j] -= f2;
            double c = fabs(k) * (r + r0) + fabs(kdr) * r;
            cond[i] += c; cond[j] += c;
            double u = 0.5 * k * dl * dl;
            U += u; Uc += 0.5 * fabs(k) * (r + r0) * (r + r0); ui[i] += u;
        }
    }
    if (s->feaForces) {
        for (int t = 0; t < s->ntri; t++) {
            double f[6], cf[3], cu;
            double e = s->fea_law ? tri_green_d(s, t, f, cf, &cu) : tri_neo_hookean_d(s, t, f, cf, &cu);
            for (int i = 0; i < 3; i++) {
                int j = s->tri[3 * t + i];
                fx[j] += f[2 * i]; fy[j] += f[2 * i + 1];
                cond[j] += cf[i];
                ui[j] += e / 3.0;
            }
            U += e; Uc += cu;
        }
    }
    for (int pi = 0; pi < N; pi++) {
        for (int q = s->nbrStart[pi]; q < s->nbrStart[pi + 1]; q++) {
            int pj = s->nbrList[q];
            int ti = s->type[pi], tj = s->type[pj], nt = s->numTypes;
            float sijf = (s->sigma[pi] + s->sigma[pj]) / 2.0f;
            float rcij = s->rc[ti * nt + tj];
            float dxr, dyr, dxo, dyo;
            image_axis(s->px[pi], s->px[pj], s->Lx, wx, 0, &dxr, &dxo);
            image_axis(s->py[pi], s->py[pj], s->Ly, wy, 0, &dyr, &dyo);
            if (!(dxr * dxr + dyr * dyr < rcij * rcij * sijf * sijf)) continue;
            double dx, dy;
            image_axis_d(s->px[pi], s->px[pj], s->Lx, wx, &dx);
            image_axis_d(s->py[pi], s->py[pj], s->Ly, wy, &dy);
            double eij = s->eps[ti * nt + tj], sij = 0.5 * ((double)s->sigma[pi] + (double)s->sigma[pj]);
            double dr2 = dx * dx + dy * dy, c = 48.0 * eij / (sij * sij), d2i = sij * sij / dr2;
            double d6i = d2i * d2i * d2i, fc = c * d6i * (d6i - 0.5) * d2i;
            fx[pi] += fc * dx; fy[pi] += fc * dy;
            double fcc = fabs(c) * d6i * (d6i + 0.5) * d2i;
            cond[pi] += fcc * sqrt(dr2);
            double u = 4.0 * eij * d6i * (d6i - 1.0) + (double)s->us[ti * nt + tj];
            U += 0.5 * u; Uc += 0.5 * (4.0 * fabs(eij) * d6i * (d6i + 1.0) + fabs((double)s->us[ti * nt + tj]));
            ui[pi] += 0.5 * u;
            W += 0.5 * fc * dr2; Wc += 0.5 * fcc * dr2;
        }
    }
    if (s->wallOn) {
        double yw = wall_y(s), range = wall_range();
        for (int i = 0; i < N; i++) {
            double dl = range * (double)s->sigma[i], y = s->py[i], k = s->wallK;
            double ht = (y + dl) - yw, hb = dl - y;
            if (ht > 0) { fy[i] -= k * ht; ui[i] += 0.5 * k * ht * ht; U += 0.5 * k * ht * ht;
                          cond[i] += k * (fabs(y) + dl + fabs(yw)); Uc += 0.5 * k * ht * ht; }
            if (hb > 0) { fy[i] += k * hb; ui[i] += 0.5 * k * hb * hb; U += 0.5 * k * hb * hb;
                          cond[i] += k * (fabs(y) + dl); Uc += 0.5 * k * hb * hb; }
        }
    }
    out[0] = U; out[1] = W; out[2] = Uc; out[3] = Wc;
}

/* ------------------------------------------------------------- accessors */

int orc_n(const orc *s) { return s->N; }
int orc_nbonds(const orc *s) { return s->nb; }
int orc_ntri(const orc *s) { return s->ntri; }
int orc_ncl(const orc *s) { return s->ncl; }
int orc_nref(const orc *s) { return s->ncl > 0 ? s->ncl * s->cl[0].nv : 0; }
int orc_steps(const orc *s) { return s->steps; }
int orc_total_updates(const orc *s) { return s->totalUpdates; }
int orc_ncells(const orc *s) { return s->ncells; }
void orc_grid(const orc *s, int *ncx, int *ncy) { *ncx = s->ncx; *ncy = s->ncy; }
long long orc_nbr_total(const orc *s) { return s->nn_ready ? s->nbrStart[s->N] : 0; }
float orc_disp_hi(const orc *s) { return s->dispHi; }

/* scalars: potEnergy, virial, feaVirial, kinEneSum, vvMax, dispHi */
void orc_scalars(const orc *s, float *out) {
    out[0] = s->potEnergy; out[1] = s->virial; out[2] = s->feaVirial;
    out[3] = s->kinEneSum; out[4] = s->vvMax; out[5] = s->dispHi;
}

static void pack2(const float *a, const float *b, int n, float *out) {
    for (int i = 0; i < n; i++) { out[2 * i] = a[i]; out[2 * i + 1] = b[i]; }
}

void orc_get_pos(const orc *s, float *o) { pack2(s->px, s->py, s->N, o); }
void orc_get_vel(const orc *s, float *o) { pack2(s->vx, s->vy, s->N, o); }
void orc_get_acc(const orc *s, float *o) { pack2(s->ax, s->ay, s->N, o); }
void orc_get_force(const orc *s, float *o) { pack2(s->fx, s->fy, s->N, o); }
void orc_get_refpos(const orc *s, float *o) { pack2(s->refx, s->refy, s->N, o); }
void orc_get_mass(const orc *s, float *o) { memcpy(o, s->mass, sizeof(float) * (size_t)s->N); }
void orc_get_excl(const orc *s, int *o) { memcpy(o, s->excl, sizeof(int) * (size_t)s->N); }
void orc_get_bonds(const orc *s, int *ij, float *r0) {
    memcpy(ij, s->bond, sizeof(int) * 2 * (size_t)s->nb);
    memcpy(r0, s->r0, sizeof(float) * (size_t)s->nb);
}
void orc_get_tris(const orc *s, int *t, float *xm, float *vol) {
    memcpy(t, s->tri, sizeof(int) * 3 * (size_t)s->ntri);
    memcpy(xm, s->xm, sizeof(float) * 9 * (size_t)s->ntri);
    memcpy(vol, s->refVol, sizeof(float) * (size_t)s->ntri);
}
void orc_get_cells(const orc *s, int *start, int *ids) {
    memcpy(start, s->cellStart, sizeof(int) * (size_t)(s->ncells + 1));
    memcpy(ids, s->cellIds, sizeof(int) * (size_t)s->N);
}
void orc_get_nbrs(const orc *s, int *start, int *list) {
    memcpy(start, s->nbrStart, sizeof(int) * (size_t)(s->N + 1));
    memcpy(list, s->nbrList, sizeof(int) * (size_t)s->nbrStart[s->N]);
}
void orc_set_pos(orc *s, const float *p) {
    for (int i = 0; i < s->N; i++) { s->px[i] = p[2 * i]; s->py[i] = p[2 * i + 1]; }
}
void orc_set_vel(orc *s, const float *v) {
    for (int i = 0; i < s->N; i++) { s->vx[i] = v[2 * i]; s->vy[i] = v[2 * i + 1]; }
}
float orc_logf_own(float x) { return own_logf(x); }

/* ================================================ FP64 trajectory and adjoint
 *
 * An independent double-precision engine for checking gradients: the same
 * physics (harmonic bonds with constant kBond, neo-Hookean triangles with
 * per-elastomer E and nu, Lennard-Jones pairs between particles of different
 * exclusion groups, harmonic walls, kick-drift-kick leapfrog) on double
 * state, with pairs found by a fresh cell search at every force evaluation
 * (no Verlet list, so no list decisions are shared with the float path).
 * Parameters are doubles: per-elastomer (E, nu), one scale on every pair
 * epsilon and one on every particle sigma.  orc_d_backward is the discrete
 * adjoint of orc_d_forward written out by hand; central differences of
 * orc_d_forward check it. */

typedef struct {
    int N, ntri, nb, ncl, steps;
    double dt, Lx, Ly;
    int wx, wy;
    double *x, *v, *m, *sig;     /* 2N, 2N, N, N */
    int *type, *excl;
    double *E, *nu;              /* per elastomer */
    int *triCl;                  /* elastomer of each triangle */
    double *B, *vol0;            /* 4 per triangle (Bm00, Bm10, Bm01, Bm11), 1 per triangle */
    double epsScale, sigScale;
    double *traj;                /* (steps+1) x 2N positions */
    double *f, *a, *w, *g;       /* scratch 2N */
    int *cstart, *cids, *ccell;  /* cell search scratch */
    int ncx, ncy;
} orc_d;

static orc_d D_;  /* one engine per process (test infrastructure) */

static double d_img(double d, double L, int wrap) {
    if (wrap) {
        if (d >= 0.5 * L) d -= L;
        else if (d < -0.5 * L) d += L;
    }
    return d;
}

void orc_d_init(const orc *s) {
    orc_d *d = &D_;
    free(d->x); free(d->v); free(d->m); free(d->sig); free(d->type); free(d->excl); free(d->E); free(d->nu);
    free(d->triCl); free(d->B); free(d->vol0); free(d->traj); free(d->f); free(d->a); free(d->w); free(d->g);
    free(d->cstart); free(d->cids); free(d->ccell);
    memset(d, 0, sizeof *d);
    int N = s->N;
    d->N = N; d->ntri = s->ntri; d->nb = s->nb; d->ncl = s->ncl;
    d->dt = s->dt; d->Lx = s->Lx; d->Ly = s->Ly;
    d->wx = (s->pbc == XYPBC || s->pbc == XPBC); d->wy = (s->pbc == XYPBC);
    d->x = (double *)calloc(2 * (size_t)N + 2, sizeof(double));
    d->v = (double *)calloc(2 * (size_t)N + 2, sizeof(double));
    d->m = (double *)calloc((size_t)N + 1, sizeof(double));
    d->sig = (double *)calloc((size_t)N + 1, sizeof(double));
    d->type = (int *)calloc((size_t)N + 1, sizeof(int));
    d->excl = (int *)calloc((size_t)N + 1, sizeof(int));
    for (int i = 0; i < N; i++) {
        d->x[2 * i] = s->px[i]; d->x[2 * i + 1] = s->py[i];
        d->v[2 * i] = s->vx[i]; d->v[2 * i + 1] = s->vy[i];
        d->m[i] = s->mass[i]; d->sig[i] = s->sigma[i]; d->type[i] = s->type[i]; d->excl[i] = s->excl[i];
    }
    d->E = (double *)calloc((size_t)d->ncl + 1, sizeof(double));
    d->nu = (double *)calloc((size_t)d->ncl + 1, sizeof(double));
    for (int e = 0; e < d->ncl; e++) {
        int own = s->clOwn && e < s->clMatCap && s->clOwn[e];
        d->E[e] = own ? s->clE[e] : s->E;
        d->nu[e] = own ? s->clNu[e] : s->nu;
    }
    d->triCl = (int *)calloc((size_t)d->ntri + 1, sizeof(int));
    d->B = (double *)calloc(4 * (size_t)d->ntri + 4, sizeof(double));
    d->vol0 = (double *)calloc((size_t)d->ntri + 1, sizeof(double));
    for (int t = 0; t < d->ntri; t++) {
        int p0 = s->tri[3 * t], p1 = s->tri[3 * t + 1], p2 = s->tri[3 * t + 2];
        d->triCl[t] = s->cluster[p0];
        double Dm00 = (double)s->refx[p0] - s->refx[p2], Dm10 = (double)s->refy[p0] - s->refy[p2];
        double Dm01 = (double)s->refx[p1] - s->refx[p2], Dm11 = (double)s->refy[p1] - s->refy[p2];
        double det = Dm00 * Dm11 - Dm01 * Dm10;
        d->B[4 * t] = Dm11 / det; d->B[4 * t + 1] = -Dm10 / det; d->B[4 * t + 2] = -Dm01 / det; d->B[4 * t + 3] = Dm00 / det;
        d->vol0[t] = det / 2;
    }
    d->epsScale = 1; d->sigScale = 1;
    d->f = (double *)calloc(2 * (size_t)N + 2, sizeof(double));
    d->a = (double *)calloc(2 * (size_t)N + 2, sizeof(double));
    d->w = (double *)calloc(2 * (size_t)N + 2, sizeof(double));
    d->g = (double *)calloc(2 * (size_t)N + 2, sizeof(double));
    d->ccell = (int *)calloc((size_t)N + 1, sizeof(int));
    d->cids = (int *)calloc((size_t)N + 1, sizeof(int));
}

void orc_d_set_material(int e, double E, double nu) { if (e >= 0 && e < D_.ncl) { D_.E[e] = E; D_.nu[e] = nu; } }
void orc_d_set_scales(double eps_scale, double sig_scale) { D_.epsScale = eps_scale; D_.sigScale = sig_scale; }
void orc_d_set_state(const double *x, const double *v) {
    memcpy(D_.x, x, sizeof(double) * 2 * (size_t)D_.N);
    memcpy(D_.v, v, sizeof(double) * 2 * (size_t)D_.N);
}
void orc_d_get_state(double *x, double *v) {
    memcpy(x, D_.x, sizeof(double) * 2 * (size_t)D_.N);
    memcpy(v, D_.v, sizeof(double) * 2 * (size_t)D_.N);
}

static void d_lame(double E, double nu, double *mu, double *la) {
    *la = E * nu / ((1 - 2 * nu) * (1 + nu));
    *mu = E / (2 * (1 + nu));
}

/* cell search over the positions x (cells of at least the largest cutoff) */
static void d_cells(const orc *s, const double *x) {
    orc_d *d = &D_;
    double rmax = 0;
    for (int k = 0; k < s->numTypes * s->numTypes; k++) if (s->rc[k] > rmax) rmax = s->rc[k];
    double smax = 0;
    for (int i = 0; i < d->N; i++) if (d->sig[i] > smax) smax = d->sig[i];
    double cut = rmax * smax * d->sigScale;
    d->ncx = (int)floor(d->Lx / cut); d->ncy = (int)floor(d->Ly / cut);
    if (d->ncx < 1) d->ncx = 1;
    if (d->ncy < 1) d->ncy = 1;
    int nc = d->ncx * d->ncy;
    free(d->cstart);
    d->cstart = (int *)calloc((size_t)nc + 1, sizeof(int));
    for (int i = 0; i < d->N; i++) {
        int ix = (int)floor(x[2 * i] / d->Lx * d->ncx), iy = (int)floor(x[2 * i + 1] / d->Ly * d->ncy);
        ix = ix < 0 ? 0 : ix >= d->ncx ? d->ncx - 1 : ix;
        iy = iy < 0 ? 0 : iy >= d->ncy ? d->ncy - 1 : iy;
        d->ccell[i] = ix + iy * d->ncx;
        d->cstart[d->ccell[i] + 1]++;
    }
    for (int c = 0; c < nc; c++) d->cstart[c + 1] += d->cstart[c];
    int *fill = (int *)calloc((size_t)nc, sizeof(int));
    for (int i = 0; i < d->N; i++) d->cids[d->cstart[d->ccell[i]] + fill[d->ccell[i]]++] = i;
    free(fill);
}

/* Forces at x (into f, 2N); with w != NULL instead the directional
 * derivative of the forces along w (into f) and the parameter terms
 * w . df/dtheta accumulated into gMu/gLam (per elastomer), ge, gs. */
static void d_forces(const orc *s, const double *x, double *f, const double *w, int step, double *gMu, double *gLam,
                     double *ge, double *gs) {
    orc_d *d = &D_;
    int N = d->N;
    for (int k = 0; k < 2 * N; k++) f[k] = 0;
    /* bonds */
    if (s->bondForces) {
        for (int l = 0; l < d->nb; l++) {
            int i = s->bond[2 * l], j = s->bond[2 * l + 1];
            double dx = d_img(x[2 * i] - x[2 * j], d->Lx, d->wx), dy = d_img(x[2 * i + 1] - x[2 * j + 1], d->Ly, d->wy);
            double r = sqrt(dx * dx + dy * dy), r0 = s->r0[l], k = s->kBond;
            double kdr = -k * (r - r0) / r;
            double f1, f2;
            if (!w) { f1 = kdr * dx; f2 = kdr * dy; }
            else {
                double ddx = w[2 * i] - w[2 * j], ddy = w[2 * i + 1] - w[2 * j + 1];
                double dr = (dx * ddx + dy * ddy) / r, dk = -k * r0 * dr / (r * r);
                f1 = dk * dx + kdr * ddx; f2 = dk * dy + kdr * ddy;
            }
            f[2 * i] += f1; f[2 * i + 1] += f2; f[2 * j] -= f1; f[2 * j + 1] -= f2;
        }
    }
    /* neo-Hookean triangles */
    if (s->feaForces) {
        for (int t = 0; t < d->ntri; t++) {
            int p[3] = {s->tri[3 * t], s->tri[3 * t + 1], s->tri[3 * t + 2]};
            double mu, la;
            d_lame(d->E[d->triCl[t]], d->nu[d->triCl[t]], &mu, &la);
            double Ds00 = d_img(x[2 * p[0]] - x[2 * p[2]], d->Lx, d->wx), Ds10 = d_img(x[2 * p[0] + 1] - x[2 * p[2] + 1], d->Ly, d->wy);
            double Ds01 = d_img(x[2 * p[1]] - x[2 * p[2]], d->Lx, d->wx), Ds11 = d_img(x[2 * p[1] + 1] - x[2 * p[2] + 1], d->Ly, d->wy);
            const double *B = d->B + 4 * t;
            double F00 = Ds00 * B[0] + Ds01 * B[1], F10 = Ds10 * B[0] + Ds11 * B[1];
            double F01 = Ds00 * B[2] + Ds01 * B[3], F11 = Ds10 * B[2] + Ds11 * B[3];
            double J = F00 * F11 - F01 * F10, lJ = log(J);
            double i00 = F11 / J, i10 = -F10 / J, i01 = -F01 / J, i11 = F00 / J;
            double nv = -d->vol0[t];
            double P00, P10, P01, P11;
            if (!w) {
                P00 = mu * (F00 - i00) + la * lJ * i00; P10 = mu * (F10 - i01) + la * lJ * i01;
                P01 = mu * (F01 - i10) + la * lJ * i10; P11 = mu * (F11 - i11) + la * lJ * i11;
            } else {
                double e00 = w[2 * p[0]] - w[2 * p[2]], e10 = w[2 * p[0] + 1] - w[2 * p[2] + 1];
                double e01 = w[2 * p[1]] - w[2 * p[2]], e11 = w[2 * p[1] + 1] - w[2 * p[2] + 1];
                double dF00 = e00 * B[0] + e01 * B[1], dF10 = e10 * B[0] + e11 * B[1];
                double dF01 = e00 * B[2] + e01 * B[3], dF11 = e10 * B[2] + e11 * B[3];
                double dJ = dF00 * F11 + F00 * dF11 - dF01 * F10 - F01 * dF10, dlJ = dJ / J;
                /* d(F^-1) = -F^-1 dF F^-1 */
                double t00 = i00 * dF00 + i01 * dF10, t01 = i00 * dF01 + i01 * dF11;
                double t10 = i10 * dF00 + i11 * dF10, t11 = i10 * dF01 + i11 * dF11;
                double di00 = -(t00 * i00 + t01 * i10), di01 = -(t00 * i01 + t01 * i11);
                double di10 = -(t10 * i00 + t11 * i10), di11 = -(t10 * i01 + t11 * i11);
                P00 = mu * (dF00 - di00) + la * dlJ * i00 + la * lJ * di00;
                P10 = mu * (dF10 - di01) + la * dlJ * i01 + la * lJ * di01;
                P01 = mu * (dF01 - di10) + la * dlJ * i10 + la * lJ * di10;
                P11 = mu * (dF11 - di11) + la * dlJ * i11 + la * lJ * di11;
                /* w . f_mu, w . f_lambda */
                double Hm00 = nv * ((F00 - i00) * B[0] + (F01 - i10) * B[2]), Hm10 = nv * ((F10 - i01) * B[0] + (F11 - i11) * B[2]);
                double Hm01 = nv * ((F00 - i00) * B[1] + (F01 - i10) * B[3]), Hm11 = nv * ((F10 - i01) * B[1] + (F11 - i11) * B[3]);
                double Hl00 = nv * lJ * (i00 * B[0] + i10 * B[2]), Hl10 = nv * lJ * (i01 * B[0] + i11 * B[2]);
                double Hl01 = nv * lJ * (i00 * B[1] + i10 * B[3]), Hl11 = nv * lJ * (i01 * B[1] + i11 * B[3]);
                int e = d->triCl[t];
                gMu[e] += e00 * Hm00 + e10 * Hm10 + e01 * Hm01 + e11 * Hm11;
                gLam[e] += e00 * Hl00 + e10 * Hl10 + e01 * Hl01 + e11 * Hl11;
            }
            double H00 = nv * (P00 * B[0] + P01 * B[2]), H10 = nv * (P10 * B[0] + P11 * B[2]);
            double H01 = nv * (P00 * B[1] + P01 * B[3]), H11 = nv * (P10 * B[1] + P11 * B[3]);
            f[2 * p[0]] += H00; f[2 * p[0] + 1] += H10;
            f[2 * p[1]] += H01; f[2 * p[1] + 1] += H11;
            f[2 * p[2]] -= H00 + H01; f[2 * p[2] + 1] -= H10 + H11;
        }
    }
    /* Lennard-Jones pairs by cell search */
    d_cells(s, x);
    int nt = s->numTypes;
    for (int i = 0; i < N; i++) {
        int c = d->ccell[i], cx = c % d->ncx, cy = c / d->ncx;
        int seen[9], ns = 0;
        for (int ox = -1; ox <= 1; ox++)
            for (int oy = -1; oy <= 1; oy++) {
                int nx = (cx + ox + d->ncx) % d->ncx, ny = (cy + oy + d->ncy) % d->ncy, nc = nx + ny * d->ncx, dup = 0;
                for (int q = 0; q < ns; q++) dup |= seen[q] == nc;
                if (dup) continue;
                seen[ns++] = nc;
                for (int q = d->cstart[nc]; q < d->cstart[nc + 1]; q++) {
                    int j = d->cids[q];
                    if (j == i) continue;
                    if (d->excl[i] != -1 && d->excl[i] == d->excl[j]) continue;
                    double dx = d_img(x[2 * i] - x[2 * j], d->Lx, d->wx), dy = d_img(x[2 * i + 1] - x[2 * j + 1], d->Ly, d->wy);
                    int tt = d->type[i] * nt + d->type[j];
                    double sij = 0.5 * (d->sig[i] + d->sig[j]) * d->sigScale, rc = s->rc[tt], eps = s->eps[tt] * d->epsScale;
                    double dr2 = dx * dx + dy * dy;
                    if (!(dr2 < rc * rc * sij * sij)) continue;
                    double s2 = sij * sij / dr2, s6 = s2 * s2 * s2, c48 = 48.0 * eps / (sij * sij);
                    double fc = c48 * s6 * (s6 - 0.5) * s2;
                    if (!w) { f[2 * i] += fc * dx; f[2 * i + 1] += fc * dy; }
                    else {
                        double cs2 = c48 * s2, dfc = -(cs2 / dr2) * (7 * s6 * s6 - 2 * s6);
                        double ddx = w[2 * i] - w[2 * j], ddy = w[2 * i + 1] - w[2 * j + 1], dot = dx * ddx + dy * ddy;
                        f[2 * i] += fc * ddx + 2 * dfc * dot * dx;
                        f[2 * i + 1] += fc * ddy + 2 * dfc * dot * dy;
                        *ge += w[2 * i] * fc * dx + w[2 * i + 1] * fc * dy;
                        double fs = cs2 * (12 * s6 * s6 - 3 * s6);
                        *gs += w[2 * i] * fs * dx + w[2 * i + 1] * fs * dy;
                    }
                }
            }
    }
    /* walls */
    if (s->wallOn) {
        double yw = (double)s->wallY0 - (double)s->wallV * (step * d->dt), k = s->wallK;
        double range = pow(2.0, 1.0 / 6.0);
        for (int i = 0; i < N; i++) {
            double dl = range * d->sig[i] * d->sigScale, y = x[2 * i + 1];
            double ht = (y + dl) - yw, hb = dl - y;
            if (!w) {
                if (ht > 0) f[2 * i + 1] -= k * ht;
                if (hb > 0) f[2 * i + 1] += k * hb;
            } else {
                if (ht > 0) { f[2 * i + 1] -= k * w[2 * i + 1]; *gs += w[2 * i + 1] * (-k * dl); }
                if (hb > 0) { f[2 * i + 1] -= k * w[2 * i + 1]; *gs += w[2 * i + 1] * (k * dl); }
            }
        }
    }
}

/* observable J = cWall (F_top + F_bottom) / (2 Lx) + cFea U_fea at x (step n) */
static double d_observable(const orc *s, const double *x, int n, double cWall, double cFea) {
    orc_d *d = &D_;
    double J = 0;
    if (s->wallOn && cWall != 0) {
        double yw = (double)s->wallY0 - (double)s->wallV * (n * d->dt), k = s->wallK, range = pow(2.0, 1.0 / 6.0), F = 0;
        for (int i = 0; i < d->N; i++) {
            double dl = range * d->sig[i] * d->sigScale, y = x[2 * i + 1];
            if ((y + dl) - yw > 0) F += k * ((y + dl) - yw);
            if (dl - y > 0) F += k * (dl - y);
        }
        J += cWall * F / (2 * d->Lx);
    }
    if (s->feaForces && cFea != 0) {
        for (int t = 0; t < d->ntri; t++) {
            int p[3] = {s->tri[3 * t], s->tri[3 * t + 1], s->tri[3 * t + 2]};
            double mu, la;
            d_lame(d->E[d->triCl[t]], d->nu[d->triCl[t]], &mu, &la);
            double Ds00 = d_img(x[2 * p[0]] - x[2 * p[2]], d->Lx, d->wx), Ds10 = d_img(x[2 * p[0] + 1] - x[2 * p[2] + 1], d->Ly, d->wy);
            double Ds01 = d_img(x[2 * p[1]] - x[2 * p[2]], d->Lx, d->wx), Ds11 = d_img(x[2 * p[1] + 1] - x[2 * p[2] + 1], d->Ly, d->wy);
            const double *B = d->B + 4 * t;
            double F00 = Ds00 * B[0] + Ds01 * B[1], F10 = Ds10 * B[0] + Ds11 * B[1];
            double F01 = Ds00 * B[2] + Ds01 * B[3], F11 = Ds10 * B[2] + Ds11 * B[3];
            double lJ = log(F00 * F11 - F01 * F10), I1 = F00 * F00 + F10 * F10 + F01 * F01 + F11 * F11;
            J += cFea * d->vol0[t] * (0.5 * mu * (I1 - 2) - mu * lJ + 0.5 * la * lJ * lJ);
        }
    }
    return J;
}

/* FP64 run of 'steps' kick-drift-kick steps from the engine state, starting
 * at step index n0 (the wall clock); keeps every position set.  Returns J at
 * the final positions. */
double orc_d_forward(const orc *s, int n0, int steps, double cWall, double cFea) {
    orc_d *d = &D_;
    int N = d->N;
    d->steps = steps;
    free(d->traj);
    d->traj = (double *)malloc(sizeof(double) * 2 * (size_t)N * (size_t)(steps + 1));
    double h = 0.5 * d->dt;
    memcpy(d->traj, d->x, sizeof(double) * 2 * (size_t)N);
    d_forces(s, d->x, d->f, NULL, n0, NULL, NULL, NULL, NULL);
    for (int i = 0; i < N; i++) { d->a[2 * i] = d->f[2 * i] / d->m[i]; d->a[2 * i + 1] = d->f[2 * i + 1] / d->m[i]; }
    for (int n = 0; n < steps; n++) {
        for (int k = 0; k < 2 * N; k++) { d->v[k] += h * d->a[k]; d->x[k] += d->dt * d->v[k]; }
        for (int i = 0; i < N; i++) {
            if (d->wx) d->x[2 * i] -= floor(d->x[2 * i] / d->Lx) * d->Lx;
            if (d->wy) d->x[2 * i + 1] -= floor(d->x[2 * i + 1] / d->Ly) * d->Ly;
        }
        memcpy(d->traj + 2 * (size_t)N * (n + 1), d->x, sizeof(double) * 2 * (size_t)N);
        d_forces(s, d->x, d->f, NULL, n0 + n + 1, NULL, NULL, NULL, NULL);
        for (int i = 0; i < N; i++) { d->a[2 * i] = d->f[2 * i] / d->m[i]; d->a[2 * i + 1] = d->f[2 * i + 1] / d->m[i]; }
        for (int k = 0; k < 2 * N; k++) d->v[k] += h * d->a[k];
    }
    return d_observable(s, d->x, n0 + steps, cWall, cFea);
}

/* Replace the stored trajectory by (steps + 1) given position sets, e.g. a
 * float run's, so that orc_d_backward differentiates along it in double. */
void orc_d_set_traj(const double *traj, int steps) {
    orc_d *d = &D_;
    free(d->traj);
    size_t n = 2 * (size_t)d->N * (size_t)(steps + 1);
    d->traj = (double *)malloc(sizeof(double) * n);
    memcpy(d->traj, traj, sizeof(double) * n);
    d->steps = steps;
}

/* dJ/dx at x by central differences would be slow; the observable's
 * gradient is formed analytically: walls and -f_fea. */
static void d_obs_grad(const orc *s, const double *x, int n, double cWall, double cFea, double *gx, double *gMu,
                       double *gLam, double *gs) {
    orc_d *d = &D_;
    int N = d->N;
    for (int k = 0; k < 2 * N; k++) gx[k] = 0;
    if (s->wallOn && cWall != 0) {
        double yw = (double)s->wallY0 - (double)s->wallV * (n * d->dt), k = s->wallK, range = pow(2.0, 1.0 / 6.0);
        double a = cWall * k / (2 * d->Lx);
        for (int i = 0; i < N; i++) {
            double dl = range * d->sig[i] * d->sigScale, y = x[2 * i + 1];
            if ((y + dl) - yw > 0) { gx[2 * i + 1] += a; *gs += a * dl; }
            if (dl - y > 0) { gx[2 * i + 1] -= a; *gs += a * dl; }
        }
    }
    if (s->feaForces && cFea != 0) {
        for (int t = 0; t < d->ntri; t++) {
            int p[3] = {s->tri[3 * t], s->tri[3 * t + 1], s->tri[3 * t + 2]};
            double mu, la;
            d_lame(d->E[d->triCl[t]], d->nu[d->triCl[t]], &mu, &la);
            double Ds00 = d_img(x[2 * p[0]] - x[2 * p[2]], d->Lx, d->wx), Ds10 = d_img(x[2 * p[0] + 1] - x[2 * p[2] + 1], d->Ly, d->wy);
            double Ds01 = d_img(x[2 * p[1]] - x[2 * p[2]], d->Lx, d->wx), Ds11 = d_img(x[2 * p[1] + 1] - x[2 * p[2] + 1], d->Ly, d->wy);
            const double *B = d->B + 4 * t;
            double F00 = Ds00 * B[0] + Ds01 * B[1], F10 = Ds10 * B[0] + Ds11 * B[1];
            double F01 = Ds00 * B[2] + Ds01 * B[3], F11 = Ds10 * B[2] + Ds11 * B[3];
            double J = F00 * F11 - F01 * F10, lJ = log(J);
            double i00 = F11 / J, i10 = -F10 / J, i01 = -F01 / J, i11 = F00 / J;
            double P00 = mu * (F00 - i00) + la * lJ * i00, P10 = mu * (F10 - i01) + la * lJ * i01;
            double P01 = mu * (F01 - i10) + la * lJ * i10, P11 = mu * (F11 - i11) + la * lJ * i11;
            double v0 = d->vol0[t];
            /* dU/dx = -f = vol0 P Bm^T on vertices 0, 1; vertex 2 minus their sum */
            double H00 = v0 * (P00 * B[0] + P01 * B[2]), H10 = v0 * (P10 * B[0] + P11 * B[2]);
            double H01 = v0 * (P00 * B[1] + P01 * B[3]), H11 = v0 * (P10 * B[1] + P11 * B[3]);
            gx[2 * p[0]] += cFea * H00; gx[2 * p[0] + 1] += cFea * H10;
            gx[2 * p[1]] += cFea * H01; gx[2 * p[1] + 1] += cFea * H11;
            gx[2 * p[2]] -= cFea * (H00 + H01); gx[2 * p[2] + 1] -= cFea * (H10 + H11);
            double I1 = F00 * F00 + F10 * F10 + F01 * F01 + F11 * F11;
            int e = d->triCl[t];
            gMu[e] += cFea * v0 * (0.5 * (I1 - 2) - lJ);
            gLam[e] += cFea * v0 * 0.5 * lJ * lJ;
        }
    }
}

/* Adjoint of orc_d_forward: gradients of J (+ <xseed, x_N> + <vseed, v_N>
 * for non-null seeds) w.r.t. the initial positions and velocities (2N each),
 * per-elastomer E and nu, log eps_scale, log sig_scale. */
void orc_d_backward(const orc *s, int n0, double cWall, double cFea, const double *xseed, const double *vseed,
                    double *gx0, double *gv0, double *gE, double *gnu, double *glogeps, double *glogsig) {
    orc_d *d = &D_;
    int N = d->N, ne = d->ncl, steps = d->steps;
    double h = 0.5 * d->dt, dt = d->dt;
    double *xb = (double *)calloc(2 * (size_t)N + 2, sizeof(double));
    double *vb = (double *)calloc(2 * (size_t)N + 2, sizeof(double));
    double *gMu = (double *)calloc((size_t)ne + 1, sizeof(double));
    double *gLam = (double *)calloc((size_t)ne + 1, sizeof(double));
    double ge = 0, gs = 0;
    d_obs_grad(s, d->traj + 2 * (size_t)N * steps, n0 + steps, cWall, cFea, xb, gMu, gLam, &gs);
    if (xseed) for (int k = 0; k < 2 * N; k++) xb[k] += xseed[k];
    if (vseed) for (int k = 0; k < 2 * N; k++) vb[k] = vseed[k];
    double c = h;
    for (int n = steps; n >= 0; n--) {
        for (int i = 0; i < N; i++) { d->w[2 * i] = c * vb[2 * i] / d->m[i]; d->w[2 * i + 1] = c * vb[2 * i + 1] / d->m[i]; }
        d_forces(s, d->traj + 2 * (size_t)N * n, d->g, d->w, n0 + n, gMu, gLam, &ge, &gs);
        for (int k = 0; k < 2 * N; k++) xb[k] += d->g[k];
        if (n == 0) break;
        for (int k = 0; k < 2 * N; k++) vb[k] += dt * xb[k];
        c = (n - 1 == 0) ? h : dt;
    }
    memcpy(gx0, xb, sizeof(double) * 2 * (size_t)N);
    memcpy(gv0, vb, sizeof(double) * 2 * (size_t)N);
    for (int e = 0; e < ne; e++) {
        double E = d->E[e], nu = d->nu[e];
        double dmu_dE = 1.0 / (2 * (1 + nu)), dmu_dnu = -E / (2 * (1 + nu) * (1 + nu));
        double Dd = (1 + nu) * (1 - 2 * nu), dla_dE = nu / Dd, dla_dnu = E * (1 + 2 * nu * nu) / (Dd * Dd);
        gE[e] = gMu[e] * dmu_dE + gLam[e] * dla_dE;
        gnu[e] = gMu[e] * dmu_dnu + gLam[e] * dla_dnu;
    }
    *glogeps = ge;
    *glogsig = gs;
    free(xb); free(vb); free(gMu); free(gLam);
}

/* ------------------------------------------------------------ observables
 * Properties::evaluate (src/properties.cpp:15-36) in double on the current
 * float state: clusters unfolded as FeaElements::unfoldPos
 * (src/feaElements.cpp:86-150), feaVirial as src/interactions.cpp:681 with
 * FP64 nodal forces, cluster virial of calcPairForcesNN
 * (src/interactions.cpp:347-389) over pairs of two cluster particles, U and W
 * from orc_forces_f64.  out[0..9] = uKinetic, uPotential, uTotal,
 * temperature, virial, feaVirial, pressure, clusterUKinetic, clusterVirial,
 * molPressure; out[10..12] = condition scales (sums of term magnitudes) of
 * virial, feaVirial and clusterVirial. */
void orc_properties(const orc *s, double *out) {
    int N = s->N, ncl = s->ncl;
    int wx = (s->pbc == XYPBC || s->pbc == XPBC), wy = (s->pbc == XYPBC);
    double *fx = (double *)calloc((size_t)N + 1, sizeof(double)), *fy = (double *)calloc((size_t)N + 1, sizeof(double));
    double *cond = (double *)calloc((size_t)N + 1, sizeof(double)), *ui = (double *)calloc((size_t)N + 1, sizeof(double));
    double tot[4];
    orc_forces_f64(s, fx, fy, cond, ui, tot);
    double *ux = (double *)calloc((size_t)N + 1, sizeof(double)), *uy = (double *)calloc((size_t)N + 1, sizeof(double));
    double *cmx = (double *)calloc((size_t)ncl + 1, sizeof(double)), *cmy = (double *)calloc((size_t)ncl + 1, sizeof(double));
    double clusterKin = 0;
    for (int c = 0; c < ncl; c++) {
        int off = s->cl[c].offset, n = s->cl[c].nv;
        float xmin = 3e38f, xmax = -3e38f, ymin = 3e38f, ymax = -3e38f;
        for (int k = 0; k < n; k++) {
            float x = s->px[off + k], y = s->py[off + k];
            if (x < xmin) xmin = x; if (x > xmax) xmax = x;
            if (y < ymin) ymin = y; if (y > ymax) ymax = y;
        }
        int fxu = xmax - xmin > s->Lx / 2.0f, fyu = ymax - ymin > s->Ly / 2.0f;
        double sx = 0, sy = 0;
        for (int k = 0; k < n; k++) {
            int i = off + k;
            ux[i] = s->px[i]; uy[i] = s->py[i];
            if (fxu && s->px[i] > s->Lx / 2.0f) ux[i] -= s->Lx;
            if (fyu && s->py[i] > s->Ly / 2.0f) uy[i] -= s->Ly;
            sx += ux[i]; sy += uy[i];
        }
        int upx = fxu && sx / n < 0, upy = fyu && sy / n < 0;
        double mx = 0, my = 0, mvx = 0, mvy = 0, M = s->cl[c].mass;
        for (int k = 0; k < n; k++) {
            int i = off + k;
            if (upx) ux[i] += s->Lx;
            if (upy) uy[i] += s->Ly;
            mx += s->mass[i] * ux[i]; my += s->mass[i] * uy[i];
            mvx += (double)s->mass[i] * s->vx[i]; mvy += (double)s->mass[i] * s->vy[i];
        }
        cmx[c] = mx / M; cmy[c] = my / M;
        double vx = mvx / M, vy = mvy / M;
        clusterKin += M * (vx * vx + vy * vy);
    }
    double feaVir = 0, feaScale = 0, clScale = 0;
    if (s->feaForces && ncl > 0) {
        for (int t = 0; t < s->ntri; t++) {
            double f[6], cf[3], cu;
            if (s->fea_law) tri_green_d(s, t, f, cf, &cu); else tri_neo_hookean_d(s, t, f, cf, &cu);
            for (int k = 0; k < 3; k++) {
                int j = s->tri[3 * t + k];
                feaVir += f[2 * k] * ux[j] + f[2 * k + 1] * uy[j];
                feaScale += (cf[k] + fabs(f[2 * k]) + fabs(f[2 * k + 1])) * (fabs(ux[j]) + fabs(uy[j]));
            }
        }
    }
    double clVir = 0, kin = 0;
    for (int i = 0; i < N; i++) kin += (double)s->mass[i] * ((double)s->vx[i] * s->vx[i] + (double)s->vy[i] * s->vy[i]);
    if (ncl > 0 && s->nn_ready) {
        for (int pi = 0; pi < N; pi++) {
            int ci = s->cluster[pi];
            if (ci < 0) continue;
            for (int q = s->nbrStart[pi]; q < s->nbrStart[pi + 1]; q++) {
                int pj = s->nbrList[q], cj = s->cluster[pj];
                if (cj < 0) continue;
                int ti = s->type[pi], tj = s->type[pj], nt = s->numTypes;
                float sijf = (s->sigma[pi] + s->sigma[pj]) / 2.0f, rcij = s->rc[ti * nt + tj];
                float dxr, dyr, dxo, dyo;
                image_axis(s->px[pi], s->px[pj], s->Lx, wx, 0, &dxr, &dxo);
                image_axis(s->py[pi], s->py[pj], s->Ly, wy, 0, &dyr, &dyo);
                if (!(dxr * dxr + dyr * dyr < rcij * rcij * sijf * sijf)) continue;
                double dx, dy;
                image_axis_d(s->px[pi], s->px[pj], s->Lx, wx, &dx);
                image_axis_d(s->py[pi], s->py[pj], s->Ly, wy, &dy);
                double eij = s->eps[ti * nt + tj], sij = 0.5 * ((double)s->sigma[pi] + (double)s->sigma[pj]);
                double dr2 = dx * dx + dy * dy, c48 = 48.0 * eij / (sij * sij), d2i = sij * sij / dr2;
                double d6i = d2i * d2i * d2i, fc = c48 * d6i * (d6i - 0.5) * d2i;
                double rx = cmx[ci] - cmx[cj], ry = cmy[ci] - cmy[cj];
                if (wx) { if (rx >= 0.5 * s->Lx) rx -= s->Lx; else if (rx < -0.5 * s->Lx) rx += s->Lx; }
                if (wy) { if (ry >= 0.5 * s->Ly) ry -= s->Ly; else if (ry < -0.5 * s->Ly) ry += s->Ly; }
                clVir += 0.5 * (fc * dx * rx + fc * dy * ry);
                clScale += 0.5 * fabs(c48) * d6i * (d6i + 0.5) * d2i * (fabs(dx) + fabs(dy)) * (fabs(rx) + fabs(ry));
            }
        }
    }
    double V = (double)s->Lx * (double)s->Ly;
    out[0] = 0.5 * kin / N; out[1] = tot[0] / N; out[2] = out[0] + out[1]; out[3] = out[0];
    out[4] = tot[1]; out[5] = feaVir; out[6] = 0.5 * kin / V + 0.5 * (tot[1] + feaVir) / V;
    out[7] = ncl > 0 ? 0.5 * clusterKin / ncl : 0; out[8] = clVir; out[9] = 0.5 * clusterKin / V - 0.5 * clVir / V;
    out[10] = tot[3]; out[11] = feaScale; out[12] = clScale;
    free(fx); free(fy); free(cond); free(ui); free(ux); free(uy); free(cmx); free(cmy);
}
