/*
 * femmd.h -- C ABI of the GB300-native femmd2D timestep (libfemmd.so).
 *
 * One opaque context per simulated system (the reference keeps one global
 * MDSystem, femmd2D/src/interface.cpp:19).  Setup calls copy their inputs into
 * the context's host arrays, exactly as the reference's System.* / c_* calls
 * copy into its thrust host vectors; femmd_allocate_cuda / femmd_run upload
 * them and all compute runs on the context's own CUDA stream with
 * hand-written sm_103a kernels.  There is no CPU compute path: every force,
 * list and integration call needs a GPU and reports FEMMD_CUDA_ERROR without
 * one.
 *
 * Every call returns a femmd_status (0 = OK).  femmd_last_error() gives the
 * message of the last failure; nothing calls exit() or traps.
 *
 * Index conventions follow the reference: particles are numbered in
 * insertion order, elastomer triangle files are 1-based (add_elastomer),
 * create_bond takes 0-based particle ids.  Arrays of 2-vectors are
 * interleaved x,y float32.
 */
#ifndef FEMMD_H
#define FEMMD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct femmd_ctx femmd_ctx;

typedef enum {
    FEMMD_OK = 0,
    FEMMD_INVALID_ARG = 1,        /* bad index, size, order or value */
    FEMMD_CAPACITY_OVERFLOW = 2,  /* a capacity could not be grown */
    FEMMD_NONFINITE = 3,          /* a force or energy became NaN/inf */
    FEMMD_CUDA_ERROR = 4,         /* a CUDA call failed (no GPU, OOM, ...) */
    FEMMD_TIMEOUT = 5,            /* a bounded device wait expired (the fast step's copies, the small-system
                                     run's grid-wide exchanges) */
    FEMMD_NOT_READY = 6,          /* call order: e.g. run before init_neighbor_list */
    FEMMD_UNSUPPORTED = 7         /* feature of the reference outside this path */
} femmd_status;

enum { FEMMD_NOPBC = 0, FEMMD_XPBC = 1, FEMMD_XYPBC = 2 };      /* PBCTYPE, femmd2D/src/def.h:41 */
enum { FEMMD_FEA_NEO_HOOKEAN = 0, FEMMD_FEA_GREEN_LINEAR = 1 }; /* interactions.cpp:532 / interactionsCuda.cu:312 */
enum { FEMMD_BONDK_KBOND = 0, FEMMD_BONDK_E_OVER_R0 = 1 };      /* interactions.cpp:161 / interactionsCuda.cu:238 */
enum { FEMMD_IMAGE_REFERENCE = 0, FEMMD_IMAGE_EXACT = 1 };
enum { FEMMD_ELASTOMER_BONDS_ALL = 0, FEMMD_ELASTOMER_BONDS_BOUNDARY = 1, FEMMD_ELASTOMER_BONDS_NONE = 2 };
enum { FEMMD_FORCE_REFERENCE = 0, FEMMD_FORCE_FAST = 1 };

/* ----------------------------------------------------------- lifecycle */
/* MDSystem(0) + setDevice(GPU): femmd2D/src/md3dsystem.h:58-84.  device is the CUDA ordinal. */
femmd_status femmd_create(int device, femmd_ctx **out);
void femmd_destroy(femmd_ctx *ctx);
const char *femmd_last_error(const femmd_ctx *ctx);
/* Library version string. */
const char *femmd_version(void);

/* --------------------------------------------------- setup (System.*) */
/* System.init(Lx, Ly): interface.cpp:229 -> MDSystem::init md3dsystem.cpp:49-80 */
femmd_status femmd_init(femmd_ctx *ctx, double Lx, double Ly);
/* System.reset(): interface.cpp:237 -> MDSystem::reset md3dsystem.cpp:82-89 */
femmd_status femmd_reset(femmd_ctx *ctx);
/* System.set_box / get_box: interface.cpp:411-427 */
femmd_status femmd_set_box(femmd_ctx *ctx, double Lx, double Ly);
femmd_status femmd_get_box(const femmd_ctx *ctx, double *Lx, double *Ly);
/* System.PBC(0|1|2): interface.cpp:353-363 */
femmd_status femmd_set_pbc(femmd_ctx *ctx, int pbc);
/* System.DEV(0|1): interface.cpp:344-351.  Recorded; compute always runs on the GPU. */
femmd_status femmd_set_dev(femmd_ctx *ctx, int dev);
/* System.set_dt / get_dt: interface.cpp:400-409 */
femmd_status femmd_set_dt(femmd_ctx *ctx, double dt);
femmd_status femmd_get_dt(const femmd_ctx *ctx, double *dt);
/* System.set_numTypes(n): interface.cpp:436-441 */
femmd_status femmd_set_num_types(femmd_ctx *ctx, int n);
/* System.set_pair_potential(eps, rc, ushift), n*n row-major each: interface.cpp:493-531 ->
 * Interactions::setPairForce interactions.cpp:65-79 (rc in units of sigma_ij). */
femmd_status femmd_set_pair_potential(femmd_ctx *ctx, const double *eps, const double *rc, const double *ushift,
                                      int n2);
/* System.set_kBond(k): interface.cpp:455-465 (k <= 0 disables bonds) */
femmd_status femmd_set_kbond(femmd_ctx *ctx, double k);
/* System.set_youngs_modulus(E): interface.cpp:479-490 (E <= 0 disables FEA) */
femmd_status femmd_set_youngs_modulus(femmd_ctx *ctx, double E);
/* Interactions::nu (C++ only in the reference, interactions.h:22; default 0.3) */
femmd_status femmd_set_poisson_ratio(femmd_ctx *ctx, double nu);
/* System.set_gravity(g): interface.cpp:443-453 (g > 0 enables f_y -= m g,
 * calcGravityForces, interactions.cpp:111-126).  System.set_kArea(k):
 * interface.cpp:466-476 (k > 0 enables the area springs of calcAreaForcesCPU,
 * interactions.cpp:696-750: after the triangle forces, each triangle in turn
 * displaces its vertices towards its reference area, and the pair forces see
 * the displaced positions; not available in the batched kernel or the
 * adjoint, which return FEMMD_UNSUPPORTED).  Boxes that are not periodic in y get the
 * reference's fixed walls (NOPBC: LJ walls on every side; XPBC: harmonic top
 * and bottom with kWall = 10), unless femmd_set_moving_wall is set. */
femmd_status femmd_set_gravity(femmd_ctx *ctx, double g);
femmd_status femmd_set_karea(femmd_ctx *ctx, double k);
/* Per-elastomer material: elastomer e (in add order) gets its own Young's
 * modulus and Poisson ratio instead of the global ones (neo-Hookean law only).
 * The reference has one global E (Interactions::E, interactions.h:20). */
femmd_status femmd_set_elastomer_material(femmd_ctx *ctx, int elastomer, double E, double nu);
/* Moving harmonic walls for boxes not periodic in y: a bottom wall at y = 0
 * and a top wall at y_w(n) = y0 - v * n * dt, n the step index of the
 * positions.  A particle closer than 2^(1/6) sigma_i to a wall (the contact
 * range of calcTopBottomWallForces, interactions.cpp:242-270) gets the force
 * k * overlap away from it and the energy k/2 overlap^2.  k <= 0 removes them. */
femmd_status femmd_set_moving_wall(femmd_ctx *ctx, double k, double y0, double v);
/* Forces the particles exert on the top and bottom walls at the current
 * positions (sum of k * overlap). */
femmd_status femmd_get_wall_forces(femmd_ctx *ctx, double *top, double *bottom);
/* List cells of factor * (rc + skin), factor in [1, 8] (1: the reference's
 * cell size); applied by the next femmd_init_neighbor_list.  A factor other
 * than 1 changes the list order and therefore the rounding of the sums. */
femmd_status femmd_set_cell_factor(femmd_ctx *ctx, double factor);
/* NeighborList::setSkin (C++ only, nn.h:64; default 0.4) */
femmd_status femmd_set_skin(femmd_ctx *ctx, double skin);
/* Neighbour-list capacity per particle (0 = size from the first build).  A
 * build that exceeds it makes femmd_run roll back to the run's start, grow the
 * list and repeat; the reference's fixed maxNeighborsPerParticle
 * (nn.cpp:223-224) is never checked. */
femmd_status femmd_set_neighbor_capacity(femmd_ctx *ctx, int cap);
femmd_status femmd_get_neighbor_capacity(const femmd_ctx *ctx, int *cap);
/* Law and convention selectors (defaults: neo-Hookean, kBond, exact image).
 * FEMMD_IMAGE_REFERENCE reproduces the reference's float minimum image
 * bit for bit; FEMMD_IMAGE_EXACT rounds a cross-boundary difference once. */
femmd_status femmd_set_fea_law(femmd_ctx *ctx, int law);
femmd_status femmd_set_bond_k_mode(femmd_ctx *ctx, int mode);
femmd_status femmd_set_image_mode(femmd_ctx *ctx, int mode);
/* Force mode (default FEMMD_FORCE_REFERENCE).  The reference mode reproduces
 * the reference's float operations and list order, so trajectories follow
 * the reference's bit for bit (in FEMMD_IMAGE_REFERENCE) or the oracle's.
 * FEMMD_FORCE_FAST keeps the same cell and neighbour sets and forces,
 * energies and virial within 1e-5 of an FP64 evaluation, but sums with fused
 * multiply-adds and the hardware reciprocal and stores the free particles in
 * cell order on the device (renewed with every neighbour list); trajectories
 * then agree with the reference-exact ones to rounding, not bit for bit.
 * Getters and setters keep the particle ids either way.  The batched kernel
 * and the adjoint run the reference mode only (FEMMD_UNSUPPORTED in fast
 * mode).  Changing the mode re-uploads the system at the next run.  No
 * counterpart in the reference, whose CPU and GPU paths each fix one
 * arithmetic. */
femmd_status femmd_set_force_mode(femmd_ctx *ctx, int mode);
femmd_status femmd_get_force_mode(const femmd_ctx *ctx, int *mode);
/* Which edges of each later add_elastomer become bonds (default: every
 * triangle edge, interior edges twice, as particles.cpp:335-337). */
femmd_status femmd_set_elastomer_bonds(femmd_ctx *ctx, int mode);

/* System.add_particle(x, y, vx, vy, m, sig, typ): interface.cpp:243-254 -> particles.cpp:226 */
femmd_status femmd_add_particle(femmd_ctx *ctx, double x, double y, double vx, double vy, double m, double sig,
                                int typ);
/* n calls of femmd_add_particle, one per array element */
femmd_status femmd_add_particles(femmd_ctx *ctx, int n, const double *x, const double *y, const double *vx,
                                 const double *vy, const double *m, const double *sig, const int *typ);
/* System.add_elastomer(verts, tris, x, y, typ, g, sig, mass, exclude): interface.cpp:533-563 ->
 * Particles::addElastomer particles.cpp:295-385.  verts: nv (x,y) float32; tris: nt 1-based int32 triples.
 * All elastomers must share one mesh and precede free particles (reference constraint). */
femmd_status femmd_add_elastomer(femmd_ctx *ctx, const float *verts, int nv, const int *tris, int nt, double x,
                                 double y, int typ, int g, double sig, double mass, int exclude);
/* c_createBond(i, j): interface.cpp:67 -> Bonds::createBond bonds.cpp:14-29 */
femmd_status femmd_create_bond(femmd_ctx *ctx, int i, int j);
/* System.set_velocities(v0): interface.cpp:337-342 -> particles.cpp:233-261, with a caller seed
 * instead of rand(): random directions, speed v0, zero net momentum. */
femmd_status femmd_set_velocities(femmd_ctx *ctx, double v0, uint64_t seed);

/* System.allocate_cuda(): interface.cpp:256 -> MDSystem::allocateCuda md3dsystem.h:86-94 */
femmd_status femmd_allocate_cuda(femmd_ctx *ctx);
/* System.init_neighbor_list(): interface.cpp:261 -> NeighborList::init nn.cpp:192-227 */
femmd_status femmd_init_neighbor_list(femmd_ctx *ctx);

/* --------------------------------------------------------- stepping */
/* System.run(n): interface.cpp:267 -> Integrator::run integrator.cpp:31-57.  Returns when done. */
femmd_status femmd_run(femmd_ctx *ctx, int steps);
/* c_doStep(): interface.cpp:73 -> Integrator::doStep integrator.cpp:8-29 (one step, no
 * forced rebuild, no initial force pass; needs a prior run or calc_forces). */
femmd_status femmd_do_step(femmd_ctx *ctx);
/* c_calcForces() after c_zeroStuff(): interface.cpp:69-71 -> Interactions::calcForces
 * interactions.cpp:83-109 on the current positions and neighbour list. */
femmd_status femmd_calc_forces(femmd_ctx *ctx);
/* c_zeroStuff(): interface.cpp:69 -> Integrator::zeroStuff integrator.cpp:146-162 */
femmd_status femmd_zero_stuff(femmd_ctx *ctx);
/* NeighborList::buildNN nn.cpp:137-143 on the current positions (no dispHi change) */
femmd_status femmd_build_neighbor_list(femmd_ctx *ctx);
/* Wait for all queued work of the context. */
femmd_status femmd_sync(femmd_ctx *ctx);

/* ---------------------------------------------------------- getters */
/* c_getNumberOfParticles / c_getNumberOfBonds: interface.cpp:41-42 */
int femmd_get_num_particles(const femmd_ctx *ctx);
int femmd_get_num_bonds(const femmd_ctx *ctx);
int femmd_get_num_triangles(const femmd_ctx *ctx);
int femmd_get_num_elastomers(const femmd_ctx *ctx);
int femmd_get_steps(const femmd_ctx *ctx);
/* c_getPosPtr / c_getVelPtr (interface.cpp:43-44) as copies: out holds 2N floats */
femmd_status femmd_get_positions(femmd_ctx *ctx, float *out);
femmd_status femmd_get_velocities(femmd_ctx *ctx, float *out);
femmd_status femmd_get_accelerations(femmd_ctx *ctx, float *out);
/* Forces of the last calc_forces (2N floats). */
femmd_status femmd_get_forces(femmd_ctx *ctx, float *out);
/* Per-particle potential energy of the last calc_forces (N floats): bond energy on the
 * bond's first particle, triangle energy split in thirds, LJ u/2 per ordered pair. */
femmd_status femmd_get_particle_energies(femmd_ctx *ctx, float *out);
femmd_status femmd_get_masses(const femmd_ctx *ctx, float *out);
/* c_getBondsPtr (interface.cpp:45) as a copy: 2*nbonds ints, and nbonds rest lengths */
femmd_status femmd_get_bonds(const femmd_ctx *ctx, int *pairs, float *rest_lengths);
/* triangles (3*nt 0-based global ids), their [1 X Y] inverses (9*nt) and signed areas (nt) */
femmd_status femmd_get_triangles(const femmd_ctx *ctx, int *tris, float *xm, float *ref_area);
femmd_status femmd_get_exclusion_groups(const femmd_ctx *ctx, int *out);
femmd_status femmd_get_reference_positions(const femmd_ctx *ctx, float *out);
/* Scalars of the last force evaluation in FP64: out[0]=U (potEnergy), out[1]=W (pair
 * virial), out[2]=sum m v^2 (kinEneSum), out[3]=max v^2, out[4]=dispHi, out[5]=totalUpdates. */
femmd_status femmd_get_energies(femmd_ctx *ctx, double *out);
/* Per-step observables of the last run: rows of (U, W, sum m v^2, max v^2, dispHi, rebuilt). */
femmd_status femmd_get_step_observables(femmd_ctx *ctx, double *out, int max_rows, int *rows);
/* Cell grid and cell lists of the last neighbour build: grid (ncx, ncy); cell_start has
 * ncx*ncy+1 entries, cell_ids N entries (ascending particle id inside a cell). */
femmd_status femmd_get_grid(const femmd_ctx *ctx, int *ncx, int *ncy);
femmd_status femmd_get_cells(femmd_ctx *ctx, int *cell_start, int *cell_ids);
/* Neighbour lists of the last build in CSR: nbr_start N+1, nbr_list total entries in the
 * reference's order.  femmd_get_neighbor_total gives the total. */
femmd_status femmd_get_neighbor_total(femmd_ctx *ctx, long long *total);
femmd_status femmd_get_neighbors(femmd_ctx *ctx, int *nbr_start, int *nbr_list);
/* Build statistics: mean neighbours per particle at the last build and builds since init. */
femmd_status femmd_get_nn_stats(femmd_ctx *ctx, double *mean_neighbors, int *max_neighbors, long long *builds);
/* System.info(): interface.cpp:565-600 -> N, nelastomers, nbonds, ntrigs, dt, kBond, kArea, E, box */
femmd_status femmd_info(const femmd_ctx *ctx, double *out9);

/* ------------------------------------------------------- state I/O */
/* Positions/velocities in (2N floats each, NULL = keep).  Marks the device copy stale. */
femmd_status femmd_set_state(femmd_ctx *ctx, const float *pos, const float *vel);
/* Copy positions/velocities/accelerations out (NULL = skip). */
femmd_status femmd_get_state(femmd_ctx *ctx, float *pos, float *vel, float *acc);

/* ------------------------------------------------- device-side access */
/* The context's CUDA stream (cudaStream_t) for event timing by the caller. */
void *femmd_get_stream(femmd_ctx *ctx);
/* Device-side trace of the next runs (on != 0): per step, %globaltimer
 * nanoseconds at the start and end of the triangle pass, the step kernel and
 * the neighbour rebuild (0 where a phase did not run), rows as the
 * observables of femmd_get_step_observables. */
femmd_status femmd_set_trace(femmd_ctx *ctx, int on);
femmd_status femmd_get_trace(femmd_ctx *ctx, unsigned long long *out, int max_rows, int *rows);
/* CUDA events on the context stream (slots 0..63) for device-side timing. */
femmd_status femmd_event_record(femmd_ctx *ctx, int slot);
femmd_status femmd_event_elapsed(femmd_ctx *ctx, int slot_a, int slot_b, float *ms);
/* Launch each kernel directly (no CUDA graph) with CUDA events around the
 * force kernel and return its summed time and launch count over the next
 * femmd_run calls (profile != 0 starts a new tally). */
femmd_status femmd_set_profiling(femmd_ctx *ctx, int profile);
femmd_status femmd_get_profile(femmd_ctx *ctx, double *force_kernel_ms, long long *force_kernel_launches,
                               double *rebuild_ms, long long *rebuilds, long long *kernel_launches);
/* For tests of the failure path: in the next run that takes the small-system
 * run (the fast mode's cooperative launch), block 0 withholds its record of
 * the first grid-wide exchange, so every block's bounded wait gives up
 * (about a second) and femmd_run returns FEMMD_TIMEOUT with the context
 * still usable.  No GPU fault, trap or endless wait is involved. */
femmd_status femmd_test_expire_next_exchange(femmd_ctx *ctx);

/* ------------------------------------------------------- batched replicas */
/* Many independent systems advanced in one persistent launch: each replica
 * is a context set up as usual (through init_neighbor_list); femmd_batch_run(n)
 * performs femmd_run(n) on every replica -- same results, bit for bit, as
 * running them one by one -- with one CTA per group of replicas
 * (longest-processing-time assignment) and no per-step launches.  Replicas
 * must share the number of types, the sigma mode, the periodicity and the
 * image mode; a replica with area springs, trajectory frames or property
 * averaging on makes femmd_batch_run return FEMMD_UNSUPPORTED (the batched
 * kernel does none of them).  A replica's results are read with the usual
 * getters on its context.  The batch does not own the contexts. */
typedef struct femmd_batch femmd_batch;
femmd_status femmd_batch_create(int device, femmd_batch **out);
void femmd_batch_destroy(femmd_batch *b);
const char *femmd_batch_last_error(const femmd_batch *b);
femmd_status femmd_batch_add(femmd_batch *b, femmd_ctx *ctx, int *index);
int femmd_batch_size(const femmd_batch *b);
femmd_status femmd_batch_run(femmd_batch *b, int steps);
/* Launch shape: threads per CTA (multiple of 32, <= 1024) and CTAs per SM. */
femmd_status femmd_batch_set_launch(femmd_batch *b, int threads, int ctas_per_sm);
/* Replicas heavier than a CTA's average share of the batch (atoms +
 * triangles) run on a pair of CTAs (a thread-block cluster of two) before
 * the rest run one per CTA, so that the largest replica no longer sets the
 * length of the launch alone; needs an even number of CTAs.  On by default;
 * results are bit-identical either way. */
femmd_status femmd_batch_set_split(femmd_batch *b, int on);
femmd_status femmd_batch_get_launch(const femmd_batch *b, int *threads, int *ctas_per_sm, int *ctas);
/* Times trial_steps on each candidate launch shape (states restored after each
 * trial) and keeps the fastest. */
femmd_status femmd_batch_autotune(femmd_batch *b, int trial_steps, int *threads, int *ctas_per_sm, double *best_ms);
/* Opt-in tuning of the rebuild cadence and cell size: every (skin, cell
 * factor) pair is timed on run(trial_steps) of the whole batch from the
 * current states (restored after each trial) and the fastest pair is applied
 * to every replica (femmd_set_skin, femmd_set_cell_factor,
 * femmd_init_neighbor_list).  Trajectories then no longer round as the
 * reference's do; the physics is unchanged. */
femmd_status femmd_batch_autotune_lists(femmd_batch *b, int trial_steps, const double *skins, int nskins,
                                        const double *factors, int nfactors, double *best_skin,
                                        double *best_factor, double *best_ms);
femmd_status femmd_batch_event_record(femmd_batch *b, int slot);
femmd_status femmd_batch_event_elapsed(femmd_batch *b, int slot_a, int slot_b, float *ms);

/* --------------------------------------------------------- trajectory */
/* System.save_trajectory / set_trajectory_steps (interface.cpp:289-299):
 * during femmd_run, every 'every' steps (at step counts that are multiples of
 * it, as Integrator::doStep, integrator.cpp:20-26) the positions and
 * velocities are copied to pinned host memory and written by a host thread
 * while the run goes on.  Layouts of the reference's writers
 * (md3dsystem.cpp), the first four appended to 'path', the others one file
 * '<path><step, 9 digits>.<ext>' per frame, elastomers unfolded:
 *   0  saveClusterXYZ (:248-273; that routine lists only the first NC
 *      particles, every particle is listed here)
 *   1  saveXYZ (:232-246)
 *   2  saveVtk (:275-328), legacy VTK '.vtk' (nothing without elastomers)
 *   3  saveVTF (:330-353), the structure block (atoms, bonds, pbc) before the first frame
 *   4  saveClusterVTF (:355-378), one atom per elastomer at its centre of mass
 *   5  saveVtkXML (:381-443), VTK XML '.vtu', ascii
 *   6  saveVtkXMLBin (:451-522), VTK XML '.vtu', raw appended arrays
 * The run's results are bit for bit those without frames.  path NULL or
 * every <= 0 stops writing. */
femmd_status femmd_set_trajectory(femmd_ctx *ctx, const char *path, int every, int format);
/* Wait until every captured frame is on disk; the count written so far. */
femmd_status femmd_flush_trajectory(femmd_ctx *ctx, long long *frames_written);
/* save_vtk / save_vtf / save_cluster_vtf / save_cluster_xyz
 * (interface.cpp:301-330, and the reference's saveXYZ, saveVtkXML and
 * saveVtkXMLBin): the current state written now in layout 'format' above,
 * named by the current step count where the layout makes one file per frame.
 * append = 0 starts the file anew (and writes the VTF structure block), as
 * the reference's s = 0; otherwise the frame is added to it. */
femmd_status femmd_save_frame(femmd_ctx *ctx, const char *path, int format, int append);
/* set_scale (interface.cpp:365-369): the cluster VTF atoms' radius is
 * 0.5 scale + 0.5.  1 until set (the reference leaves it unset). */
femmd_status femmd_set_scale(femmd_ctx *ctx, double scale);

/* -------------------------------------------------------- observables */
/* Properties::evaluate (properties.cpp:15-36) at the current state, FP64
 * sums on the device: out[0..9] = uKinetic, uPotential, uTotal, temperature,
 * virial, feaVirial, pressure, clusterUKinetic, clusterVirial, molPressure.
 * Clusters are unfolded across the periodic boundary as
 * FeaElements::unfoldPos (feaElements.cpp:86-150) does; the cluster virial
 * sums pairs of two cluster particles (the reference indexes clusters[-1] for
 * free particles). */
femmd_status femmd_get_properties(femmd_ctx *ctx, double *out);
/* Properties::compute (properties.cpp:85-95), run after every doStep
 * (integrator.cpp:18): with on != 0 the ten values of femmd_get_properties
 * are evaluated at the end of every step of run() and do_step() and summed;
 * at steps past step_equi that are multiples of step_avg the window's
 * average and standard deviation (Prop::avg, properties.h:11) are kept and a
 * new window starts (accumulate(2), accumulate(0)).  The reference's
 * defaults are step_avg 1000, step_equi 10000.  Switching on starts from
 * empty sums.  Each averaged step costs the observables kernels on top of the
 * step.  System.print_props (interface.cpp:270-286) prints the averages. */
femmd_status femmd_set_property_averaging(femmd_ctx *ctx, int on, int step_avg, int step_equi);
/* FeaElements::calcClusterProps (feaElements.cpp:199-204) at the current
 * state: per cluster (elastomer, in add order) the centre of mass of the
 * unfolded vertices and its velocity (unfoldPos, :86-150) and the periodic
 * centroid from the mean angle per axis (updateClustersCentroid, :162-197;
 * the reference's y uses the x sums, here y uses its own).  2 doubles per
 * cluster in each array; a NULL array is skipped. */
femmd_status femmd_get_clusters(femmd_ctx *ctx, double *cm, double *cm_vel, double *centroid);
/* The last completed window's averages and standard deviations, the last
 * step's values, the steps summed in the open window, the windows closed so
 * far and the step that closed the last one (any pointer may be NULL; arrays
 * of 10 in femmd_get_properties' order). */
femmd_status femmd_get_average_properties(femmd_ctx *ctx, double *avg, double *stdv, double *val, int *count,
                                          int *windows, int *last_step);

/* ------------------------------------------------------------ adjoint */
/* Gradients of an observable of the final state through the whole run, by the
 * discrete adjoint of the leapfrog step (no counterpart in the reference).
 *
 * femmd_adjoint_forward runs 'steps' steps as run(every) segments (the same
 * kernels as femmd_run) and keeps positions and velocities at the start of
 * every segment.  femmd_adjoint_backward then sweeps the segments backwards:
 * each segment is recomputed from its checkpoint, its positions recorded, and
 * the reverse steps applied with the forward's own neighbour lists.  The
 * observable is
 *   J = c_wall * (F_top + F_bottom) / (2 Lx) + c_fea * U_fea
 *       + <xbar_final, x_N> + <vbar_final, v_N>
 * (wall stress and FEA energy at the final positions; the two seed arrays,
 * 2N floats each, may be null).  Outputs (host arrays, each may be null):
 * dJ/dx_0 and dJ/dv_0 (2N floats), dJ/dE and dJ/dnu per elastomer (neo-Hookean
 * law; the elastomer's own values or the global ones), and dJ/d(log eps),
 * dJ/d(log sigma) for one common scale on every pair epsilon and every
 * particle sigma (the wall contact ranges scale with sigma).  The context's
 * final state is restored afterwards.  Bond stiffness is taken as the
 * constant kBond. */
femmd_status femmd_adjoint_forward(femmd_ctx *ctx, int steps, int every);
femmd_status femmd_adjoint_backward(femmd_ctx *ctx, double c_wall, double c_fea, const float *xbar_final,
                                    const float *vbar_final, float *xbar_init, float *vbar_init, double *dJ_dE,
                                    double *dJ_dnu, double *dJ_dlog_eps, double *dJ_dlog_sigma);
/* Wall stress (F_top + F_bottom) / (2 Lx) and FEA energy at the current positions. */
femmd_status femmd_adjoint_observable(femmd_ctx *ctx, double *wall_stress, double *fea_energy);

/* ------------------------------------------ cell binning without allocation */
/* Limits of femmd_bin_cells_noalloc.  Its working memory is one fixed array of
 * about 9 MB inside the library, which every GPU that loads the library holds
 * until the process exits. */
#define FEMMD_NOALLOC_MAX_PARTICLES (1 << 20)
#define FEMMD_NOALLOC_MAX_CELLS (1 << 18)
/* Bins n particles into the ncx x ncy cell grid of a (Lx, Ly) box exactly as
 * the context's neighbour-list build does (the reference's cell ids, ascending
 * particle id inside a cell), without allocating anything.  It has no
 * counterpart in the reference.  It is meant for callers that cannot call
 * cudaMalloc where they need the binning: code being captured into a CUDA
 * graph (allocation is not permitted during capture) or running under a host
 * framework that owns all device memory through its own pool (cudaMalloc and
 * cudaFree would synchronise the device and bypass that pool).
 * All pointers are device memory owned by the caller: d_pos holds 2n floats,
 * d_cell_start receives ncx*ncy+1 ints, d_cell_ids receives n ints.  The work
 * is enqueued on 'stream' (a cudaStream_t; NULL = the default stream) and the
 * call returns without waiting.  n above FEMMD_NOALLOC_MAX_PARTICLES or
 * ncx*ncy above FEMMD_NOALLOC_MAX_CELLS returns FEMMD_CAPACITY_OVERFLOW and
 * does nothing.  The kernels name the working array in device code, so each
 * call uses the array of the context it runs in; nothing is cached on the
 * host, and after cudaDeviceReset the next call simply runs in the new
 * context.  Make the first call on a device outside stream capture (it may
 * load the library's kernels).  Every call uses the same working array and
 * leaves its contents behind, so calls that can overlap on the GPU (different
 * streams without ordering between them) race.  A CUDA error that an earlier,
 * unrelated call left pending is left in place; FEMMD_CUDA_ERROR means one of
 * this call's launches failed. */
femmd_status femmd_bin_cells_noalloc(const float *d_pos, int n, double Lx, double Ly, int ncx, int ncy,
                                     int *d_cell_start, int *d_cell_ids, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FEMMD_H */
