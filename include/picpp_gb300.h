/*
 * picpp_gb300.h -- C ABI of the GB300 (sm_103a) implementation of PIC++'s
 * per-timestep hot path.
 *
 * The reference has no plugin or FFI layer: the hot path sits behind the
 * member functions of class Simulation that the step loop of
 * Simulation::simulate calls (PIC++/simulation.cpp:164-259, 296-309, 360).
 * Each phase entry point below names the member function it replaces.  All
 * of them act on one context that owns every device buffer; host buffers
 * stay owned by the caller.  Every call is synchronous on the context's
 * CUDA stream (it returns after the GPU work finished) and returns a status
 * code; the reference instead prints, writes errorLog.dat and exits
 * (PIC++/util.cpp:119-129).
 *
 * Layout shared by every grid argument: a periodic box of nx*ny*nz cells,
 * component-major then k, j, i with i fastest (a[c][k][j][i]).  Explicit
 * (Yee) runs keep Ex at (i+1/2, j, k), Ey at (i, j+1/2, k), Ez at
 * (i, j, k+1/2), Bx at (i, j+1/2, k+1/2), By at (i+1/2, j, k+1/2),
 * Bz at (i+1/2, j+1/2, k), J like E (PIC++/correlation.cpp:585-591).  Implicit
 * runs keep E on nodes (i, j, k) and B on cell centres (i+1/2, j+1/2, k+1/2)
 * (PIC++/correlation.cpp:23-164).  The reference's ghosted index r maps to
 * our (r - 2) mod n.  Particles are given by a linear cell index (i fastest),
 * in-cell offsets in [0,1) and momentum p = m*gamma*v; units are the
 * reference's normalised units with c = 1.
 */
#ifndef PICPP_GB300_H
#define PICPP_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pic_ctx pic_ctx;

typedef enum {
    PIC_OK = 0,
    PIC_ERR_ARG = 1,        /* invalid argument or configuration            */
    PIC_ERR_CUDA = 2,       /* CUDA runtime error (message in pic_last_error) */
    PIC_ERR_STATE = 3,      /* call not valid for this solver / state        */
    PIC_ERR_NOMEM = 4,      /* device allocation failed or capacity exceeded */
    PIC_ERR_NUMERIC = 5,    /* NaN/Inf detected in an input or a solve       */
    PIC_ERR_NOT_CONVERGED = 6 /* field solve missed its tolerance            */
} pic_status;

typedef enum { PIC_SOLVER_BUNEMAN = 0, PIC_SOLVER_IMPLICIT = 1 } pic_solver_type;
typedef enum { PIC_REAL_F32 = 0, PIC_REAL_F64 = 1 } pic_real;

/* One run's configuration; replaces the input deck and the compile-time
 * constants of PIC++/constants.h that the hot path reads. */
typedef struct {
    int nx, ny, nz;          /* cells per axis (an axis of 1 is a reduced dimension) */
    double dx, dy, dz, dt;
    double theta;            /* implicit centring, initialTheta (constants.h:40)       */
    double eta;              /* mover centring, Simulation::eta (initialization.cpp:320) */
    double cfix;             /* speed_of_light_correction (constants.h:45), 1.025      */
    int solver;              /* pic_solver_type                                         */
    int particle_real;       /* pic_real of particle offsets/momenta and of the push    */
    int field_real;          /* pic_real of the Yee E and B grids (explicit runs)       */
    int pressure_compat;     /* 1: reproduce the reference's pressure-tensor indexing
                                (momentum_collecting.cpp:565,577) and fold
                                (momentum_exchange.cpp:1643-1741); 0: periodic          */
    int sort_every;          /* re-sort particles by cell every n steps (0: never)     */
    int tile[3];             /* tile extents of the sort key / deposit tiles (0: 8)     */
    int max_species;         /* species slots to reserve (0: 8)                         */
    int smoothing_count;     /* smoothingCount: passes of the 3x3x3 smoothing of the
                                current (explicit, simulation.cpp:186-188) or of
                                rho-hat, J-hat and mu (implicit, simulation.cpp:213-217;
                                needs pressure_compat = 0)                              */
    double smoothing_parameter; /* smoothingParameter s: weights s/2, 1-s, s/2 per axis
                                (createSmoothingMatrix, smoothing.cpp:105-137)          */
    int boundary_x;          /* pic_boundary_x                                          */
    double e_right[3], b_right[3]; /* PIC_BOUNDARY_WALL_OPEN: the open boundary's constant
                                fields (ConstantBoundaryFieldEvaluator, set up by
                                initializeFluxFromRight, initialization.cpp:5201-5207) */
} pic_config;

/* Boundary along x.  PIC_BOUNDARY_WALL_OPEN is boundaryConditionTypeX =
 * SUPER_CONDUCTOR_LEFT of one rank (3-D boxes, no smoothing): a conductor
 * wall at x = 0 and an open boundary at x = (nx - 2) dx.  The physical
 * domain is nodes 0 .. nx - 2 and cells 0 .. nx - 3 of the nx-cell storage;
 * storage column nx - 2 holds the ghost cell beyond the open boundary,
 * column nx - 1 the ghost cell left of the wall and the ghost node beyond
 * the open boundary.  Particles may not be placed in the two ghost columns.
 *   Implicit runs: the boundary field E_right, B_right in the ghost cells
 * and boundary rows (fields.cpp:690-781, 2738-2756); the mover reflects
 * particles at the wall x = 0 (mover.cpp:247-260, 312-330, 435-445).
 *   Explicit runs (nx >= 24): E_y = E_z = 0 on the wall node and E_right's
 * y, z components (Simulation::E0) on the open boundary node
 * (fields.cpp:116-121, 136-141), the ghost column left of the wall as the
 * reference's exchanges set it; the mover reflects particles at node 18
 * (xgrid[reflectingWallPoint], mover.cpp:744-772) and the zigzag current
 * mirrors the old position there (momentum_collecting.cpp:93-99).
 * Both erase the particles that cross the open boundary after they
 * deposited their current (mover.cpp:447-458, 760-770,
 * eraseEscapedPaticles mover.cpp:167-192); particles are fed in with
 * pic_append_particles (injectNewParticles, mover.cpp:910-1000, with the
 * caller's particles). */
typedef enum { PIC_BOUNDARY_PERIODIC = 0, PIC_BOUNDARY_WALL_OPEN = 1 } pic_boundary_x;

/* Field-solve options for the implicit Maxwell system. */
typedef enum {
    PIC_GMRES_REFERENCE = 0, /* generalizedMinimalResidualMethod semantics
                                (specialmath.cpp:367-671): unrestarted, MGS,
                                stop at |r|/|b| <= tol/(3N) or max_iter vectors */
    PIC_GMRES_RESTARTED = 1, /* GMRES(restart), classical Gram-Schmidt with
                                re-orthogonalisation, true FP64 residual checked
                                against tol at every restart                     */
    PIC_FGMRES_LEARNED = 2,  /* flexible GMRES(restart) with the learned right
                                preconditioner; plain GMRES when it stalls       */
    PIC_FGMRES_MIXED = 3     /* flexible GMRES(restart) in FP64 whose right
                                preconditioner is an FP32 GMRES solve of at most
                                `inner` Arnoldi steps, stopped as soon as it
                                meets what the outer iteration needs (the FP64
                                true residual still reaches tol); plain GMRES
                                when it stalls                                  */
} pic_gmres_method;

typedef struct {
    int method;              /* pic_gmres_method                              */
    int restart;             /* Krylov vectors per cycle (methods 1-3)        */
    int max_iter;            /* total iteration cap (outer iterations)        */
    double tol;              /* relative residual target                      */
    int inner;               /* PIC_FGMRES_MIXED: at most this many FP32 steps
                                per apply, 0..64 (0: 12)                       */
} pic_solve_opts;

typedef struct {
    int iterations;          /* Krylov iterations performed (the FP64 outer
                                iterations for PIC_FGMRES_LEARNED and
                                PIC_FGMRES_MIXED)                             */
    int restarts;
    int used_fallback;       /* 1 if the learned preconditioner was abandoned */
    double rel_residual;     /* final true |b - A x| / |b| (FP64)             */
    double seconds;          /* device time of the solve                      */
} pic_solve_info;

/* ---- lifecycle ---------------------------------------------------------- */
/* Replaces the Simulation constructor and createArrays
 * (PIC++/initialization.cpp:204-505, 6618-7395). */
pic_status pic_create(const pic_config* cfg, pic_ctx** out);
/* Replaces ~Simulation (PIC++/initialization.cpp:1278). */
pic_status pic_destroy(pic_ctx* ctx);
/* Last error message of this context ("" if none). */
const char* pic_last_error(const pic_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * work around the library's calls. */
void* pic_stream(pic_ctx* ctx);

/* ---- state -------------------------------------------------------------- */
/* Adds a particle species (ParticleTypeContainer, PIC++/particle.h:16-43):
 * charge q, mass m, macro-particle weight w, room for capacity particles. */
pic_status pic_add_species(pic_ctx* ctx, double q, double m, double w, long capacity, int* species_id);
/* Replaces the particle list of a species with n particles from host FP64
 * SoA arrays (the state Simulation::particles holds, PIC++/simulation.h:488).
 * ids may be NULL (then 0..n-1). */
pic_status pic_upload_particles(pic_ctx* ctx, int species, long n, const int* cell,
                                const double* ox, const double* oy, const double* oz,
                                const double* px, const double* py, const double* pz,
                                const int* ids);
/* Appends n particles (same arrays as pic_upload_particles) to a species,
 * after the ones it holds: the injection of new particles at an open
 * boundary (injectNewParticles, PIC++/mover.cpp:910-1000, whose positions
 * and momenta come from the caller here).  ids NULL numbers them on from
 * the species' last number. */
pic_status pic_append_particles(pic_ctx* ctx, int species, long n, const int* cell,
                                const double* ox, const double* oy, const double* oz,
                                const double* px, const double* py, const double* pz,
                                const int* ids);
/* Fills a species on the device with ppc particles per cell (the physical
 * cells of a wall box, from the reflecting wall at node 18 on in explicit
 * runs, as createParticles does, initialization.cpp:8152-8155): uniform
 * in-cell offsets, Maxwell-Juttner momenta of
 * temperature theta (kT/mc^2), boosted along x with Lorentz factor
 * drift_gamma (> 1) -- towards +x with alternate_drift 0, every other
 * particle towards -x with 1, all towards -x with -1.  Seeded and
 * independent of the launch shape.  A workload generator for runs too large to build on the
 * host; no reference counterpart (the reference's initialisers,
 * PIC++/initialization.cpp:8145-8574, are out of scope). */
pic_status pic_fill_species(pic_ctx* ctx, int species, int ppc, unsigned long long seed, double theta,
                            double drift_gamma, int alternate_drift);
/* Copies a species back in the current device order.  Any output pointer may
 * be NULL.  *n receives the count. */
pic_status pic_download_particles(pic_ctx* ctx, int species, long* n, int* cell,
                                  double* ox, double* oy, double* oz,
                                  double* px, double* py, double* pz, int* ids);
/* Sets E and B (3*N doubles each, layout above).  Replaces the grids the
 * initialisers fill (Efield/Bfield or bunemanE/B, PIC++/simulation.h:283-326). */
pic_status pic_upload_fields(pic_ctx* ctx, const double* E, const double* B);
/* Copies E, B and the last current J (3*N each; any may be NULL). */
pic_status pic_download_fields(pic_ctx* ctx, double* E, double* B, double* J);

/* ---- explicit Buneman / Tristan phases (PIC++/simulation.cpp:164-204) ---- */
/* tristanEvaluateBhalfStep (PIC++/fields.cpp:21-79) */
pic_status pic_tristan_evaluate_b_half_step(pic_ctx* ctx);
/* moveParticles (PIC++/mover.cpp:21-55): Boris push (moveParticleTristan,
 * PIC++/mover.cpp:718-808) for Buneman runs, the implicit mover (moveParticle,
 * PIC++/mover.cpp:194-491) for implicit runs; periodic wrap included
 * (exchangeParticles, PIC++/mover.cpp:1002-1210). */
pic_status pic_move_particles(pic_ctx* ctx);
/* tristanUpdateFlux (PIC++/momentum_collecting.cpp:20-82) */
pic_status pic_tristan_update_flux(pic_ctx* ctx);
/* tristanEvaluateE (PIC++/fields.cpp:81-150) */
pic_status pic_tristan_evaluate_e(pic_ctx* ctx);
/* nsteps of the whole Buneman branch of the step loop, fused kernels. */
pic_status pic_buneman_step(pic_ctx* ctx, int nsteps);

/* ---- implicit phases (PIC++/simulation.cpp:205-259) ---------------------- */
/* evaluateParticlesRotationTensor + updateElectroMagneticParameters
 * (PIC++/mover.cpp:810-841, PIC++/momentum_collecting.cpp:365-758):
 * J-hat, dielectric tensor, rho-hat and pressure tensor with their folds
 * and divergence corrections. */
pic_status pic_update_electromagnetic_parameters(pic_ctx* ctx);
/* evaluateElectricField (PIC++/fields.cpp:152-376) with
 * evaluateMaxwellEquationMatrix (fields.cpp:441-600) done matrix-free and
 * generalizedMinimalResidualMethod (specialmath.cpp:367-671) replaced by
 * the solver chosen in opts.  info may be NULL. */
pic_status pic_evaluate_electric_field(pic_ctx* ctx, const pic_solve_opts* opts, pic_solve_info* info);
/* evaluateMagneticField (PIC++/fields.cpp:2717-2773) */
pic_status pic_evaluate_magnetic_field(pic_ctx* ctx);
/* updateFields (PIC++/fields.cpp:422-439) */
pic_status pic_update_fields(pic_ctx* ctx);
/* One whole implicit step: the four calls above plus moveParticles. */
pic_status pic_implicit_step(pic_ctx* ctx, const pic_solve_opts* opts, pic_solve_info* info);
/* Copies the last moments: J-hat (3N), mu (9N, row-major 3x3 per node),
 * rho-hat with one low ghost layer ((nx+1)(ny+1)(nz+1) for 3-D, an axis of 1
 * stays 1) and the right part of the Maxwell system (3N).  NULL skips. */
pic_status pic_download_moments(pic_ctx* ctx, double* J, double* mu, double* rho_ext, double* rhs);
/* Applies the implicit Maxwell operator built from mu to x (3N each, host). */
pic_status pic_maxwell_apply(pic_ctx* ctx, const double* mu, const double* x, double* y);
/* Applies the transpose A(mu)^T to y (no reference counterpart; the
 * learned preconditioner's training back-propagates through it). */
pic_status pic_maxwell_apply_transpose(pic_ctx* ctx, const double* mu, const double* y, double* out);
/* Solves A(mu) x = rhs (host arrays) with the given options. */
pic_status pic_maxwell_solve(pic_ctx* ctx, const double* mu, const double* rhs, double* x,
                             const pic_solve_opts* opts, pic_solve_info* info);

/* ---- checkpoint ---------------------------------------------------------- */
/* Binary checkpoint of the device state: configuration, step counter, every
 * species (particles in their device order and precision, ids), the field
 * grids and the learned preconditioner's parameters when present.  Replaces
 * the text backup of outputSimulationBackup / readBackup
 * (PIC++/output.cpp:3432-3601, PIC++/input.cpp:342-624), which rounds to 10
 * digits (%15.10g) and reads the type table at type - 1 (input.cpp:608).
 * Loading needs a context of the same configuration (and tile extents); it
 * adds missing species, restores the particle order and tile offsets of the
 * last sort, and resumes bit for bit. */
pic_status pic_save_checkpoint(pic_ctx* ctx, const char* path);
pic_status pic_load_checkpoint(pic_ctx* ctx, const char* path);

/* ---- learned preconditioner --------------------------------------------- */
/* No counterpart in the reference (PIC++ solves with plain GMRES,
 * specialmath.cpp:367-671).  A linear 3-level encoder-decoder of 3x3x3
 * convolutions (16/32/64 channels, no activation, 2x2x2 average pooling,
 * nearest upsampling with skip concatenation) maps (r / s, mu_xx, mu_yy,
 * mu_zz) to a correction c / s, s = rms(r); z = g r + c approximates
 * A(mu)^-1 r, g a trained gate (training starts it at 1 where the identity
 * already reduces the residual, else at 0; g = 1 with a zero network is
 * plain GMRES); used by PIC_FGMRES_LEARNED.
 * Activations BF16, FP32 accumulation.  Input tensors have 16 channels
 * (0-2 residual, 3-5 mu diagonal, 6-15 zero), outputs 16 (0-2 used).
 * Parameters: one FP32 vector, per layer W[27][cout][cin] then b[cout],
 * the gate g last. */
typedef struct {
    int steps;                    /* Adam steps                                   */
    int batch;                    /* random fields per step                       */
    double lr;                    /* Adam step size                               */
    unsigned long long seed;      /* random fields                                */
    int smooth_max;               /* fields get 0..smooth_max binomial passes     */
    int source;                   /* 0: random fields on the context's operator;
                                     1: the triples recorded by pic_nn_record      */
    double supervised_weight;     /* source 1: weight w of |z - x|^2 / |x|^2 against
                                     (1 - w) |A z - b|^2 / |b|^2                    */
} pic_train_opts;
typedef struct {
    double first_loss, last_loss; /* relative residual loss of the first step / of the
                                     returned parameters (the lowest loss seen at a check
                                     every 50 steps, restored if the run degraded later) */
    double seconds;               /* device time                                  */
    int steps;
} pic_train_info;
/* Number of FP32 parameters. */
long pic_nn_param_count(void);
/* He-normal initialisation (seeded), zero biases, zero output layer. */
pic_status pic_nn_init(pic_ctx* ctx, unsigned long long seed);
pic_status pic_nn_set_params(pic_ctx* ctx, const float* params);
pic_status pic_nn_get_params(pic_ctx* ctx, float* params);
/* source 0: trains on the operator of the last
 * pic_update_electromagnetic_parameters (or the mu of the last
 * pic_maxwell_apply / pic_maxwell_solve): random fields r of unit rms on the
 * whole box, loss |A(mu) z - r|^2 / |r|^2 for z = network(r, mu diagonal),
 * back-propagated through A^T.  source 1: trains on the recorded triples
 * (b, mu, x) (pic_nn_record), each scaled to a unit-rms b, loss
 * w |z - x|^2 / |x|^2 + (1 - w) |A(mu) z - b|^2 / |b|^2 with
 * z = network(b, mu diagonal).  Box axes must be multiples of 4; periodic
 * boxes only. */
pic_status pic_nn_train(pic_ctx* ctx, const pic_train_opts* opts, pic_train_info* info);
/* The number of non-blocking mbarrier polls (test_wait) the network's
 * tensor-core convolutions make while waiting for their MMAs to complete
 * before they give up: the calls
 * that ran the network then return PIC_ERR_CUDA ("an MMA completion wait
 * ran out") and the context stays usable; the wait before a CTA releases
 * its tensor memory keeps the built-in bound, so no memory is released
 * under an MMA in flight.  0 restores the built-in bound (2^22 blocking
 * try_wait polls).  No
 * reference counterpart (failure detection of the device waits). */
pic_status pic_nn_wait_limit(pic_ctx* ctx, unsigned polls);
/* Starts keeping, for training, the (right-hand side, mu, FP64 solution)
 * triples that the next plain field solves of pic_evaluate_electric_field
 * (PIC_GMRES_REFERENCE / PIC_GMRES_RESTARTED) produce: the first capacity of
 * them, in FP32 on the device (60 bytes per cell each), over any number of
 * steps and reloaded species (runs); capacity 0 stops and frees them.  No
 * reference counterpart.  count (may be NULL) receives the number kept. */
pic_status pic_nn_record(pic_ctx* ctx, int capacity);
pic_status pic_nn_record_count(pic_ctx* ctx, int* count);
/* Forward pass on host input x0[n][d][h][w][16] (FP32, rounded to BF16),
 * out[n][d][h][w][16] FP32.  d, h, w multiples of 4. */
pic_status pic_nn_forward(pic_ctx* ctx, int n, int d, int h, int w, const float* x0, float* out);
/* Mean squared error against target[n][d][h][w][3] and its gradient with
 * respect to every parameter (grad: pic_nn_param_count() floats). */
pic_status pic_nn_loss_grad(pic_ctx* ctx, int n, int d, int h, int w, const float* x0, const float* target,
                            double* loss, float* grad);

/* ---- particle order ----------------------------------------------------- */
/* Stable counting sort of every species by tile-major cell key (no reference
 * counterpart; the reference keeps an unordered std::vector<Particle*>). */
pic_status pic_sort_particles(pic_ctx* ctx);
/* Source index of every slot after the last sort of a species (n ints). */
pic_status pic_download_permutation(pic_ctx* ctx, int species, long* n, int* perm);

/* ---- diagnostics -------------------------------------------------------- */
/* updateEnergy (PIC++/simulation.cpp:1506-1600) in normalised units:
 * out = {particle kinetic, electric, magnetic energy, px, py, pz momentum}. */
pic_status pic_energy(pic_ctx* ctx, double out[6]);

/* updateDensityParameters (PIC++/momentum_collecting.cpp:760-1020) on the
 * current particles: per species the concentration sum w S / V, the energy
 * density sum w gamma m S / V (fullEnergy, PIC++/particle.cpp:398-401) and
 * the bulk velocity (sum w p S / V) / energy density (0 where that is 0), with
 * the cell-centred weights S; and the charge density sum_s q_s conc_s. */
pic_status pic_update_density_parameters(pic_ctx* ctx);
/* Copies one species' conc (N), energy (N) and vel (3N) and the charge
 * density rho (N) of the last update; any pointer may be NULL. */
pic_status pic_download_density(pic_ctx* ctx, int species, double* conc, double* energy, double* vel, double* rho);

/* Phase timing, the GPU counterpart of the reference's per-phase clock()
 * prints (PIC++/mover.cpp:23-54, simulation.cpp:157-159).  enable = 1 starts
 * (and clears) recording of CUDA events around every phase on the context
 * stream; enable = 0 stops.  phase_ms (may be NULL) receives the accumulated
 * device milliseconds of PIC_PHASE_COUNT phases, launches the number of
 * kernels launched while recording. */
typedef enum {
    PIC_PHASE_SORT = 0, PIC_PHASE_FIELDS = 1, PIC_PHASE_PUSH_DEPOSIT = 2, PIC_PHASE_ASSEMBLE = 3,
    PIC_PHASE_MOMENTS = 4, PIC_PHASE_SOLVE = 5, PIC_PHASE_MOVER = 6,
    PIC_PHASE_DEPOSIT = 7,   /* the particle deposit kernels of the implicit moments alone
                                (part of PIC_PHASE_MOMENTS, which adds the grid passes) */
    PIC_PHASE_COUNT = 8
} pic_phase;
pic_status pic_profile(pic_ctx* ctx, int enable, double* phase_ms, long* launches);

/* ---- allocation-free diagnostics ---------------------------------------- */
/* No counterpart in the reference.  The sums of pic_energy (same order of
 * outputs) for device arrays owned by the caller, for callers that cannot
 * allocate device memory where they need them: hosts that fix a memory pool
 * at start-up and forbid later allocations, embedders whose device memory
 * comes from their own allocator.  Nothing is allocated: the partial sums
 * live in a file-scope device array of 548,864 bytes that every GPU loading
 * the library keeps until exit and that every call shares, so calls that
 * overlap on the GPU race.  The first call on a device looks that array's
 * device address up (cudaGetSymbolAddress) with the device current and
 * caches it; make no call on a device after a cudaDeviceReset of it.
 * Limit: at most
 * PIC_NOALLOC_MAX_SPECIES species (more returns PIC_ERR_ARG) and fewer than
 * 2^31 cells.
 * E, B: 3*nx*ny*nz FP64 device arrays (either may be NULL); per species s,
 * counts[s] particles of mass masses[s] and weight weights[s] with FP64
 * device momenta px[s], py[s], pz[s].  Runs on the given cudaStream_t, copies
 * the sums to the host array out and synchronises that stream before it
 * returns. */
#define PIC_NOALLOC_MAX_SPECIES 16
pic_status pic_energy_noalloc(int nx, int ny, int nz, double dx, double dy, double dz,
                              const double* E, const double* B, int nspecies, const long* counts,
                              const double* masses, const double* weights, const double* const* px,
                              const double* const* py, const double* const* pz, void* stream, double out[6]);

#ifdef __cplusplus
}
#endif
#endif
