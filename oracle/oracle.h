/*
 * oracle.h -- CPU restatement of PIC++'s per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against; nothing in the product (picpp_gb300/) links, loads or
 * calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it.
 *
 * Parity status: pinned.  tests/golden/ holds outputs of the reference
 * itself (PIC++ compiled from its own sources with a single-rank MPI stub,
 * driven by oracle/ref/harness.cpp), and tests/test_oracle_golden.py checks
 * this restatement against them.
 *
 * Conventions (shared with the CUDA path):
 *   - The box is periodic with nx*ny*nz cells.  Every grid array is stored
 *     component-major, then k, j, i with i fastest:  a[c][k][j][i].
 *   - Node (i,j,k) sits at (i*dx, j*dy, k*dz); cell (i,j,k) spans
 *     [i*dx,(i+1)*dx) x ...  The reference keeps two ghost layers on each
 *     side; its index r maps to our (r-2) mod n (PIC++/initialization.cpp:
 *     71-196 puts xgrid[2] at the left edge of the interior for one rank).
 *   - Particles carry an integer cell index (linear, i fastest) and an
 *     in-cell offset in [0,1) per axis, plus momentum p = m*gamma*v.
 *   - Units are the reference's normalised units: c = 1.
 */
#ifndef PICPP_ORACLE_H
#define PICPP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;
    int tx, ty, tz;         /* tile extents of the cell sort key            */
    double dx, dy, dz, dt;
    double theta, eta;      /* implicit time-centering (constants.h:40, initialization.cpp:320) */
    double cfix;            /* speed_of_light_correction (constants.h:45)    */
    int pressure_compat;    /* 1: deposit the pressure tensor at the stencil
                               loop index (momentum_collecting.cpp:565,577)  */
    int gmres_max_iter;     /* reference: maxGMRESIterations = 50            */
    double gmres_tol;       /* reference: maxErrorLevel = 1e-8               */
    int smoothing_count;    /* Simulation::smoothingCount passes per step     */
    double smoothing_parameter; /* Simulation::smoothingParameter             */
    int wall_x;             /* 1: conductor wall at x = 0 and an open boundary
                               at x = (nx - 2) dx (SUPER_CONDUCTOR_LEFT, one
                               rank); storage columns nx - 2 and nx - 1 are the
                               ghost cells beyond the open boundary and left of
                               the wall (3-D boxes).  The explicit path
                               reflects particles at node
                               ORC_TRISTAN_WALL_NODE, the implicit path at
                               the field wall x = 0                          */
    double e_right[3], b_right[3]; /* the open boundary's constant E and B
                               (ConstantBoundaryFieldEvaluator)              */
} orc_grid;

typedef struct {
    double q, m, w;
    long n;
    int *cell;
    double *ox, *oy, *oz;
    double *px, *py, *pz;
} orc_particles;

/* One pass of the periodic 3x3x3 smoothing of createSmoothingMatrix /
 * smooth*Parameter (PIC++/smoothing.cpp:105-137, 251-412, 535-739): weights
 * s/2, 1-s, s/2 per active axis, on ncomp planar components of N values. */
void orc_smooth(const orc_grid* g, double* a, int ncomp);

/* The implicit moments' smoothing passes (periodic placement only):
 * rho-hat with its low ghost layer, J-hat, mu. */
void orc_smooth_moments(const orc_grid* g, double* J, double* mu, double* rho_ext);

/* ---- explicit Buneman / Tristan path ---- */
/* The reflecting wall of the explicit path: xgrid[reflectingWallPoint]
 * (constants.h:64, reflectingWallPoint = 20 in the reference's ghosted
 * index, two ghost layers left of node 0 here). */
#define ORC_TRISTAN_WALL_NODE 18
void orc_wall_yee_ghosts(const orc_grid* g, double* E, double* B);
void orc_yee_b_half(const orc_grid* g, const double* E, double* B);
void orc_yee_e(const orc_grid* g, double* E, const double* B, const double* J);
void orc_boris_push(const orc_grid* g, orc_particles* p, const double* E, const double* B);
void orc_zigzag(const orc_grid* g, const orc_particles* p, double* J);
void orc_buneman_step(const orc_grid* g, orc_particles* sp, int nspecies,
                      double* E, double* B, double* J);

/* ---- cell sort ---- */
long orc_sort_key(const orc_grid* g, int cell);
void orc_counting_sort(const orc_grid* g, long n, const int* cell, long* perm);

/* ---- implicit path ---- */
void orc_gather_node(const orc_grid* g, int cell, double ox, double oy, double oz,
                     const double* F, double out[3]);
void orc_gather_cell(const orc_grid* g, int cell, double ox, double oy, double oz,
                     const double* F, double out[3]);
void orc_alpha(double beta, const double v[3], double gamma, const double E[3],
               const double B[3], double alpha[9]);
void orc_implicit_deposit(const orc_grid* g, const orc_particles* p,
                          const double* E, const double* B,
                          double* J, double* mu, double* rho, double* Pi);
long orc_pi_size(const orc_grid* g);
long orc_rho_ext_size(const orc_grid* g);
/* J-hat and mu vanish on the wall node of a conductor-wall box (no-op
 * otherwise), after the deposits and before orc_implicit_moments_finish. */
void orc_wall_node_moments(const orc_grid* g, double* J, double* mu);
void orc_implicit_moments_finish(const orc_grid* g, double* J, const double* rho, double* Pi,
                                 double* rho_ext);
void orc_maxwell_rhs(const orc_grid* g, const double* E, const double* B,
                     const double* J, const double* rho_ext, double* rhs);
void orc_maxwell_apply(const orc_grid* g, const double* mu, const double* x, double* y);
int  orc_gmres(const orc_grid* g, const double* mu, const double* rhs, double* x,
               double* rel_err_out);
void orc_field_update(const orc_grid* g, const double* Etheta, const double* E,
                      const double* B, double* Enew, double* Bnew);
void orc_implicit_push(const orc_grid* g, orc_particles* p, const double* E,
                       const double* B, const double* Etheta);
int  orc_implicit_step(const orc_grid* g, orc_particles* sp, int nspecies,
                       double* E, double* B, double* work);
long orc_implicit_work_size(const orc_grid* g);

/* ---- diagnostics ---- */
void orc_energy(const orc_grid* g, const orc_particles* sp, int nspecies,
                const double* E, const double* B, double out[6]);
/* updateDensityParameters (momentum_collecting.cpp:760-1020), periodic box:
 * conc[s][N], energy[s][N] (gamma m), vel[s][3][N] (momentum / energy
 * density), rho[N]. */
void orc_density_moments(const orc_grid* g, const orc_particles* sp, int nspecies, double* conc, double* energy,
                         double* vel, double* rho);

#ifdef __cplusplus
}
#endif
#endif
