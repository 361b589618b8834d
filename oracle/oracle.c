/*
 * oracle.c -- plain-C FP64 restatement of PIC++'s per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker for the CUDA path.  The
 * product library never links or calls it.  Conventions are in oracle.h.
 *
 * Each function names the reference lines (paths within the PICpp project)
 * whose arithmetic it restates.  Positions are kept as cell + offset instead
 * of the reference's absolute FP64 coordinates, so intermediate roundings
 * differ from the reference by a few ulp; tests/golden/ pins the result
 * against the reference's own output.
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared (see oracle/Makefile).
 * -ffp-contract=off keeps every multiply and add separately rounded, which is
 * what the FP64 CUDA path does with explicit __dmul_rn/__dadd_rn where
 * integer cell decisions depend on the result.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

#define PI_D 3.14159265358979323846
static const double FOUR_PI = 4.0 * PI_D;

/* ------------------------------------------------------------------ */
/* indexing                                                             */
/* ------------------------------------------------------------------ */
static inline int wrapi(int a, int n) { a %= n; return a < 0 ? a + n : a; }
static inline long NC(const orc_grid* g) { return (long)g->nx * g->ny * g->nz; }
static inline long IX(const orc_grid* g, int i, int j, int k) {
    return ((long)wrapi(k, g->nz) * g->ny + wrapi(j, g->ny)) * g->nx + wrapi(i, g->nx);
}
static inline void decode(const orc_grid* g, int cell, int* i, int* j, int* k) {
    *i = cell % g->nx;
    *j = (cell / g->nx) % g->ny;
    *k = cell / (g->nx * g->ny);
}

/* ------------------------------------------------------------------ */
/* relativistic kinematics (PIC++/particle.cpp:216-235, 366-390)        */
/* ------------------------------------------------------------------ */
static inline double gamma_of(const double p[3], double m) {
    double p2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    return sqrt(p2 / (m * m) + 1.0);                 /* particle.cpp:381-390 */
}
static inline void velocity_of(const double p[3], double m, double v[3]) {
    double g = gamma_of(p, m);                        /* particle.cpp:216-235 */
    v[0] = p[0] / (m * g); v[1] = p[1] / (m * g); v[2] = p[2] / (m * g);
}
/* Particle::evaluateVelocity, with its non-relativistic shortcut
 * (particle.cpp:366-379, relativisticPrecision = 1e-4, constants.h:39). */
static inline void evaluate_velocity(const double p[3], double m, double v[3]) {
    double p2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    if (p2 < 1e-4 * m * m) {
        v[0] = p[0] / m; v[1] = p[1] / m; v[2] = p[2] / m;
    } else {
        double gg = sqrt(p2 + m * m) / m;
        v[0] = p[0] / (m * gg); v[1] = p[1] / (m * gg); v[2] = p[2] / (m * gg);
    }
}
static inline void cross(const double a[3], const double b[3], double r[3]) {
    /* Vector3d::vectorMult (vector3d.cpp:82-88) */
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = -a[0] * b[2] + a[2] * b[0];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

/* Advance an in-cell offset by a displacement measured in cells and wrap
 * the cell index.  Shared rule with the CUDA path: s = floor(u); u -= s;
 * an offset that rounds up to exactly 1.0 moves into the next cell. */
static inline void advance_axis(double* u, int* c, double du, int n) {
    double un = *u + du;
    double s = floor(un);
    un = un - s;
    int ci = *c + (int)s;
    if (un >= 1.0) { un -= 1.0; ci += 1; }
    *u = un;
    *c = wrapi(ci, n);
}

/* ------------------------------------------------------------------ */
/* shape weights                                                        */
/* ------------------------------------------------------------------ */
/* Linear weights between the two nearest nodes (positions i*d).  This is
 * the top-hat overlap of a particle of half-width d/2 with node-centred
 * bins, correlationBspline case 0 (correlation.cpp:798-836) applied by
 * updateCorrelationMapNodeX (correlation.cpp:1283-1329); for the Yee path
 * the same weights come from correlation.cpp:484-496. */
static inline void node_w(double u, int c, int n, int idx[2], double w[2]) {
    if (n == 1) { idx[0] = idx[1] = 0; w[0] = 1.0; w[1] = 0.0; return; }
    double wl, wr;
    if (u < 0.5) { wl = 0.5 + (0.5 - u); wr = 1.0 - wl; }
    else         { wr = 0.5 + (u - 0.5); wl = 1.0 - wr; }
    idx[0] = c; idx[1] = c + 1; w[0] = wl; w[1] = wr;
}
/* Linear weights between the two nearest cell centres ((i+1/2)*d);
 * correlation.cpp:471-482 and updateCorrelationMapCellX
 * (correlation.cpp:1112-1158). */
static inline void cell_w(double u, int c, int n, int idx[2], double w[2]) {
    if (n == 1) { idx[0] = idx[1] = 0; w[0] = 1.0; w[1] = 0.0; return; }
    double wl, wr;
    if (u < 0.5) { wr = 0.5 + u; wl = 1.0 - wr; idx[0] = c - 1; idx[1] = c; }
    else         { wl = 0.5 + (1.0 - u); wr = 1.0 - wl; idx[0] = c; idx[1] = c + 1; }
    w[0] = wl; w[1] = wr;
}

/* ================================================================== */
/* Explicit Buneman / Tristan path                                      */
/* ================================================================== */
/* Yee staggering (PIC++/initialization.cpp:7146-7170 sizes, correlation.cpp
 * 585-591 indexing): Ex[cell][node][node], Ey[node][cell][node],
 * Ez[node][node][cell]; Bx[node][cell][cell], By[cell][node][cell],
 * Bz[cell][cell][node]; J like E. */

/* tristanEvaluateBhalfStep (fields.cpp:21-79) with the curls of
 * evaluateBunemanRotE{x,y,z} (fields.cpp:3273-3304). */
void orc_yee_b_half(const orc_grid* g, const double* E, double* B) {
    const long N = NC(g);
    const double* Ex = E; const double* Ey = E + N; const double* Ez = E + 2 * N;
    double* Bx = B; double* By = B + N; double* Bz = B + 2 * N;
    const double cdtd2 = g->cfix * g->dt / 2.0;
    const int y3 = g->ny > 1, z3 = g->nz > 1;
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                long c = IX(g, i, j, k);
                /* conductor wall: the reference updates Bx on nodes
                 * minI..maxI and By, Bz on cells minI..maxI-1 (fields.cpp
                 * 44-70); the ghost columns keep their values */
                if (g->wall_x && i == g->nx - 1) continue;
                const int cells = !(g->wall_x && i == g->nx - 2);
                double rx = 0.0;
                if (y3) rx += (Ez[IX(g, i, j + 1, k)] - Ez[c]) / g->dy;
                if (z3) rx -= (Ey[IX(g, i, j, k + 1)] - Ey[c]) / g->dz;
                double ry = -((Ez[IX(g, i + 1, j, k)] - Ez[c]) / g->dx);
                if (z3) ry += (Ex[IX(g, i, j, k + 1)] - Ex[c]) / g->dz;
                double rz = (Ey[IX(g, i + 1, j, k)] - Ey[c]) / g->dx;
                if (y3) rz -= (Ex[IX(g, i, j + 1, k)] - Ex[c]) / g->dy;
                Bx[c] = Bx[c] - rx * cdtd2;
                if (cells) {
                    By[c] = By[c] - ry * cdtd2;
                    Bz[c] = Bz[c] - rz * cdtd2;
                }
            }
}

/* tristanEvaluateE (fields.cpp:81-150), curls evaluateBunemanRotB{x,y,z}
 * (fields.cpp:3306-3337).  Conductor wall (wall_x): Ex on cells
 * minI..maxI-1, Ey and Ez on nodes minI..maxI, zero on the wall node and
 * E_right on the open boundary node (fields.cpp:116-121, 136-141); the
 * ghost columns keep their values. */
void orc_yee_e(const orc_grid* g, double* E, const double* B, const double* J) {
    const long N = NC(g);
    double* Ex = E; double* Ey = E + N; double* Ez = E + 2 * N;
    const double* Bx = B; const double* By = B + N; const double* Bz = B + 2 * N;
    const double* Jx = J; const double* Jy = J + N; const double* Jz = J + 2 * N;
    const int y3 = g->ny > 1, z3 = g->nz > 1;
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                long c = IX(g, i, j, k);
                double rx = 0.0;
                if (y3) rx += (Bz[c] - Bz[IX(g, i, j - 1, k)]) / g->dy;
                if (z3) rx -= (By[c] - By[IX(g, i, j, k - 1)]) / g->dz;
                double ry = -((Bz[c] - Bz[IX(g, i - 1, j, k)]) / g->dx);
                if (z3) ry += (Bx[c] - Bx[IX(g, i, j, k - 1)]) / g->dz;
                double rz = (By[c] - By[IX(g, i - 1, j, k)]) / g->dx;
                if (y3) rz -= (Bx[c] - Bx[IX(g, i, j - 1, k)]) / g->dy;
                if (g->wall_x && i == g->nx - 1) continue;
                if (!(g->wall_x && i == g->nx - 2)) Ex[c] = Ex[c] + (g->cfix * rx - FOUR_PI * Jx[c]) * g->dt;
                Ey[c] = Ey[c] + (g->cfix * ry - FOUR_PI * Jy[c]) * g->dt;
                Ez[c] = Ez[c] + (g->cfix * rz - FOUR_PI * Jz[c]) * g->dt;
                if (g->wall_x && i == 0) { Ey[c] = 0.0; Ez[c] = 0.0; }
                if (g->wall_x && i == g->nx - 2) { Ey[c] = g->e_right[1]; Ez[c] = g->e_right[2]; }
            }
}

/* The ghost columns of a conductor-wall box as the reference's one-rank
 * exchanges leave them (exchangeBuneman{E,B}field, fields_exchange.cpp
 * 2537-2661 and the y, z, B counterparts, non-periodic branch): the column
 * left of the wall (storage column nx - 1) holds zero in the cell-centred
 * components Ex, By, Bz and the wall node's value in Ey, Ez, Bx; the column
 * beyond the open boundary keeps whatever it held. */
void orc_wall_yee_ghosts(const orc_grid* g, double* E, double* B) {
    if (!g->wall_x) return;
    const long N = NC(g);
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j) {
            const long c = IX(g, g->nx - 1, j, k), w = IX(g, 0, j, k);
            E[c] = 0.0; E[N + c] = E[N + w]; E[2 * N + c] = E[2 * N + w];
            B[c] = B[w]; B[N + c] = 0.0; B[2 * N + c] = 0.0;
        }
}

/* correlationBunemanEBfieldsWithoutMaps (correlation.cpp:441-600): E and B
 * at the particle from the staggered Yee grids with linear weights. */
static void yee_gather(const orc_grid* g, int cell, double ox, double oy, double oz,
                       const double* E, const double* B, double e[3], double b[3]) {
    const long N = NC(g);
    int i, j, k; decode(g, cell, &i, &j, &k);
    int nX[2], cX[2], nY[2], cY[2], nZ[2], cZ[2];
    double wnX[2], wcX[2], wnY[2], wcY[2], wnZ[2], wcZ[2];
    node_w(ox, i, g->nx, nX, wnX); cell_w(ox, i, g->nx, cX, wcX);
    node_w(oy, j, g->ny, nY, wnY); cell_w(oy, j, g->ny, cY, wcY);
    node_w(oz, k, g->nz, nZ, wnZ); cell_w(oz, k, g->nz, cZ, wcZ);
    e[0] = e[1] = e[2] = 0.0; b[0] = b[1] = b[2] = 0.0;
    for (int a = 0; a < 2; ++a)
        for (int bb = 0; bb < 2; ++bb)
            for (int cc = 0; cc < 2; ++cc) {
                e[0] += E[IX(g, cX[a], nY[bb], nZ[cc])] * wcX[a] * wnY[bb] * wnZ[cc];
                e[1] += E[N + IX(g, nX[a], cY[bb], nZ[cc])] * wnX[a] * wcY[bb] * wnZ[cc];
                e[2] += E[2 * N + IX(g, nX[a], nY[bb], cZ[cc])] * wnX[a] * wnY[bb] * wcZ[cc];
                b[0] += B[IX(g, nX[a], cY[bb], cZ[cc])] * wnX[a] * wcY[bb] * wcZ[cc];
                b[1] += B[N + IX(g, cX[a], nY[bb], cZ[cc])] * wcX[a] * wnY[bb] * wcZ[cc];
                b[2] += B[2 * N + IX(g, cX[a], cY[bb], nZ[cc])] * wcX[a] * wcY[bb] * wnZ[cc];
            }
}

/* The x move of moveParticleTristan next to a conductor wall
 * (mover.cpp:744-772): x = x^n + v_x dt without a periodic wrap; a
 * position left of the reflecting wall (node ORC_TRISTAN_WALL_NODE) is
 * mirrored there (bit 1 of the result: p_x is to be reversed,
 * reflectMomentumX); a position beyond the open boundary x = (nx - 2) dx
 * sets bit 2 (escaped: the particle still deposits its current this step
 * and is erased after it).  Cell and offset of the result in c, u. */
static int tristan_wall_x(const orc_grid* g, int* c, double* u, double disp) {
    const int W = ORC_TRISTAN_WALL_NODE;
    const double s = *u + disp;
    const double fl = floor(s);
    int cn = *c + (int)fl;
    double un = s - fl;
    if (un >= 1.0) { un -= 1.0; cn += 1; }
    int r = 0;
    if (cn < W) {   /* x' = 2 W - x */
        if (un > 0.0) { cn = 2 * W - cn - 1; un = 1.0 - un; }
        else cn = 2 * W - cn;
        r = 1;
    }
    if (cn > g->nx - 2 || (cn == g->nx - 2 && un > 0.0)) r |= 2;
    *c = cn; *u = un;
    return r;
}

/* moveParticleTristan (mover.cpp:718-742): Boris push, then x += v*dt.
 * Periodic wrap replaces exchangeParticles (mover.cpp:1002-1210).  Note the
 * reference's rotation factor f = 2/sqrt(1 + t^2) (mover.cpp:738), kept. */
void orc_boris_push(const orc_grid* g, orc_particles* p, const double* E, const double* B) {
    const double beta = p->q * g->dt / (2.0 * p->m);  /* Particle::beta, particle.cpp:47 */
    for (long n = 0; n < p->n; ++n) {
        if (p->cell[n] < 0) continue;   /* escaped (wall_x), erased after the step */
        double e[3], b[3];
        yee_gather(g, p->cell[n], p->ox[n], p->oy[n], p->oz[n], E, B, e, b);
        double s = p->q * g->dt * 0.5;
        double dp[3] = {e[0] * s, e[1] * s, e[2] * s};
        double mom[3] = {p->px[n] + dp[0], p->py[n] + dp[1], p->pz[n] + dp[2]};
        double gam = gamma_of(mom, p->m);
        double bs = beta / gam;
        double b2 = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
        double f = 2.0 / sqrt(1.0 + bs * bs * b2);
        double pxb[3]; cross(mom, b, pxb);
        double tm[3] = {mom[0] + pxb[0] * bs, mom[1] + pxb[1] * bs, mom[2] + pxb[2] * bs};
        double txb[3]; cross(tm, b, txb);
        double fb = f * bs;
        mom[0] += txb[0] * fb + dp[0];
        mom[1] += txb[1] * fb + dp[1];
        mom[2] += txb[2] * fb + dp[2];
        p->px[n] = mom[0]; p->py[n] = mom[1]; p->pz[n] = mom[2];
        double v[3]; velocity_of(mom, p->m, v);
        int i, j, k; decode(g, p->cell[n], &i, &j, &k);
        double ux = p->ox[n], uy = p->oy[n], uz = p->oz[n];
        if (g->wall_x) {
            if (tristan_wall_x(g, &i, &ux, (v[0] * g->dt) * (1.0 / g->dx)) & 1) p->px[n] = -p->px[n];
        } else {
            advance_axis(&ux, &i, (v[0] * g->dt) * (1.0 / g->dx), g->nx);
        }
        advance_axis(&uy, &j, (v[1] * g->dt) * (1.0 / g->dy), g->ny);
        advance_axis(&uz, &k, (v[2] * g->dt) * (1.0 / g->dz), g->nz);
        p->ox[n] = ux; p->oy[n] = uy; p->oz[n] = uz;
        p->cell[n] = (int)IX(g, i, j, k);
    }
}

/* One axis of the zigzag split (momentum_collecting.cpp:91-96, 200-221):
 * the new position X (length units from the new cell's lower face), the
 * old position P = X - v*dt, the relay point R and the cell shift of the
 * first segment. */
static inline void zig_axis(double X, double v, double dt, double d, int n, int mirror,
                            double* P, double* R, int* sh) {
    double prev = X - v * dt;
    /* the particle's cell is the one right of the reflecting wall and it
     * moves away from it: an old position left of the wall is mirrored
     * (momentum_collecting.cpp:93-99) */
    if (mirror && v > 0 && prev < 0) prev = -prev;
    if (n == 1) { *P = prev; *R = (X + prev) / 2; *sh = 0; return; }
    int s = (int)floor(prev / d);
    double r = (X + prev) / 2;
    if (s != 0) r = (s > 0 ? s : 0) * d;             /* max2(grid[previ], grid[i]) */
    *P = prev; *R = r; *sh = s;
}

/* addParticleFluxZigzag (momentum_collecting.cpp:84-230), 3-D and 2-D
 * branches: the Umeda charge-conserving current of one particle. */
void orc_zigzag(const orc_grid* g, const orc_particles* p, double* J) {
    const long N = NC(g);
    double* Jx = J; double* Jy = J + N; double* Jz = J + 2 * N;
    const double vol = g->dx * g->dy * g->dz;
    const double fcd = p->q * p->w / vol;
    const int y3 = g->ny > 1, z3 = g->nz > 1;
    for (long n = 0; n < p->n; ++n) {
        if (p->cell[n] < 0) continue;
        double mom[3] = {p->px[n], p->py[n], p->pz[n]};
        double v[3]; velocity_of(mom, p->m, v);
        int i, j, k; decode(g, p->cell[n], &i, &j, &k);
        double X = p->ox[n] * g->dx, Y = p->oy[n] * g->dy, Z = p->oz[n] * g->dz;
        double PX, PY, PZ, RX, RY, RZ; int si, sj, sk;
        zig_axis(X, v[0], g->dt, g->dx, g->nx, g->wall_x && i == ORC_TRISTAN_WALL_NODE, &PX, &RX, &si);
        zig_axis(Y, v[1], g->dt, g->dy, g->ny, 0, &PY, &RY, &sj);
        zig_axis(Z, v[2], g->dt, g->dz, g->nz, 0, &PZ, &RZ, &sk);
        double Fx1 = fcd * (RX - PX) / g->dt;
        double Fy1 = fcd * (RY - PY) / g->dt;
        double Fz1 = fcd * (RZ - PZ) / g->dt;
        double Fx2 = fcd * (X - RX) / g->dt;
        double Fy2 = fcd * v[1] - Fy1;
        double Fz2 = fcd * v[2] - Fz1;
        double Wx1 = (PX + RX) / (2 * g->dx) - si;
        double Wy1 = (PY + RY) / (2 * g->dy) - sj;
        double Wz1 = (PZ + RZ) / (2 * g->dz) - sk;
        double Wx2 = (X + RX) / (2 * g->dx);
        double Wy2 = (Y + RY) / (2 * g->dy);
        double Wz2 = (Z + RZ) / (2 * g->dz);
        if (!y3) { Wy1 = 0.0; Wy2 = 0.0; }
        if (!z3) { Wz1 = 0.0; Wz2 = 0.0; }
        int a = i + si, b = j + sj, c = k + sk;
        /* first segment, from the old position to the relay point */
        Jx[IX(g, a, b, c)] += Fx1 * (1.0 - Wy1) * (1.0 - Wz1);
        if (y3) Jx[IX(g, a, b + 1, c)] += Fx1 * Wy1 * (1.0 - Wz1);
        if (z3) Jx[IX(g, a, b, c + 1)] += Fx1 * (1.0 - Wy1) * Wz1;
        if (y3 && z3) Jx[IX(g, a, b + 1, c + 1)] += Fx1 * Wy1 * Wz1;
        Jy[IX(g, a, b, c)] += Fy1 * (1.0 - Wx1) * (1.0 - Wz1);
        Jy[IX(g, a + 1, b, c)] += Fy1 * Wx1 * (1.0 - Wz1);
        if (z3) Jy[IX(g, a, b, c + 1)] += Fy1 * (1.0 - Wx1) * Wz1;
        if (z3) Jy[IX(g, a + 1, b, c + 1)] += Fy1 * Wx1 * Wz1;
        Jz[IX(g, a, b, c)] += Fz1 * (1.0 - Wx1) * (1.0 - Wy1);
        if (y3) Jz[IX(g, a, b + 1, c)] += Fz1 * (1.0 - Wx1) * Wy1;
        Jz[IX(g, a + 1, b, c)] += Fz1 * Wx1 * (1.0 - Wy1);
        if (y3) Jz[IX(g, a + 1, b + 1, c)] += Fz1 * Wx1 * Wy1;
        /* second segment, from the relay point to the new position */
        Jx[IX(g, i, j, k)] += Fx2 * (1.0 - Wy2) * (1.0 - Wz2);
        if (y3) Jx[IX(g, i, j + 1, k)] += Fx2 * Wy2 * (1.0 - Wz2);
        if (z3) Jx[IX(g, i, j, k + 1)] += Fx2 * (1.0 - Wy2) * Wz2;
        if (y3 && z3) Jx[IX(g, i, j + 1, k + 1)] += Fx2 * Wy2 * Wz2;
        Jy[IX(g, i, j, k)] += Fy2 * (1.0 - Wx2) * (1.0 - Wz2);
        Jy[IX(g, i + 1, j, k)] += Fy2 * Wx2 * (1.0 - Wz2);
        if (z3) Jy[IX(g, i, j, k + 1)] += Fy2 * (1.0 - Wx2) * Wz2;
        if (z3) Jy[IX(g, i + 1, j, k + 1)] += Fy2 * Wx2 * Wz2;
        Jz[IX(g, i, j, k)] += Fz2 * (1.0 - Wx2) * (1.0 - Wy2);
        if (y3) Jz[IX(g, i, j + 1, k)] += Fz2 * (1.0 - Wx2) * Wy2;
        Jz[IX(g, i + 1, j, k)] += Fz2 * Wx2 * (1.0 - Wy2);
        if (y3) Jz[IX(g, i + 1, j + 1, k)] += Fz2 * Wx2 * Wy2;
    }
}

void orc_smooth(const orc_grid* g, double* a, int ncomp) {
    const long N = NC(g);
    const double sp = g->smoothing_parameter;
    double w[3][3];
    const int n[3] = {g->nx, g->ny, g->nz};
    for (int ax = 0; ax < 3; ++ax) {
        w[ax][0] = n[ax] > 1 ? sp / 2 : 0.0;
        w[ax][1] = n[ax] > 1 ? 1 - sp : 1.0;
        w[ax][2] = n[ax] > 1 ? sp / 2 : 0.0;
    }
    double* t = (double*)malloc(sizeof(double) * (size_t)N);
    for (int c = 0; c < ncomp; ++c) {
        double* f = a + (long)c * N;
        for (int k = 0; k < g->nz; ++k)
            for (int j = 0; j < g->ny; ++j)
                for (int i = 0; i < g->nx; ++i) {
                    double s = 0.0;
                    for (int di = -1; di <= 1; ++di)
                        for (int dj = -1; dj <= 1; ++dj)
                            for (int dk = -1; dk <= 1; ++dk) {
                                const double wt = w[0][di + 1] * w[1][dj + 1] * w[2][dk + 1];
                                if (wt == 0.0) continue;
                                s += f[IX(g, wrapi(i + di, g->nx), wrapi(j + dj, g->ny), wrapi(k + dk, g->nz))] * wt;
                            }
                    t[IX(g, i, j, k)] = s;
                }
        memcpy(f, t, sizeof(double) * (size_t)N);
    }
    free(t);
}

/* The BUNEMAN branch of Simulation::simulate (simulation.cpp:164-204): B half
 * step, push, B half step, current (smoothed smoothingCount times,
 * simulation.cpp:186-188), E step. */
void orc_buneman_step(const orc_grid* g, orc_particles* sp, int nspecies,
                      double* E, double* B, double* J) {
    orc_wall_yee_ghosts(g, E, B);
    orc_yee_b_half(g, E, B);
    for (int s = 0; s < nspecies; ++s) orc_boris_push(g, &sp[s], E, B);
    orc_yee_b_half(g, E, B);
    memset(J, 0, sizeof(double) * 3 * NC(g));
    for (int s = 0; s < nspecies; ++s) orc_zigzag(g, &sp[s], J);
    for (int q = 0; q < g->smoothing_count; ++q) orc_smooth(g, J, 3);
    orc_yee_e(g, E, B, J);
    if (!g->wall_x) return;
    /* particles beyond the open boundary were marked escaped by the mover
     * and deposited their current; eraseEscapedPaticles (mover.cpp:167-192)
     * drops them now (cell -1 here; the caller compacts the arrays) */
    for (int s = 0; s < nspecies; ++s)
        for (long n = 0; n < sp[s].n; ++n) {
            if (sp[s].cell[n] < 0) continue;
            int i, j, k; decode(g, sp[s].cell[n], &i, &j, &k);
            if (i > g->nx - 2 || (i == g->nx - 2 && sp[s].ox[n] > 0.0)) sp[s].cell[n] = -1;
        }
}

/* ================================================================== */
/* Cell sort (no reference counterpart: the reference keeps unordered    */
/* std::vector<Particle*>).  Stable counting sort by a tile-major key.   */
/* ================================================================== */
long orc_sort_key(const orc_grid* g, int cell) {
    int i, j, k; decode(g, cell, &i, &j, &k);
    int ntx = g->nx / g->tx, nty = g->ny / g->ty;
    long tile = ((long)(k / g->tz) * nty + (j / g->ty)) * ntx + (i / g->tx);
    long local = ((long)(k % g->tz) * g->ty + (j % g->ty)) * g->tx + (i % g->tx);
    return tile * ((long)g->tx * g->ty * g->tz) + local;
}

/* perm[d] = source index of the particle that goes to slot d. */
void orc_counting_sort(const orc_grid* g, long n, const int* cell, long* perm) {
    long nc = NC(g);
    long* cnt = (long*)calloc((size_t)nc + 1, sizeof(long));
    long* key = (long*)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
    for (long a = 0; a < n; ++a) { key[a] = orc_sort_key(g, cell[a]); cnt[key[a] + 1]++; }
    for (long c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    for (long a = 0; a < n; ++a) perm[cnt[key[a]]++] = a;
    free(cnt); free(key);
}

/* ================================================================== */
/* Implicit (theta-scheme) path                                          */
/* ================================================================== */
/* correlationGeneralEfield (correlation.cpp:103-164): 8-node gather of a
 * node-centred 3-vector field. */
void orc_gather_node(const orc_grid* g, int cell, double ox, double oy, double oz,
                     const double* F, double out[3]) {
    const long N = NC(g);
    int i, j, k; decode(g, cell, &i, &j, &k);
    int X[2], Y[2], Z[2]; double wx[2], wy[2], wz[2];
    node_w(ox, i, g->nx, X, wx); node_w(oy, j, g->ny, Y, wy); node_w(oz, k, g->nz, Z, wz);
    out[0] = out[1] = out[2] = 0.0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                long id = IX(g, X[a], Y[b], Z[c]);
                double w = wx[a] * wy[b] * wz[c];
                out[0] += F[id] * w; out[1] += F[N + id] * w; out[2] += F[2 * N + id] * w;
            }
}

/* correlationBfield (correlation.cpp:23-58): 8-cell gather of a
 * cell-centred 3-vector field. */
void orc_gather_cell(const orc_grid* g, int cell, double ox, double oy, double oz,
                     const double* F, double out[3]) {
    const long N = NC(g);
    int i, j, k; decode(g, cell, &i, &j, &k);
    int X[2], Y[2], Z[2]; double wx[2], wy[2], wz[2];
    cell_w(ox, i, g->nx, X, wx); cell_w(oy, j, g->ny, Y, wy); cell_w(oz, k, g->nz, Z, wz);
    out[0] = out[1] = out[2] = 0.0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                long id = IX(g, X[a], Y[b], Z[c]);
                double w = wx[a] * wy[b] * wz[c];
                out[0] += F[id] * w; out[1] += F[N + id] * w; out[2] += F[2 * N + id] * w;
            }
}

/* evaluateAlphaRotationTensor (mover.cpp:851-880):
 * alpha_ij = (delta_ij + bs^2 B_i B_j - bs eps_{jil} B_l) / (G (1 + bs^2 B^2)),
 * G = beta E.v + gamma, bs = beta / G. */
void orc_alpha(double beta, const double v[3], double gamma, const double E[3],
               const double B[3], double alpha[9]) {
    double G = (beta * (E[0] * v[0] + E[1] * v[1] + E[2] * v[2])) + gamma;
    double bs = beta / G;
    double b2c = bs * bs;
    double den = G * (1 + b2c * (B[0] * B[0] + B[1] * B[1] + B[2] * B[2]));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double r = (i == j ? 1.0 : 0.0) + (b2c * B[i] * B[j]);
            /* -bs * eps_{j i l} B_l (LeviCivita[j][i][l], initialization.cpp:52-57) */
            for (int l = 0; l < 3; ++l) {
                int e = 0;
                if (j != i && i != l && j != l) e = ((i - j + 3) % 3 == 1) ? 1 : -1; /* eps_{jil} */
                if (e != 0) r -= (bs * e * B[l]);
            }
            alpha[3 * i + j] = r / den;
        }
}

/* ------------------------------------------------------------------ */
/* Reference-layout helpers for the pressure-tensor path.               */
/* The reference folds Pi with the wrong partner (momentum_exchange.cpp  */
/* 1643-1741 pairs ghost cell r with r+N+1 instead of r+N) and deposits  */
/* it at the stencil loop index in y and z (momentum_collecting.cpp:565, */
/* 577).  J-hat and rho-hat then pick the result up through div(Pi) on   */
/* ghost nodes.  With pressure_compat set these steps run on arrays in   */
/* the reference's ghosted index space r (interior cells r = 2..n+1) so  */
/* that the outcome is the reference's; with it clear the same formulas  */
/* run on the periodic box.                                              */
/* ------------------------------------------------------------------ */
typedef struct { int n, ce, ne, g; } gaxis;      /* cells, nodes, ghost offset */
static inline gaxis mk_axis(int n) {
    gaxis a; a.n = n;
    if (n > 1) { a.ce = n + 4; a.ne = n + 5; a.g = 2; } else { a.ce = 1; a.ne = 1; a.g = 0; }
    return a;
}
static inline int gclamp(const gaxis* a, int r) { return a->n > 1 ? r : 0; }
static inline int gphys(const gaxis* a, int r) { return a->n > 1 ? wrapi(r - 2, a->n) : 0; }

long orc_pi_size(const orc_grid* g) {
    if (!g->pressure_compat) return 9 * NC(g);
    gaxis ax = mk_axis(g->nx), ay = mk_axis(g->ny), az = mk_axis(g->nz);
    return 9L * ax.ce * ay.ce * az.ce;
}
long orc_rho_ext_size(const orc_grid* g) {
    return (long)(g->nx > 1 ? g->nx + 1 : 1) * (g->ny > 1 ? g->ny + 1 : 1) * (g->nz > 1 ? g->nz + 1 : 1);
}

/* evaluateParticlesRotationTensor (mover.cpp:810-841) + the particle loops of
 * updateElectroMagneticParameters (momentum_collecting.cpp:397-584):
 * accumulates J-hat (node, 3), the dielectric tensor mu (node, 9, row-major
 * a*3+b), rho-hat (cell) and the pressure tensor Pi (cell, 9; reference
 * ghosted layout when pressure_compat is set, see orc_pi_size).  The
 * caller zeroes the outputs before the first species. */
void orc_implicit_deposit(const orc_grid* g, const orc_particles* p,
                          const double* E, const double* B,
                          double* J, double* mu, double* rho, double* Pi) {
    const long N = NC(g);
    const double vol = g->dx * g->dy * g->dz;
    const double beta = 0.5 * p->q * g->dt / p->m;
    const double omega = p->w * g->theta * g->dt * g->dt * 2 * PI_D * p->q * p->q / p->m;
    const double qw = p->q * p->w;
    gaxis ax = mk_axis(g->nx), ay = mk_axis(g->ny), az = mk_axis(g->nz);
    const long PN = g->pressure_compat ? (long)ax.ce * ay.ce * az.ce : N;
    for (long n = 0; n < p->n; ++n) {
        if (p->cell[n] < 0) continue;   /* escaped (wall_x), erased after the step */
        double mom[3] = {p->px[n], p->py[n], p->pz[n]};
        double gam = gamma_of(mom, p->m);
        double v[3]; velocity_of(mom, p->m, v);
        double e[3], b[3];
        orc_gather_node(g, p->cell[n], p->ox[n], p->oy[n], p->oz[n], E, e);
        orc_gather_cell(g, p->cell[n], p->ox[n], p->oy[n], p->oz[n], B, b);
        double al[9]; orc_alpha(beta, v, gam, e, b, al);
        double vg[3] = {v[0] * gam, v[1] * gam, v[2] * gam};
        double rv[3];
        for (int a = 0; a < 3; ++a) rv[a] = al[3 * a] * vg[0] + al[3 * a + 1] * vg[1] + al[3 * a + 2] * vg[2];
        int i, j, k; decode(g, p->cell[n], &i, &j, &k);
        int X[2], Y[2], Z[2]; double wx[2], wy[2], wz[2];
        node_w(p->ox[n], i, g->nx, X, wx); node_w(p->oy[n], j, g->ny, Y, wy); node_w(p->oz[n], k, g->nz, Z, wz);
        for (int a = 0; a < 2; ++a)
            for (int bb = 0; bb < 2; ++bb)
                for (int c = 0; c < 2; ++c) {
                    if ((g->ny == 1 && bb) || (g->nz == 1 && c)) continue;
                    long id = IX(g, X[a], Y[bb], Z[c]);
                    double corr = wx[a] * wy[bb] * wz[c] / vol;
                    for (int d = 0; d < 3; ++d) J[d * N + id] += rv[d] * (qw * corr);
                    double om = omega * corr;
                    for (int d = 0; d < 9; ++d) mu[d * N + id] = mu[d * N + id] - al[d] * om;
                }
        double ten[9];
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) ten[3 * a + c] = rv[a] * rv[c];
        cell_w(p->ox[n], i, g->nx, X, wx); cell_w(p->oy[n], j, g->ny, Y, wy); cell_w(p->oz[n], k, g->nz, Z, wz);
        for (int a = 0; a < 2; ++a)
            for (int bb = 0; bb < 2; ++bb)
                for (int c = 0; c < 2; ++c) {
                    if ((g->ny == 1 && bb) || (g->nz == 1 && c)) continue;
                    /* conductor wall: the ghost cell left of the wall is
                     * mirrored onto the first cell (momentum_collecting.cpp:
                     * 560-568) */
                    const int mirror = g->wall_x && X[a] < 0;
                    long id = IX(g, mirror ? -X[a] - 1 : X[a], Y[bb], Z[c]);
                    double corr = wx[a] * wy[bb] * wz[c] / vol;
                    rho[id] += qw * corr;
                    long pid;
                    if (g->pressure_compat) {
                        /* x: the reference cell index of the stencil point
                         * (interior cell i is r = i + 2, neighbours r +- 1,
                         * no wrap); y, z: the loop counters j, k
                         * (momentum_collecting.cpp:565,577). */
                        int rx = ax.n > 1 ? (mirror ? -X[a] - 1 : X[a]) + ax.g : 0;
                        int ry = ay.n > 1 ? bb : 0;
                        int rz = az.n > 1 ? c : 0;
                        pid = ((long)rz * ay.ce + ry) * ax.ce + rx;
                    } else {
                        pid = id;
                    }
                    for (int d = 0; d < 9; ++d) Pi[d * PN + pid] += qw * corr * ten[d];
                }
    }
}

/* sumCellMatrixParameters{X,Y,Z} (momentum_exchange.cpp:1643-1741),
 * single-rank periodic branch, on the reference-layout Pi. */
static void pi_fold_reference(const orc_grid* g, double* P) {
    gaxis ax = mk_axis(g->nx), ay = mk_axis(g->ny), az = mk_axis(g->nz);
    const long PN = (long)ax.ce * ay.ce * az.ce;
#define PG(d, x, y, z) P[(d) * PN + ((long)(z) * ay.ce + (y)) * ax.ce + (x)]
    for (int d = 0; d < 9; ++d) {
        if (ax.n > 1 && !g->wall_x)   /* no x fold next to a wall (one rank) */
            for (int y = 0; y < ay.ce; ++y)
                for (int z = 0; z < az.ce; ++z)
                    for (int t = 0; t < 3; ++t) {
                        PG(d, ax.ce - 1 - t, y, z) = PG(d, ax.ce - 1 - t, y, z) + PG(d, 2 - t, y, z);
                        PG(d, 2 - t, y, z) = PG(d, ax.ce - 1 - t, y, z);
                    }
        if (ay.n > 1)
            for (int x = 0; x < ax.ce; ++x)
                for (int z = 0; z < az.ce; ++z)
                    for (int t = 0; t < 3; ++t) {
                        PG(d, x, ay.ce - 1 - t, z) = PG(d, x, ay.ce - 1 - t, z) + PG(d, x, 2 - t, z);
                        PG(d, x, 2 - t, z) = PG(d, x, ay.ce - 1 - t, z);
                    }
        if (az.n > 1)
            for (int x = 0; x < ax.ce; ++x)
                for (int y = 0; y < ay.ce; ++y)
                    for (int t = 0; t < 3; ++t) {
                        PG(d, x, y, az.ce - 1 - t) = PG(d, x, y, az.ce - 1 - t) + PG(d, x, y, 2 - t);
                        PG(d, x, y, 2 - t) = PG(d, x, y, az.ce - 1 - t);
                    }
    }
#undef PG
}

/* evaluateDivPressureTensor (fields.cpp:3158-3223) at one node, reading the
 * pressure tensor through an accessor P(a, b, i, j, k) of cell indices. */
#define DIV_PI_BODY(PT, i, j, k, out)                                                                  \
    for (int col = 0; col < 3; ++col) {                                                                \
        double rA = (PT(0, col, i, j, k) + PT(0, col, i, j - 1, k) + PT(0, col, i, j, k - 1) + PT(0, col, i, j - 1, k - 1)) * 0.25;       \
        double lA = (PT(0, col, i - 1, j, k) + PT(0, col, i - 1, j - 1, k) + PT(0, col, i - 1, j, k - 1) + PT(0, col, i - 1, j - 1, k - 1)) * 0.25; \
        double bA = 0, fA = 0, tA = 0, boA = 0;                                                        \
        if (y3) {                                                                                       \
            bA = (PT(1, col, i, j, k) + PT(1, col, i - 1, j, k) + PT(1, col, i, j, k - 1) + PT(1, col, i - 1, j, k - 1)) * 0.25;  \
            fA = (PT(1, col, i, j - 1, k) + PT(1, col, i - 1, j - 1, k) + PT(1, col, i, j - 1, k - 1) + PT(1, col, i - 1, j - 1, k - 1)) * 0.25; \
        }                                                                                               \
        if (z3) {                                                                                       \
            tA = (PT(2, col, i, j, k) + PT(2, col, i, j - 1, k) + PT(2, col, i - 1, j, k) + PT(2, col, i - 1, j - 1, k)) * 0.25;  \
            boA = (PT(2, col, i, j, k - 1) + PT(2, col, i, j - 1, k - 1) + PT(2, col, i - 1, j, k - 1) + PT(2, col, i - 1, j - 1, k - 1)) * 0.25; \
        }                                                                                               \
        out[col] = ((rA - lA) / g->dx) + ((bA - fA) / g->dy) + ((tA - boA) / g->dz);                 \
    }

/* evaluateDivFlux (fields.cpp:3060-3156) at one cell through an accessor
 * JF(d, i, j, k) of node indices. */
#define DIV_J_BODY(JF, i, j, k, div)                                                                   \
    {                                                                                                   \
        double rX = (JF(0, i + 1, j, k) + JF(0, i + 1, j + 1, k) + JF(0, i + 1, j, k + 1) + JF(0, i + 1, j + 1, k + 1)) * 0.25; \
        double lX = (JF(0, i, j, k) + JF(0, i, j + 1, k) + JF(0, i, j, k + 1) + JF(0, i, j + 1, k + 1)) * 0.25; \
        double rY = 0, lY = 0, rZ = 0, lZ = 0;                                                         \
        if (y3) {                                                                                       \
            rY = (JF(1, i, j + 1, k) + JF(1, i + 1, j + 1, k) + JF(1, i, j + 1, k + 1) + JF(1, i + 1, j + 1, k + 1)) * 0.25; \
            lY = (JF(1, i, j, k) + JF(1, i + 1, j, k) + JF(1, i, j, k + 1) + JF(1, i + 1, j, k + 1)) * 0.25; \
        }                                                                                               \
        if (z3) {                                                                                       \
            rZ = (JF(2, i + 1, j, k + 1) + JF(2, i, j, k + 1) + JF(2, i, j + 1, k + 1) + JF(2, i + 1, j + 1, k + 1)) * 0.25; \
            lZ = (JF(2, i + 1, j, k) + JF(2, i, j, k) + JF(2, i, j + 1, k) + JF(2, i + 1, j + 1, k)) * 0.25; \
        }                                                                                               \
        div = ((rX - lX) / g->dx) + ((rY - lY) / g->dy) + ((rZ - lZ) / g->dz);                         \
    }

/* The node moments at a conductor wall after the particle deposits
 * (momentum_collecting.cpp:496-505): J-hat and mu vanish on the wall node. */
void orc_wall_node_moments(const orc_grid* g, double* J, double* mu) {
    if (!g->wall_x) return;
    const long N = NC(g);
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j) {
            const long c = IX(g, 0, j, k);
            for (int d = 0; d < 3; ++d) J[d * N + c] = 0;
            for (int d = 0; d < 9; ++d) mu[d * N + c] = 0;
        }
}

/* updateElectroMagneticParameters after the deposits
 * (momentum_collecting.cpp:590-663): fold Pi, J-hat -= eta dt div(Pi) at
 * every node, rho-hat -= theta dt div(J-hat) at every cell.  Writes J-hat on
 * the periodic nodes and rho_ext, rho-hat with one low ghost layer per axis
 * ((n+1) cells, index 0 = the cell left of cell 0), which is what the right
 * part's gradient reads (fields.cpp:3229-3259 at node 0 uses cell -1). */
void orc_implicit_moments_finish(const orc_grid* g, double* J, const double* rho, double* Pi,
                                 double* rho_ext) {
    const long N = NC(g);
    const int y3 = g->ny > 1, z3 = g->nz > 1;
    const int ex = g->nx > 1 ? g->nx + 1 : 1, ey = g->ny > 1 ? g->ny + 1 : 1, ez = g->nz > 1 ? g->nz + 1 : 1;
    const int single = (g->nx == 1 || !y3 || !z3);   /* div(Pi) vanishes, fields.cpp:3159-3167 */
    if (!g->pressure_compat) {
        double* dJ = (double*)calloc((size_t)(3 * N), sizeof(double));
#define PT(a, b, ii, jj, kk) Pi[(3 * (a) + (b)) * N + IX(g, ii, jj, kk)]
        if (!single)
            for (int k = 0; k < g->nz; ++k)
                for (int j = 0; j < g->ny; ++j)
                    for (int i = 0; i < g->nx; ++i) {
                        double out[3];
                        DIV_PI_BODY(PT, i, j, k, out)
                        for (int d = 0; d < 3; ++d) dJ[d * N + IX(g, i, j, k)] = out[d];
                    }
#undef PT
        for (long c = 0; c < 3 * N; ++c) J[c] = J[c] - dJ[c] * g->eta * g->dt;
        free(dJ);
        if (g->wall_x)   /* J-hat at the wall node (momentum_collecting.cpp:638-646) */
            for (int k = 0; k < g->nz; ++k)
                for (int j = 0; j < g->ny; ++j)
                    for (int d = 0; d < 3; ++d) J[d * N + IX(g, 0, j, k)] = 0;
#define JF(d, ii, jj, kk) J[(d) * N + IX(g, ii, jj, kk)]
        for (int k = -1; k < ez - 1; ++k)
            for (int j = -1; j < ey - 1; ++j)
                for (int i = -1; i < ex - 1; ++i) {
                    int ii = g->nx > 1 ? i : 0, jj = g->ny > 1 ? j : 0, kk = g->nz > 1 ? k : 0;
                    double div;
                    DIV_J_BODY(JF, ii, jj, kk, div)
                    long e = ((long)(kk + (g->nz > 1)) * ey + (jj + (g->ny > 1))) * ex + (ii + (g->nx > 1));
                    rho_ext[e] = rho[IX(g, ii, jj, kk)] - g->dt * g->theta * div;
                }
#undef JF
        return;
    }
    /* reference ghosted layout */
    gaxis ax = mk_axis(g->nx), ay = mk_axis(g->ny), az = mk_axis(g->nz);
    pi_fold_reference(g, Pi);
    const long PN = (long)ax.ce * ay.ce * az.ce;
    const long JN = (long)ax.ne * ay.ne * az.ne;
    double* Jg = (double*)malloc(sizeof(double) * 3 * (size_t)JN);
#define PT(a, b, ii, jj, kk) Pi[(3 * (a) + (b)) * PN + ((long)gclamp(&az, kk) * ay.ce + gclamp(&ay, jj)) * ax.ce + gclamp(&ax, ii)]
#define JG(d, ii, jj, kk) Jg[(d) * JN + ((long)gclamp(&az, kk) * ay.ne + gclamp(&ay, jj)) * ax.ne + gclamp(&ax, ii)]
    for (int k = 0; k < az.ne; ++k)
        for (int j = 0; j < ay.ne; ++j)
            for (int i = 0; i < ax.ne; ++i) {
                long src = IX(g, gphys(&ax, i), gphys(&ay, j), gphys(&az, k));
                double out[3] = {0, 0, 0};
                int edge = (i == 0 || i == ax.ne - 1 || j == 0 || j == ay.ne - 1 || k == 0 || k == az.ne - 1);
                if (!single && !edge) { DIV_PI_BODY(PT, i, j, k, out) }
                for (int d = 0; d < 3; ++d) JG(d, i, j, k) = J[d * N + src] - out[d] * g->eta * g->dt;
                if (g->wall_x && i <= ax.g)   /* the wall node and the ghosts left of it */
                    for (int d = 0; d < 3; ++d) JG(d, i, j, k) = 0;
            }
    for (int k = 0; k < ez; ++k)
        for (int j = 0; j < ey; ++j)
            for (int i = 0; i < ex; ++i) {
                /* ext index 0 is reference cell 1; ext c+1 is reference c+2 */
                int ri = g->nx > 1 ? i + 1 : 0, rj = g->ny > 1 ? j + 1 : 0, rk = g->nz > 1 ? k + 1 : 0;
                double div;
                DIV_J_BODY(JG, ri, rj, rk, div)
                long src = IX(g, gphys(&ax, ri), gphys(&ay, rj), gphys(&az, rk));
                rho_ext[((long)k * ey + j) * ex + i] = rho[src] - g->dt * g->theta * div;
            }
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i)
                for (int d = 0; d < 3; ++d)
                    J[d * N + IX(g, i, j, k)] = JG(d, i + ax.g, j + ay.g, k + az.g);
#undef PT
#undef JG
    free(Jg);
}

/* createInternalEquation right part (fields.cpp:2635-2658) with evaluateRotB
 * (fields.cpp:2799-2860) and evaluateGradDensity (fields.cpp:3229-3259):
 * rhs = E + (c' rot B - 4 pi J) theta dt - grad(rho) c'^2 theta^2 dt^2 4 pi.
 * rho_ext is rho-hat with one low ghost layer (orc_implicit_moments_finish). */
void orc_maxwell_rhs(const orc_grid* g, const double* E, const double* B,
                     const double* J, const double* rho_ext, double* rhs) {
    const long N = NC(g);
    const int y3 = g->ny > 1, z3 = g->nz > 1;
    const double cf = g->cfix, cf2 = g->cfix * g->cfix;
    const double td = g->theta * g->dt;
    const int ex = g->nx > 1 ? g->nx + 1 : 1, ey = g->ny > 1 ? g->ny + 1 : 1;
#define BF(d, ii, jj, kk) B[(d) * N + IX(g, ii, jj, kk)]
#define RH(ii, jj, kk) rho_ext[((long)(g->nz > 1 ? (kk) + 1 : 0) * ey + (g->ny > 1 ? (jj) + 1 : 0)) * ex + (g->nx > 1 ? (ii) + 1 : 0)]
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                int pi_ = i - 1, pj = j - 1, pk = k - 1;
                double BrX[3], BlX[3], BrY[3], BlY[3], BrZ[3], BlZ[3];
                for (int d = 0; d < 3; ++d) {
                    BrX[d] = (BF(d, i, j, k) + BF(d, i, pj, k) + BF(d, i, j, pk) + BF(d, i, pj, pk)) / 4.0;
                    BlX[d] = (BF(d, pi_, j, k) + BF(d, pi_, pj, k) + BF(d, pi_, j, pk) + BF(d, pi_, pj, pk)) / 4.0;
                    BrY[d] = (BF(d, i, j, k) + BF(d, pi_, j, k) + BF(d, i, j, pk) + BF(d, pi_, j, pk)) / 4.0;
                    BlY[d] = (BF(d, i, pj, k) + BF(d, pi_, pj, k) + BF(d, i, pj, pk) + BF(d, pi_, pj, pk)) / 4.0;
                    BrZ[d] = (BF(d, i, j, k) + BF(d, pi_, j, k) + BF(d, i, pj, k) + BF(d, pi_, pj, k)) / 4.0;
                    BlZ[d] = (BF(d, i, j, pk) + BF(d, pi_, j, pk) + BF(d, i, pj, pk) + BF(d, pi_, pj, pk)) / 4.0;
                    if (!y3) { BrY[d] = 0; BlY[d] = 0; }
                    if (!z3) { BrZ[d] = 0; BlZ[d] = 0; }
                }
                double rot[3];
                rot[0] = (BrY[2] - BlY[2]) / g->dy - (BrZ[1] - BlZ[1]) / g->dz;
                rot[1] = (BrZ[0] - BlZ[0]) / g->dz - (BrX[2] - BlX[2]) / g->dx;
                rot[2] = (BrX[1] - BlX[1]) / g->dx - (BrY[0] - BlY[0]) / g->dy;
                double dRX = (RH(i, j, k) + RH(i, pj, k) + RH(i, j, pk) + RH(i, pj, pk)) * 0.25;
                double dLX = (RH(pi_, j, k) + RH(pi_, pj, k) + RH(pi_, j, pk) + RH(pi_, pj, pk)) * 0.25;
                double dRY = (RH(i, j, k) + RH(pi_, j, k) + RH(i, j, pk) + RH(pi_, j, pk)) * 0.25;
                double dLY = (RH(i, pj, k) + RH(pi_, pj, k) + RH(i, pj, pk) + RH(pi_, pj, pk)) * 0.25;
                double dRZ = (RH(i, j, k) + RH(i, pj, k) + RH(pi_, j, k) + RH(pi_, pj, k)) * 0.25;
                double dLZ = (RH(i, j, pk) + RH(i, pj, pk) + RH(pi_, j, pk) + RH(pi_, pj, pk)) * 0.25;
                double grad[3] = {(dRX - dLX) / g->dx, (dRY - dLY) / g->dy, (dRZ - dLZ) / g->dz};
                long c = IX(g, i, j, k);
                for (int d = 0; d < 3; ++d)
                    rhs[d * N + c] = E[d * N + c] + (rot[d] * cf - (J[d * N + c] * 4 * PI_D)) * td
                                   - (grad[d] * cf2 * g->theta * g->theta * g->dt * g->dt * 4 * PI_D);
            }
    if (g->wall_x) {
        /* right parts of the boundary rows (wall_rows_apply): the wall's
         * Gauss row -pi (four cells of rho-hat around the node, fields.cpp:
         * 759-760), E_y = E_z = 0; the open boundary's constant field
         * (ConstantBoundaryFieldEvaluator, initializeFluxFromRight,
         * initialization.cpp:5207) */
        for (int k = 0; k < g->nz; ++k)
            for (int j = 0; j < g->ny; ++j) {
                const long c0 = IX(g, 0, j, k);
                rhs[c0] = -PI_D * (RH(0, j, k) + RH(0, j - 1, k) + RH(0, j, k - 1) + RH(0, j - 1, k - 1));
                rhs[N + c0] = 0;
                rhs[2 * N + c0] = 0;
                for (int i = g->nx - 2; i < g->nx; ++i) {
                    const long c = IX(g, i, j, k);
                    for (int d = 0; d < 3; ++d) rhs[d * N + c] = g->e_right[d];
                }
            }
    }
#undef BF
#undef RH
}

/* Rows of the Maxwell system at the x boundaries of a conductor-wall box
 * (evaluateMaxwellEquationMatrix, fields.cpp:519-548, one rank).  Storage
 * column 0 is the wall node (reference index 2): createSuperConductorLeft-
 * Equation (fields.cpp:690-765), E_x(0) - E_x(1) for 3-D boxes and
 * E_y = E_z = 0; columns nx - 2 and nx - 1 are the open boundary node and
 * the ghost node beyond it (reference xnumber + 2 and + 3): identity rows
 * of createFreeRightEquation (fields.cpp:767-781).  The physical nodes are
 * 0 .. nx - 2 and the cells 0 .. nx - 3; cell nx - 2 is the ghost cell
 * beyond the open boundary and cell nx - 1 the ghost cell left of the wall
 * (reference index 1), so the periodic index wrap of every stencil reaches
 * the reference's ghost values. */
static void wall_rows_apply(const orc_grid* g, const double* x, double* y) {
    const long N = NC(g);
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j) {
            const long c0 = IX(g, 0, j, k), c1 = IX(g, 1, j, k);
            y[c0] = x[c0] * 1.0 + x[c1] * -1.0;
            y[N + c0] = x[N + c0];
            y[2 * N + c0] = x[2 * N + c0];
            for (int i = g->nx - 2; i < g->nx; ++i) {
                const long c = IX(g, i, j, k);
                for (int d = 0; d < 3; ++d) y[d * N + c] = x[d * N + c];
            }
        }
}

/* Matrix-free restatement of the Maxwell operator rows assembled by
 * createInternalEquationX/Y/Z (fields.cpp:1396-1509, 1961-2073, 2521-2633)
 * with K = (theta dt c')^2 (fields.cpp:888); multiplySpecialMatrixVector
 * (specialmath.cpp:202-252) sums the row entries in assembly order, which is
 * the order used here.  mu is node-centred, row-major 3x3. */
void orc_maxwell_apply(const orc_grid* g, const double* mu, const double* x, double* y) {
    const long N = NC(g);
    const double K = (g->theta * g->dt) * (g->theta * g->dt) * (g->cfix * g->cfix);
    const double d[3] = {g->dx, g->dy, g->dz};
    const double d2[3] = {g->dx * g->dx, g->dy * g->dy, g->dz * g->dz};
    const int has[3] = {g->nx > 1, g->ny > 1, g->nz > 1};
#define MU(a, b, id) mu[(3 * (a) + (b)) * N + (id)]
#define XV(c, id) x[(c) * N + (id)]
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                const long c0 = IX(g, i, j, k);
                const int pos[3] = {i, j, k};
                for (int a = 0; a < 3; ++a) {
                    int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
                    /* the two other axes in increasing order, as in the
                     * reference rows (X: y then z; Y: x then z; Z: y then x
                     * for the plain neighbours, see fields.cpp) */
                    double acc = 0.0;
                    /* diagonal */
                    double el = 1.0 - MU(a, a, c0);
                    for (int ax = 0; ax < 3; ++ax) {
                        if (!has[ax]) continue;
                        if (ax == a) el += K * ((2.0 - 2 * MU(a, a, c0)) / d2[ax]);
                        else el += K * 2.0 / d2[ax];
                    }
                    acc += el * XV(a, c0);
                    /* same node, other components (row X: E_y then E_z;
                     * row Y: E_x then E_z; row Z: E_x then E_y) */
                    int oc[2]; if (a == 0) { oc[0] = 1; oc[1] = 2; } else if (a == 1) { oc[0] = 0; oc[1] = 2; } else { oc[0] = 0; oc[1] = 1; }
                    for (int t = 0; t < 2; ++t) {
                        int b = oc[t];
                        double e2 = -MU(a, b, c0);
                        if (has[a]) e2 -= K * 2 * MU(a, b, c0) / d2[a];
                        acc += e2 * XV(b, c0);
                    }
                    /* +-a neighbours */
                    if (has[a]) {
                        for (int sgn = 1; sgn >= -1; sgn -= 2) {
                            int q[3] = {pos[0], pos[1], pos[2]}; q[a] += sgn;
                            long cn = IX(g, q[0], q[1], q[2]);
                            /* component order: row X: 0,1,2; row Y: 1,0,2; row Z: 2,1,0 */
                            int co[3];
                            if (a == 0) { co[0] = 0; co[1] = 1; co[2] = 2; }
                            else if (a == 1) { co[0] = 1; co[1] = 0; co[2] = 2; }
                            else { co[0] = 2; co[1] = 1; co[2] = 0; }
                            for (int t = 0; t < 3; ++t) {
                                int b = co[t];
                                double e3 = (b == a) ? K * (-1.0 + MU(a, a, cn)) / d2[a]
                                                     : K * MU(a, b, cn) / d2[a];
                                acc += e3 * XV(b, cn);
                            }
                        }
                    }
                    /* plain Laplacian neighbours along the other axes, in the
                     * reference's order: X row y,z; Y row x,z; Z row y,x */
                    int oax[2];
                    if (a == 0) { oax[0] = 1; oax[1] = 2; }
                    else if (a == 1) { oax[0] = 0; oax[1] = 2; }
                    else { oax[0] = 1; oax[1] = 0; }
                    for (int t = 0; t < 2; ++t) {
                        int ax = oax[t];
                        if (!has[ax]) continue;
                        double e4 = -K / d2[ax];
                        for (int sgn = 1; sgn >= -1; sgn -= 2) {
                            int q[3] = {pos[0], pos[1], pos[2]}; q[ax] += sgn;
                            acc += e4 * XV(a, IX(g, q[0], q[1], q[2]));
                        }
                    }
                    /* mixed-derivative corners in the (a, ax) planes, in the
                     * reference's plane order: X row xy,xz; Y row xy,yz;
                     * Z row yz,xz.  Corners: (+,+), (-,-), (-,+), (+,-) in
                     * (first axis, second axis) of the reference's naming. */
                    int pl[2][2];  /* [plane][axis pair as written in the reference] */
                    if (a == 0) { pl[0][0] = 0; pl[0][1] = 1; pl[1][0] = 0; pl[1][1] = 2; }
                    else if (a == 1) { pl[0][0] = 0; pl[0][1] = 1; pl[1][0] = 1; pl[1][1] = 2; }
                    else { pl[0][0] = 1; pl[0][1] = 2; pl[1][0] = 0; pl[1][1] = 2; }
                    for (int t = 0; t < 2; ++t) {
                        int A0 = pl[t][0], A1 = pl[t][1];
                        if (!has[A0] || !has[A1]) continue;
                        int other = (A0 == a) ? A1 : A0;   /* mu row index used: the non-a axis */
                        double den = 4 * d[A0] * d[A1];
                        const int sg[4][3] = {{1, 1, 1}, {-1, -1, 1}, {-1, 1, -1}, {1, -1, -1}};
                        for (int cidx = 0; cidx < 4; ++cidx) {
                            int q[3] = {pos[0], pos[1], pos[2]};
                            q[A0] += sg[cidx][0]; q[A1] += sg[cidx][1];
                            long cn = IX(g, q[0], q[1], q[2]);
                            for (int b = 0; b < 3; ++b) {
                                double e5 = K * MU(other, b, cn) / den;
                                if (sg[cidx][2] < 0) e5 = -K * MU(other, b, cn) / den;
                                acc += e5 * XV(b, cn);
                            }
                        }
                    }
                    (void)b1; (void)b2;
                    y[a * N + c0] = acc;
                }
            }
    if (g->wall_x) wall_rows_apply(g, x, y);
#undef MU
#undef XV
}

static double dotv(long n, const double* a, const double* b) {
    double s = 0.0;
    for (long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* generalizedMinimalResidualMethod (specialmath.cpp:367-671) with
 * arnoldiIterations (specialmath.cpp:254-365): unrestarted GMRES from x = 0
 * on the normalised right part, modified Gram-Schmidt, Givens QR kept as a
 * dense Q, stop when |beta Q[n-1][0]| / |r| <= max(tol / (3N), 1e-15) or
 * n >= min(maxIter, 3N + 3).  Returns the number of Krylov vectors used. */
int orc_gmres(const orc_grid* g, const double* mu, const double* rhs, double* x,
              double* rel_err_out) {
    const long N = NC(g);
    const long L = 3 * N;
    const int maxIter = g->gmres_max_iter;
    double norm = sqrt(dotv(L, rhs, rhs));
    if (norm == 0) { memset(x, 0, sizeof(double) * L); if (rel_err_out) *rel_err_out = 0; return 0; }
    int cap = maxIter + 2;
    double** V = (double**)calloc((size_t)cap, sizeof(double*));
    V[0] = (double*)malloc(sizeof(double) * L);
    for (long c = 0; c < L; ++c) V[0][c] = rhs[c] / norm;
    double normR = sqrt(dotv(L, V[0], V[0]));
    /* matrixDimension of the reference: 3 x the physical cells */
    long dim = g->wall_x ? 3L * (g->nx - 2) * g->ny * g->nz : L;
    double tolRel = g->gmres_tol / (double)dim;
    if (tolRel < 1e-15) tolRel = 1e-15;
    /* H[i][j], Q[i][j], R[i][j] dense, (cap x cap) */
    double* H = (double*)calloc((size_t)cap * cap, sizeof(double));
    double* Q = (double*)calloc((size_t)cap * cap, sizeof(double));
    double* Qo = (double*)calloc((size_t)cap * cap, sizeof(double));
    double* R = (double*)calloc((size_t)cap * cap, sizeof(double));
    double* y = (double*)calloc((size_t)cap, sizeof(double));
#define M2(A, i, j) A[(long)(i) * cap + (j)]
    int n = 2;
    double beta = 1.0, relErr = 1.0;
    long lim = maxIter < dim + 3 ? maxIter : dim + 3;
    while (relErr > tolRel && n < lim) {
        /* Arnoldi step for column n-2 */
        V[n - 1] = (double*)malloc(sizeof(double) * L);
        orc_maxwell_apply(g, mu, V[n - 2], V[n - 1]);
        for (int m = 0; m < n - 1; ++m) {
            double h = dotv(L, V[m], V[n - 1]);
            M2(H, m, n - 2) = h;
            for (long c = 0; c < L; ++c) V[n - 1][c] -= h * V[m][c];
        }
        double hn = sqrt(dotv(L, V[n - 1], V[n - 1]));
        M2(H, n - 1, n - 2) = hn;
        if (hn > 0) { for (long c = 0; c < L; ++c) V[n - 1][c] /= hn; }
        else { for (long c = 0; c < L; ++c) V[n - 1][c] = 0; }
        /* Givens update (specialmath.cpp:499-578) */
        if (n == 2) {
            double rho = M2(H, 0, 0), sigma = M2(H, 1, 0);
            double mod = sqrt(rho * rho + sigma * sigma);
            double cs = rho / mod, sn = sigma / mod;
            M2(Q, 0, 0) = cs; M2(Q, 0, 1) = sn; M2(Q, 1, 0) = -sn; M2(Q, 1, 1) = cs;
            M2(R, 0, 0) = mod; M2(R, 1, 0) = 0;
        } else {
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) M2(Qo, i, j) = M2(Q, i, j);
            for (int j = 0; j < n - 2; ++j) M2(R, n - 1, j) = 0;
            for (int i = 0; i < n - 1; ++i) M2(Q, i, n - 1) = 0;
            for (int j = 0; j < n - 1; ++j) M2(Q, n - 1, j) = 0;
            M2(Q, n - 1, n - 1) = 1;
            for (int i = 0; i < n; ++i) {
                double s = 0;
                for (int j = 0; j < n; ++j) s += M2(Q, i, j) * M2(H, j, n - 2);
                M2(R, i, n - 2) = s;
            }
            double rho = M2(R, n - 2, n - 2), sigma = M2(R, n - 1, n - 2);
            double mod = sqrt(rho * rho + sigma * sigma);
            double cs = rho / mod, sn = sigma / mod;
            M2(R, n - 2, n - 2) = mod; M2(R, n - 1, n - 2) = 0;
            for (int j = 0; j < n - 1; ++j) {
                M2(Q, n - 2, j) = cs * M2(Qo, n - 2, j);
                M2(Q, n - 1, j) = -sn * M2(Qo, n - 2, j);
            }
            M2(Q, n - 2, n - 1) = sn; M2(Q, n - 1, n - 1) = cs;
        }
        /* back substitution (specialmath.cpp:580-593) */
        for (int i = n - 2; i >= 0; --i) {
            y[i] = beta * M2(Q, i, 0);
            for (int j = n - 2; j > i; --j) y[i] -= M2(R, i, j) * y[j];
            if (M2(R, i, i) > 0) y[i] /= M2(R, i, i); else y[i] = 0;
        }
        relErr = fabs(beta * M2(Q, n - 1, 0)) / normR;
        n++;
    }
    n = n - 1;
    for (long c = 0; c < L; ++c) {
        double s = 0;
        for (int m = 0; m < n - 1; ++m) s += V[m][c] * y[m] * norm;
        x[c] = s;
    }
#undef M2
    for (int i = 0; i < cap; ++i) free(V[i]);
    free(V); free(H); free(Q); free(Qo); free(R); free(y);
    if (rel_err_out) *rel_err_out = relErr;
    return n - 1;
}

/* evaluateElectricField (fields.cpp:326-339): E^{n+1} = (Etheta - (1-theta)E^n)/theta,
 * and evaluateMagneticField (fields.cpp:2717-2738) with evaluateRotEgeneral
 * (fields.cpp:2862-2953): B^{n+1} = B^n - c' dt rot(Etheta) at cells. */
void orc_field_update(const orc_grid* g, const double* Et, const double* E,
                      const double* B, double* Enew, double* Bnew) {
    const long N = NC(g);
    const int y3 = g->ny > 1, z3 = g->nz > 1;
    for (long c = 0; c < 3 * N; ++c) Enew[c] = (Et[c] - E[c] * (1 - g->theta)) / g->theta;
#define EF(d, ii, jj, kk) Et[(d) * N + IX(g, ii, jj, kk)]
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                double rX[3], lX[3], rY[3], lY[3], rZ[3], lZ[3];
                for (int d = 0; d < 3; ++d) {
                    rX[d] = (EF(d, i + 1, j, k) + EF(d, i + 1, j + 1, k) + EF(d, i + 1, j, k + 1) + EF(d, i + 1, j + 1, k + 1)) / 4.0;
                    lX[d] = (EF(d, i, j, k) + EF(d, i, j + 1, k) + EF(d, i, j, k + 1) + EF(d, i, j + 1, k + 1)) / 4.0;
                    rY[d] = (EF(d, i, j + 1, k) + EF(d, i + 1, j + 1, k) + EF(d, i, j + 1, k + 1) + EF(d, i + 1, j + 1, k + 1)) / 4.0;
                    lY[d] = (EF(d, i, j, k) + EF(d, i + 1, j, k) + EF(d, i, j, k + 1) + EF(d, i + 1, j, k + 1)) / 4.0;
                    rZ[d] = (EF(d, i, j, k + 1) + EF(d, i + 1, j, k + 1) + EF(d, i, j + 1, k + 1) + EF(d, i + 1, j + 1, k + 1)) / 4.0;
                    lZ[d] = (EF(d, i, j, k) + EF(d, i + 1, j, k) + EF(d, i, j + 1, k) + EF(d, i + 1, j + 1, k)) / 4.0;
                    if (!y3) { rY[d] = 0; lY[d] = 0; }
                    if (!z3) { rZ[d] = 0; lZ[d] = 0; }
                }
                double rot[3];
                rot[0] = (rY[2] - lY[2]) / g->dy - (rZ[1] - lZ[1]) / g->dz;
                rot[1] = (rZ[0] - lZ[0]) / g->dz - (rX[2] - lX[2]) / g->dx;
                rot[2] = (rX[1] - lX[1]) / g->dx - (rY[0] - lY[0]) / g->dy;
                long c = IX(g, i, j, k);
                for (int d = 0; d < 3; ++d) Bnew[d * N + c] = B[d * N + c] - rot[d] * (g->cfix * g->dt);
            }
    if (g->wall_x) {
        /* the ghost cell beyond the open boundary takes the boundary field,
         * the ghost cell left of the wall the first cell's new field
         * (evaluateMagneticField, fields.cpp:2738-2756) */
        for (int k = 0; k < g->nz; ++k)
            for (int j = 0; j < g->ny; ++j) {
                const long cr = IX(g, g->nx - 2, j, k), cl = IX(g, g->nx - 1, j, k), c0 = IX(g, 0, j, k);
                for (int d = 0; d < 3; ++d) {
                    Bnew[d * N + cr] = g->b_right[d];
                    Bnew[d * N + cl] = Bnew[d * N + c0];
                }
            }
    }
#undef EF
}

/* Particle::setMomentumByV (particle.cpp:337-364): p = m v below
 * v^2 < relativisticPrecision = 1e-4 (constants.h:39), m gamma(v) v above. */
static inline void momentum_by_v(const double v[3], double m, double p[3]) {
    const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (v2 < 1e-4) {
        for (int d = 0; d < 3; ++d) p[d] = v[d] * m;
        return;
    }
    const double gam = 1 / sqrt(1 - v2);
    for (int d = 0; d < 3; ++d) p[d] = v[d] * (m * gam);
}

/* x in length units from the origin of our storage -> cell and offset. */
static inline void set_x(double x, double idx, int* c, double* u) {
    const double a = x * idx;
    const double f = floor(a);
    *c = (int)f;
    *u = a - f;
    if (*u >= 1.0) { *u -= 1.0; *c += 1; }
}

/* The reflection of moveParticle at the conductor wall (mover.cpp:247-260
 * after the predictor, mover.cpp:312-330 inside the Picard loop), wall at
 * x = 0: the trial position x = x^n + eta dt vbar crossed the wall; the
 * particle is mirrored with the rest of the step, |vbar_x| (1 - eta) dt,
 * carries on in y and z by vbar (1 - eta) dt, and leaves with the
 * predictor's velocity, its x component made positive. */
static void wall_reflect(const orc_grid* g, const double id[3], const int nn[3], int ci[3], double u0[3],
                         const double xtrial, const double mv[3], const double vnew[3], double m, double pout[3]) {
    const double redt = (1 - g->eta) * g->dt;
    const double edt = g->eta * g->dt;
    set_x(-xtrial + fabs(mv[0] * redt), id[0], &ci[0], &u0[0]);
    for (int d = 1; d < 3; ++d) {
        advance_axis(&u0[d], &ci[d], (mv[d] * edt) * id[d], nn[d]);
        advance_axis(&u0[d], &ci[d], (mv[d] * redt) * id[d], nn[d]);
    }
    const double vr[3] = {fabs(vnew[0]), vnew[1], vnew[2]};
    momentum_by_v(vr, m, pout);
}

/* moveParticle (mover.cpp:194-491): predictor, then up to 3 Picard
 * iterations re-gathering E^{n+theta} (nodes) and B^n (cells) at
 * x^n + eta dt vbar, then x^{n+1} = x^n + dt vbar.  alpha is recomputed
 * from E^n, B^n at x^n, exactly as evaluateParticlesRotationTensor
 * (mover.cpp:810-841) stored it.  With a conductor wall (g->wall_x) a trial
 * position left of the wall reflects the particle there and then
 * (mover.cpp:247-260, 312-330); a final position left of it is mirrored
 * with p_x reversed (mover.cpp:435-445); a final position right of the open
 * boundary x = (nx - 2) dx marks the particle escaped (cell = -1,
 * mover.cpp:447-458), to be erased after the step
 * (eraseEscapedPaticles, mover.cpp:167-192).  Escaped particles are
 * skipped. */
void orc_implicit_push(const orc_grid* g, orc_particles* p, const double* E,
                       const double* B, const double* Et) {
    const double beta = 0.5 * p->q * g->dt / p->m;
    const double edt = g->eta * g->dt;
    const double qdt = p->q * g->dt;
    const double id[3] = {1.0 / g->dx, 1.0 / g->dy, 1.0 / g->dz};
    const int nn[3] = {g->nx, g->ny, g->nz};
    const double xright = (g->nx - 2) * g->dx;
    for (long n = 0; n < p->n; ++n) {
        if (p->cell[n] < 0) continue;
        int ci[3]; decode(g, p->cell[n], &ci[0], &ci[1], &ci[2]);
        double u0[3] = {p->ox[n], p->oy[n], p->oz[n]};
        const double xold = (ci[0] + u0[0]) * g->dx;
        double mom0[3] = {p->px[n], p->py[n], p->pz[n]};
        double gam = gamma_of(mom0, p->m);
        double v[3]; velocity_of(mom0, p->m, v);
        double e0[3], b0[3], al[9];
        orc_gather_node(g, p->cell[n], u0[0], u0[1], u0[2], E, e0);
        orc_gather_cell(g, p->cell[n], u0[0], u0[1], u0[2], B, b0);
        orc_alpha(beta, v, gam, e0, b0, al);
        double e[3], b[3];
        orc_gather_node(g, p->cell[n], u0[0], u0[1], u0[2], Et, e);
        orc_gather_cell(g, p->cell[n], u0[0], u0[1], u0[2], B, b);
        /* predictor (mover.cpp:236-245) */
        double vxb[3]; cross(v, b, vxb);
        double pnew[3];
        for (int d = 0; d < 3; ++d) pnew[d] = mom0[d] + (e[d] + vxb[d]) * qdt;
        double vnew[3]; evaluate_velocity(pnew, p->m, vnew);
        double mv[3];
        for (int d = 0; d < 3; ++d) mv[d] = v[d] * (1 - g->eta) + vnew[d] * g->eta;
        int reflected = 0;
        if (g->wall_x && xold + mv[0] * edt < 0) {
            wall_reflect(g, id, nn, ci, u0, xold + mv[0] * edt, mv, vnew, p->m, pnew);
            reflected = 1;
        }
        if (!reflected) {
            double disp[3];   /* current trial displacement from x^n, length units */
            for (int d = 0; d < 3; ++d) disp[d] = mv[d] * edt;
            /* velocityHat = (alpha * gamma) * v (mover.cpp:276) */
            double vh[3];
            for (int a = 0; a < 3; ++a)
                vh[a] = (al[3 * a] * gam) * v[0] + (al[3 * a + 1] * gam) * v[1] + (al[3 * a + 2] * gam) * v[2];
            double momNorm = sqrt(mom0[0] * mom0[0] + mom0[1] * mom0[1] + mom0[2] * mom0[2]);
            double err = sqrt((mom0[0] - pnew[0]) * (mom0[0] - pnew[0]) + (mom0[1] - pnew[1]) * (mom0[1] - pnew[1]) +
                              (mom0[2] - pnew[2]) * (mom0[2] - pnew[2]));
            double cerr = g->dx;
            double prevDisp[3] = {disp[0], disp[1], disp[2]};
            double newDisp[3] = {disp[0], disp[1], disp[2]};
            int it = 0;
            while (err > 1e-14 * momNorm && cerr > 1e-8 * g->dx && it < 3) {
                ++it;
                double prevMom[3] = {pnew[0], pnew[1], pnew[2]};
                for (int d = 0; d < 3; ++d) prevDisp[d] = newDisp[d];
                double re[3];
                for (int a = 0; a < 3; ++a) re[a] = al[3 * a] * e[0] + al[3 * a + 1] * e[1] + al[3 * a + 2] * e[2];
                for (int d = 0; d < 3; ++d) mv[d] = vh[d] + re[d] * beta;
                for (int d = 0; d < 3; ++d) newDisp[d] = mv[d] * edt;
                if (g->wall_x && xold + newDisp[0] < 0) {
                    wall_reflect(g, id, nn, ci, u0, xold + newDisp[0], mv, vnew, p->m, pnew);
                    reflected = 1;
                    break;
                }
                /* trial position and re-gather */
                int tc[3]; double tu[3];
                for (int d = 0; d < 3; ++d) {
                    tc[d] = ci[d]; tu[d] = u0[d];
                    advance_axis(&tu[d], &tc[d], newDisp[d] * id[d], nn[d]);
                }
                int tcell = (int)IX(g, tc[0], tc[1], tc[2]);
                orc_gather_node(g, tcell, tu[0], tu[1], tu[2], Et, e);
                orc_gather_cell(g, tcell, tu[0], tu[1], tu[2], B, b);
                double mvxb[3]; cross(mv, b, mvxb);
                for (int d = 0; d < 3; ++d) pnew[d] = mom0[d] + (e[d] + mvxb[d]) * qdt;
                err = sqrt((prevMom[0] - pnew[0]) * (prevMom[0] - pnew[0]) + (prevMom[1] - pnew[1]) * (prevMom[1] - pnew[1]) +
                           (prevMom[2] - pnew[2]) * (prevMom[2] - pnew[2]));
                cerr = sqrt((prevDisp[0] - newDisp[0]) * (prevDisp[0] - newDisp[0]) + (prevDisp[1] - newDisp[1]) * (prevDisp[1] - newDisp[1]) +
                            (prevDisp[2] - newDisp[2]) * (prevDisp[2] - newDisp[2]));
            }
            if (!reflected) {
                if (g->wall_x) {
                    const double xn = xold + mv[0] * g->dt;
                    if (xn < 0) {            /* mirrored, p_x reversed (reflectMomentumX) */
                        set_x(-xn, id[0], &ci[0], &u0[0]);
                        pnew[0] = -pnew[0];
                    } else if (xn > xright) {
                        p->cell[n] = -1;     /* escaped through the open boundary */
                        continue;
                    } else {
                        advance_axis(&u0[0], &ci[0], (mv[0] * g->dt) * id[0], nn[0]);
                    }
                    for (int d = 1; d < 3; ++d) advance_axis(&u0[d], &ci[d], (mv[d] * g->dt) * id[d], nn[d]);
                } else {
                    for (int d = 0; d < 3; ++d) advance_axis(&u0[d], &ci[d], (mv[d] * g->dt) * id[d], nn[d]);
                }
            }
        }
        p->px[n] = pnew[0]; p->py[n] = pnew[1]; p->pz[n] = pnew[2];
        p->ox[n] = u0[0]; p->oy[n] = u0[1]; p->oz[n] = u0[2];
        p->cell[n] = (int)IX(g, ci[0], ci[1], ci[2]);
    }
}

/* smoothChargeDensityHat, smoothFlux, smoothMatrixNodeParameter
 * (smoothing.cpp:100-103, 251-412) on a periodic box: rho-hat (with its low
 * ghost layer refilled from the smoothed cells), J-hat and mu. */
void orc_smooth_moments(const orc_grid* g, double* J, double* mu, double* rho_ext) {
    const long N = NC(g);
    orc_smooth(g, J, 3);
    orc_smooth(g, mu, 9);
    const int ex = g->nx > 1 ? g->nx + 1 : 1, ey = g->ny > 1 ? g->ny + 1 : 1, ez = g->nz > 1 ? g->nz + 1 : 1;
    double* r = (double*)malloc(sizeof(double) * (size_t)N);
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                const int ri = g->nx > 1 ? i + 1 : 0, rj = g->ny > 1 ? j + 1 : 0, rk = g->nz > 1 ? k + 1 : 0;
                r[IX(g, i, j, k)] = rho_ext[((long)rk * ey + rj) * ex + ri];
            }
    orc_smooth(g, r, 1);
    for (int rk = 0; rk < ez; ++rk)
        for (int rj = 0; rj < ey; ++rj)
            for (int ri = 0; ri < ex; ++ri) {
                const int i = g->nx > 1 ? wrapi(ri - 1, g->nx) : 0;
                const int j = g->ny > 1 ? wrapi(rj - 1, g->ny) : 0;
                const int k = g->nz > 1 ? wrapi(rk - 1, g->nz) : 0;
                rho_ext[((long)rk * ey + rj) * ex + ri] = r[IX(g, i, j, k)];
            }
    free(r);
}

long orc_implicit_work_size(const orc_grid* g) {
    return NC(g) * (3 + 9 + 1 + 3 + 3 + 3 + 3) + orc_pi_size(g) + orc_rho_ext_size(g);
}

/* One implicit step, the IMPLICIT branch of Simulation::simulate
 * (simulation.cpp:205-259; smoothingCount passes over rho-hat, J-hat and mu
 * before the field solve, simulation.cpp:213-217), followed by the
 * particle move and updateFields (fields.cpp:422-439).  work must hold
 * orc_implicit_work_size(g) doubles.  Returns the GMRES iteration count. */
int orc_implicit_step(const orc_grid* g, orc_particles* sp, int nspecies,
                      double* E, double* B, double* work) {
    const long N = NC(g);
    double* J = work;
    double* mu = J + 3 * N;
    double* rho = mu + 9 * N;
    double* rhs = rho + N;
    double* Et = rhs + 3 * N;
    double* En = Et + 3 * N;
    double* Bn = En + 3 * N;
    double* Pi = Bn + 3 * N;
    double* rho_ext = Pi + orc_pi_size(g);
    memset(work, 0, sizeof(double) * (size_t)orc_implicit_work_size(g));
    for (int s = 0; s < nspecies; ++s) orc_implicit_deposit(g, &sp[s], E, B, J, mu, rho, Pi);
    orc_wall_node_moments(g, J, mu);
    orc_implicit_moments_finish(g, J, rho, Pi, rho_ext);
    if (!g->pressure_compat)
        for (int q = 0; q < g->smoothing_count; ++q) orc_smooth_moments(g, J, mu, rho_ext);
    orc_maxwell_rhs(g, E, B, J, rho_ext, rhs);
    double rel;
    int it = orc_gmres(g, mu, rhs, Et, &rel);
    orc_field_update(g, Et, E, B, En, Bn);
    for (int s = 0; s < nspecies; ++s) orc_implicit_push(g, &sp[s], E, B, Et);
    memcpy(E, En, sizeof(double) * 3 * N);
    memcpy(B, Bn, sizeof(double) * 3 * N);
    return it;
}

/* updateEnergy (simulation.cpp:1506-1600) in normalised units:
 * out = {sum w (gamma-1) m, sum E^2 V / 8pi, sum B^2 V / 8pi, sum w px, sum w py, sum w pz}.
 * E and B are taken at the stored grid points, as the reference does. */
void orc_energy(const orc_grid* g, const orc_particles* sp, int nspecies,
                const double* E, const double* B, double out[6]) {
    const long N = NC(g);
    const double vol = g->dx * g->dy * g->dz;
    double pe = 0, ee = 0, be = 0, mx = 0, my = 0, mz = 0;
    for (long c = 0; c < N; ++c) {
        double e2 = E[c] * E[c] + E[N + c] * E[N + c] + E[2 * N + c] * E[2 * N + c];
        double b2 = B[c] * B[c] + B[N + c] * B[N + c] + B[2 * N + c] * B[2 * N + c];
        ee += e2 * vol / (8 * PI_D);
        be += b2 * vol / (8 * PI_D);
    }
    for (int s = 0; s < nspecies; ++s) {
        const orc_particles* p = &sp[s];
        for (long n = 0; n < p->n; ++n) {
            double mom[3] = {p->px[n], p->py[n], p->pz[n]};
            pe += (gamma_of(mom, p->m) - 1) * p->m * p->w;
            mx += mom[0] * p->w; my += mom[1] * p->w; mz += mom[2] * p->w;
        }
    }
    out[0] = pe; out[1] = ee; out[2] = be; out[3] = mx; out[4] = my; out[5] = mz;
}

/* updateDensityParameters (PIC++/momentum_collecting.cpp:760-1020) on a
 * periodic box: per species s the concentration n_s = sum w S / V, the
 * energy density e_s = sum w gamma m S / V (fullEnergy, particle.cpp:398-401)
 * and the bulk velocity u_s = (sum w p S / V) / e_s (0 where e_s = 0), with
 * the cell-centred weights S of the correlation map; the charge density
 * rho = sum_s q_s n_s.  Outputs: conc[s][N], energy[s][N], vel[s][3][N],
 * rho[N]. */
void orc_density_moments(const orc_grid* g, const orc_particles* sp, int nspecies, double* conc, double* energy,
                         double* vel, double* rho) {
    const long N = NC(g);
    const double vol = g->dx * g->dy * g->dz;
    for (long c = 0; c < N; ++c) rho[c] = 0.0;
    for (int s = 0; s < nspecies; ++s) {
        const orc_particles* p = &sp[s];
        double* cs = conc + s * N;
        double* es = energy + s * N;
        double* vs = vel + 3 * s * N;
        for (long c = 0; c < N; ++c) { cs[c] = 0; es[c] = 0; vs[c] = 0; vs[N + c] = 0; vs[2 * N + c] = 0; }
        for (long n = 0; n < p->n; ++n) {
            int i, j, k;
            decode(g, p->cell[n], &i, &j, &k);
            int X[2], Y[2], Z[2];
            double wx[2], wy[2], wz[2];
            cell_w(p->ox[n], i, g->nx, X, wx);
            cell_w(p->oy[n], j, g->ny, Y, wy);
            cell_w(p->oz[n], k, g->nz, Z, wz);
            const double mom[3] = {p->px[n], p->py[n], p->pz[n]};
            const double en = gamma_of(mom, p->m) * p->m;
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b)
                    for (int cc = 0; cc < 2; ++cc) {
                        if ((g->ny == 1 && b) || (g->nz == 1 && cc)) continue;
                        const long id = IX(g, X[a], Y[b], Z[cc]);
                        const double corr = wx[a] * wy[b] * wz[cc] / vol;
                        cs[id] += p->w * corr;
                        es[id] += p->w * en * corr;
                        vs[id] += mom[0] * p->w * corr;
                        vs[N + id] += mom[1] * p->w * corr;
                        vs[2 * N + id] += mom[2] * p->w * corr;
                    }
        }
        if (g->wall_x) {
            /* conductor wall: deposits in the ghost cell left of the wall go
             * to the first cell with p_x reflected (momentum_collecting.cpp
             * 945-960), those beyond the open boundary to the last physical
             * cell; both ghost columns end empty (sumCellParametersX and
             * sumCellVectorParametersX, one rank, momentum_exchange.cpp
             * 968-988, 1351-1361) */
            for (int k = 0; k < g->nz; ++k)
                for (int j = 0; j < g->ny; ++j) {
                    const long gl = IX(g, g->nx - 1, j, k), f = IX(g, 0, j, k);
                    const long gr = IX(g, g->nx - 2, j, k), l = IX(g, g->nx - 3, j, k);
                    cs[f] += cs[gl]; es[f] += es[gl];
                    vs[f] -= vs[gl]; vs[N + f] += vs[N + gl]; vs[2 * N + f] += vs[2 * N + gl];
                    cs[l] += cs[gr]; es[l] += es[gr];
                    for (int d = 0; d < 3; ++d) vs[d * N + l] += vs[d * N + gr];
                    cs[gl] = es[gl] = cs[gr] = es[gr] = 0.0;
                    for (int d = 0; d < 3; ++d) vs[d * N + gl] = vs[d * N + gr] = 0.0;
                }
        }
        for (long c = 0; c < N; ++c) {
            rho[c] += p->q * cs[c];
            if (es[c] > 0) {
                vs[c] /= es[c]; vs[N + c] /= es[c]; vs[2 * N + c] /= es[c];
            } else {
                vs[c] = vs[N + c] = vs[2 * N + c] = 0.0;
            }
        }
    }
}
