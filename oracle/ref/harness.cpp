// harness.cpp -- drives the PIC++ reference's own Simulation methods on a
// given periodic state and writes the result, to pin the C restatement in
// oracle/oracle.c.  TEST INFRASTRUCTURE ONLY: linked against the reference's
// object files (built by oracle/Makefile into oracle/_ref/, never shipped).
//
// It replays the step loop of Simulation::simulate (PIC++/simulation.cpp
// 164-259, 266-409) phase by phase instead of calling simulate(), so that the
// state can be loaded from a file (no text decks, no srand(time)), the time
// step is not clamped by updateDeltaT (simulation.cpp:1065-1078) and no
// output files are written.  The wall time of the step loop goes to stdout.
//
// Input file (little endian):
//   int32[10]  solver (0 Buneman, 1 implicit), nx, ny, nz, nspecies, steps,
//              dump_first_step_moments, density_pass, smoothing_count, wall_x
//   float64[11] dx, dt, theta, eta, smoothing_parameter, E_right[3], B_right[3]
// wall_x = 1: SUPER_CONDUCTOR_LEFT with a constant field E_right, B_right
// at the open right boundary (initializeFluxFromRight,
// initialization.cpp:5201-5207; for Buneman runs E_right is Simulation::E0,
// which tristanEvaluateE writes on the boundary node); the reference box
// then has nx - 2 cells along x, the two remaining storage columns being
// its ghost cells beyond the open boundary and left of the wall.  Particles
// that escape are written back with NaN coordinates; no particles are
// injected.
//   per species: float64 q, m, w; int64 n; float64 x[n], y[n], z[n] (in
//              [0, L) of the periodic box), px[n], py[n], pz[n]
//   float64 E[3][nz][ny][nx], B[3][nz][ny][nx] on our periodic layout
//              (Yee staggering for Buneman, node E / cell B for implicit)
// Output file: per species int64 n and x,y,z,px,py,pz in input order; then
// E[3][N], B[3][N]; Buneman adds J[3][N]; implicit with the dump flag adds
// the first step's J-hat[3][N], mu[9][N], rho-hat[N], Pi[9][N], rhs[3][N],
// E-theta[3][N].
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cmath>
#include <vector>
#include <algorithm>
#include <chrono>
#include <mpi.h>
#include "simulation.h"
#include "particle.h"
#include "vector3d.h"
#include "matrix3d.h"
#include "boundaryFieldEvaluator.h"

static void die(const char* m) { fprintf(stderr, "harness: %s\n", m); exit(2); }

template <class T> static T rd(FILE* f) { T v; if (fread(&v, sizeof(T), 1, f) != 1) die("short read"); return v; }
static void rdv(FILE* f, double* p, size_t n) { if (fread(p, sizeof(double), n, f) != n) die("short read"); }
static void wrv(FILE* f, const double* p, size_t n) { fwrite(p, sizeof(double), n, f); }

struct Box { int nx, ny, nz; };
static inline int wrap(int a, int n) { a %= n; return a < 0 ? a + n : a; }
// reference index r (ghosted) -> our periodic index
static inline int per(int r, int n) { return n == 1 ? 0 : wrap(r - 2, n); }
static inline long pidx(const Box& b, int i, int j, int k) { return ((long)k * b.ny + j) * b.nx + i; }

int main(int argc, char** argv) {
    if (argc != 3) die("usage: harness in.bin out.bin");
    FILE* f = fopen(argv[1], "rb");
    if (!f) die("cannot open input");
    int32_t hdr[10];
    for (int a = 0; a < 10; ++a) hdr[a] = rd<int32_t>(f);
    const int solver = hdr[0], nx = hdr[1], ny = hdr[2], nz = hdr[3], ns = hdr[4], steps = hdr[5], dump = hdr[6];
    const int density = hdr[7];   // 1: append updateDensityParameters' grids after the run
    const int smoothing = hdr[8];  // smoothingCount
    double dx = rd<double>(f), dt = rd<double>(f), theta = rd<double>(f), eta = rd<double>(f);
    const double smoothing_parameter = rd<double>(f);
    const int wall = hdr[9];
    double eright[3], bright[3];
    for (int a = 0; a < 3; ++a) eright[a] = rd<double>(f);
    for (int a = 0; a < 3; ++a) bright[a] = rd<double>(f);
    // Buneman runs reflect at xgrid[reflectingWallPoint = 20] (constants.h:64)
    if (wall && (nx < (solver == 0 ? 24 : 4) || ny < 2 || nz < 2)) die("wall_x needs a 3-D box (nx >= 24 for Buneman)");
    Box bx{nx, ny, nz};
    const long N = (long)nx * ny * nz;

    struct Sp { double q, m, w; long n; std::vector<double> x, y, z, px, py, pz; };
    std::vector<Sp> sp(ns);
    for (int s = 0; s < ns; ++s) {
        sp[s].q = rd<double>(f); sp[s].m = rd<double>(f); sp[s].w = rd<double>(f);
        sp[s].n = rd<int64_t>(f);
        for (auto* v : {&sp[s].x, &sp[s].y, &sp[s].z, &sp[s].px, &sp[s].py, &sp[s].pz}) {
            v->resize(sp[s].n); rdv(f, v->data(), sp[s].n);
        }
    }
    std::vector<double> E(3 * N), B(3 * N);
    rdv(f, E.data(), 3 * N); rdv(f, B.data(), 3 * N);
    fclose(f);

    MPI_Comm comm = 0;
    int ppb[8] = {1, 0, 0, 0, 0, 0, 0, 0};
    double conc[8] = {1, 0, 0, 0, 0, 0, 0, 0};
    // Theoretical input type (1) keeps dx as given (initialization.cpp:449-460).
    Simulation* S = new Simulation(wall ? nx - 2 : nx, ny, nz, dx, 0.0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0, 0, 1.0,
                                   steps, 1e300, 1 << 30, 1 << 30, 1 << 30, 1 << 30, 0, 0.0, false, 8, ppb,
                                   conc, 1, 1, 0, dt, 1.0, comm);
    S->timing = false;
    S->verbosity = 0;
    S->solverType = solver == 0 ? BUNEMAN : IMPLICIT;
    S->boundaryConditionTypeX = wall ? SUPER_CONDUCTOR_LEFT : PERIODIC;
    S->boundaryConditionTypeY = PERIODIC;
    S->boundaryConditionTypeZ = PERIODIC;
    S->smoothingCount = smoothing;
    S->smoothingParameter = smoothing_parameter;
    S->theta = theta;
    S->eta = eta;
    S->deltaT = dt;
    S->V0 = Vector3d(0, 0, 0);
    S->E0 = Vector3d(0, 0, 0);
    S->B0 = Vector3d(0, 0, 0);
    S->createArrays();
    Vector3d Er(eright[0], eright[1], eright[2]), Br(bright[0], bright[1], bright[2]);
    if (wall) S->rightBoundaryFieldEvaluator = new ConstantBoundaryFieldEvaluator(Er, Br);
    if (wall && solver == 0) S->E0 = Er;
    // grid coordinates as Simulation::initialize builds them (initialization.cpp:1989-2023)
    S->xgrid[0] = S->leftX;
    for (int i = 1; i <= S->xnumberAdded; ++i) S->xgrid[i] = S->xgrid[0] + i * S->deltaX;
    S->ygrid[0] = S->leftY;
    for (int j = 0; j <= S->ynumberAdded; ++j) S->ygrid[j] = S->ygrid[0] + j * S->deltaY;
    S->zgrid[0] = S->leftZ;
    for (int k = 0; k <= S->znumberAdded; ++k) S->zgrid[k] = S->zgrid[0] + k * S->deltaZ;
    for (int i = 0; i < S->xnumberAdded; ++i) S->middleXgrid[i] = (S->xgrid[i] + S->xgrid[i + 1]) / 2;
    for (int j = 0; j < S->ynumberAdded; ++j) S->middleYgrid[j] = (S->ygrid[j] + S->ygrid[j + 1]) / 2;
    for (int k = 0; k < S->znumberAdded; ++k) S->middleZgrid[k] = (S->zgrid[k] + S->zgrid[k + 1]) / 2;
    // evaluateElectricField reads the species table for a diagnostic only
    S->types = new ParticleTypeContainer[8];
    for (int t = 0; t < 8; ++t) { S->types[t].concentration = 0; S->types[t].charge = 1; S->types[t].mass = 1; }

    const int XA = S->xnumberAdded, YA = S->ynumberAdded, ZA = S->znumberAdded;
    if (solver == 0) {
        // Yee components, every reference index including ghosts
        for (int i = 0; i <= XA; ++i)
            for (int j = 0; j <= YA; ++j)
                for (int k = 0; k <= ZA; ++k) {
                    long c = pidx(bx, per(i, nx), per(j, ny), per(k, nz));
                    if (i < XA) { S->bunemanEx[i][j][k] = E[c]; S->bunemanNewEx[i][j][k] = E[c]; }
                    if (j < YA) { S->bunemanEy[i][j][k] = E[N + c]; S->bunemanNewEy[i][j][k] = E[N + c]; }
                    if (k < ZA) { S->bunemanEz[i][j][k] = E[2 * N + c]; S->bunemanNewEz[i][j][k] = E[2 * N + c]; }
                    if (j < YA && k < ZA) S->bunemanBx[i][j][k] = B[c];
                    if (i < XA && k < ZA) S->bunemanBy[i][j][k] = B[N + c];
                    if (i < XA && j < YA) S->bunemanBz[i][j][k] = B[2 * N + c];
                }
    } else {
        for (int i = 0; i <= XA; ++i)
            for (int j = 0; j <= YA; ++j)
                for (int k = 0; k <= ZA; ++k) {
                    long c = pidx(bx, per(i, nx), per(j, ny), per(k, nz));
                    Vector3d e(E[c], E[N + c], E[2 * N + c]);
                    S->Efield[i][j][k] = e; S->newEfield[i][j][k] = e; S->tempEfield[i][j][k] = e;
                    S->explicitEfield[i][j][k] = e;
                    if (i < XA && j < YA && k < ZA) {
                        Vector3d b(B[c], B[N + c], B[2 * N + c]);
                        S->Bfield[i][j][k] = b; S->newBfield[i][j][k] = b;
                    }
                }
    }

    // particles: reference coordinate = xgrid[2] + physical position
    int number = 0;
    std::vector<long> base(ns + 1, 0);
    for (int s = 0; s < ns; ++s) base[s + 1] = base[s] + sp[s].n;
    for (int s = 0; s < ns; ++s) {
        for (long a = 0; a < sp[s].n; ++a) {
            double x = S->xgrid[2] + sp[s].x[a];
            double y = ny > 1 ? S->ygrid[2] + sp[s].y[a] : S->ygrid[0] + sp[s].y[a];
            double z = nz > 1 ? S->zgrid[2] + sp[s].z[a] : S->zgrid[0] + sp[s].z[a];
            Particle* p = new Particle(number++, sp[s].m, 1, sp[s].q, sp[s].w, ELECTRON, x, y, z,
                                       sp[s].px[a], sp[s].py[a], sp[s].pz[a],
                                       S->deltaX / 2, S->deltaY / 2, S->deltaZ / 2, dt);
            S->particles.push_back(p);
        }
    }
    S->updateParticlesBeta();

    std::vector<double> dJ, dMu, dRho, dPi, dRhs, dEt;
    const auto t_loop = std::chrono::steady_clock::now();   // the step loop's wall time goes to stdout
    if (solver == 0) {
        S->exchangeBunemanBfield(S->bunemanBx, S->bunemanBy, S->bunemanBz);
        S->exchangeBunemanEfield(S->bunemanEx, S->bunemanEy, S->bunemanEz);
        for (int it = 0; it < steps; ++it) {
            // simulation.cpp:164-204
            S->tristanEvaluateBhalfStep();
            S->exchangeBunemanBfield(S->bunemanBx, S->bunemanBy, S->bunemanBz);
            S->moveParticles();
            S->tristanEvaluateBhalfStep();
            S->exchangeBunemanBfield(S->bunemanBx, S->bunemanBy, S->bunemanBz);
            S->tristanUpdateFlux();
            for (int n = 0; n < S->smoothingCount; ++n)   // simulation.cpp:186-188
                S->smoothBunemanEfieldGeneral(S->bunemanJx, S->bunemanJy, S->bunemanJz);
            S->tristanEvaluateE();
            S->exchangeBunemanEfield(S->bunemanEx, S->bunemanEy, S->bunemanEz);
            // simulation.cpp:266-279, 394
            S->eraseEscapedPaticles();
            S->exchangeParticles();
            S->removeEscapedParticles();
            S->time += dt;
            S->currentIteration++;
        }
    } else {
        S->exchangeEfield();
        S->exchangeGeneralBfield(S->Bfield);
        S->exchangeGeneralBfield(S->newBfield);
        S->updateParticleCorrelationMaps();
        for (int it = 0; it < steps; ++it) {
            // simulation.cpp:205-259
            S->evaluateParticlesRotationTensor();
            S->updateElectroMagneticParameters();
            for (int n = 0; n < S->smoothingCount; ++n) {   // simulation.cpp:213-217
                S->smoothChargeDensityHat();
                S->smoothFlux();
                S->smoothMatrixNodeParameter(S->dielectricTensor);
            }
            S->evaluateElectricField();
            S->exchangeEfield();
            S->evaluateMagneticField();
            S->exchangeGeneralBfield(S->newBfield);
            S->exchangeGeneralEfield(S->tempEfield);
            S->exchangeGeneralEfield(S->newEfield);
            if (it == 0 && dump) {
                dJ.assign(3 * N, 0); dMu.assign(9 * N, 0); dRho.assign(N, 0); dPi.assign(9 * N, 0);
                dRhs.assign(3 * N, 0); dEt.assign(3 * N, 0);
                for (int k = 0; k < nz; ++k)
                    for (int j = 0; j < ny; ++j)
                        for (int i = 0; i < nx; ++i) {
                            int ri = i + 2, rj = ny > 1 ? j + 2 : 0, rk = nz > 1 ? k + 2 : 0;
                            long c = pidx(bx, i, j, k);
                            for (int d = 0; d < 3; ++d) {
                                dJ[d * N + c] = S->electricFlux[ri][rj][rk][d];
                                dRhs[d * N + c] = S->maxwellEquationRightPart[ri][rj][rk][d];
                                dEt[d * N + c] = S->tempEfield[ri][rj][rk][d];
                            }
                            for (int a = 0; a < 3; ++a)
                                for (int b = 0; b < 3; ++b) {
                                    dMu[(3 * a + b) * N + c] = S->dielectricTensor[ri][rj][rk].matrix[a][b];
                                    dPi[(3 * a + b) * N + c] = S->pressureTensor[ri][rj][rk].matrix[a][b];
                                }
                            dRho[c] = S->chargeDensityHat[ri][rj][rk];
                        }
            }
            S->moveParticles();
            // simulation.cpp:266-279, 294-350, 360
            S->eraseEscapedPaticles();
            S->exchangeParticles();
            S->updateParticleCorrelationMaps();
            S->exchangeGeneralEfield(S->newEfield);
            S->updateFields();
            S->exchangeGeneralEfield(S->newEfield);
            S->exchangeGeneralEfield(S->Efield);
            S->exchangeGeneralBfield(S->Bfield);
            S->removeEscapedParticles();
            S->time += dt;
            S->currentIteration++;
        }
    }

    printf("harness: %d steps in %.6f s\n", steps,
           std::chrono::duration<double>(std::chrono::steady_clock::now() - t_loop).count());

    // collect particles back in input order (Particle::number)
    long total = base[ns];
    std::vector<Particle*> byNum(total, nullptr);
    for (Particle* p : S->particles) {
        if (p->number < 0 || p->number >= total) die("bad particle number");
        byNum[p->number] = p;
    }
    for (long a = 0; a < total; ++a) if (!byNum[a] && !wall) die("particle lost");
    FILE* o = fopen(argv[2], "wb");
    if (!o) die("cannot open output");
    const double Lx = (wall ? nx - 2 : nx) * S->deltaX, Ly = ny * S->deltaY, Lz = nz * S->deltaZ;
    for (int s = 0; s < ns; ++s) {
        int64_t n = sp[s].n; fwrite(&n, sizeof(n), 1, o);
        std::vector<double> X(n), Y(n), Z(n), PX(n), PY(n), PZ(n);
        for (long a = 0; a < n; ++a) {
            Particle* p = byNum[base[s] + a];
            if (!p) {   // escaped through the open boundary
                X[a] = Y[a] = Z[a] = PX[a] = PY[a] = PZ[a] = std::nan("");
                continue;
            }
            double x = p->coordinates.x - S->xgrid[2];
            double y = ny > 1 ? p->coordinates.y - S->ygrid[2] : p->coordinates.y - S->ygrid[0];
            double z = nz > 1 ? p->coordinates.z - S->zgrid[2] : p->coordinates.z - S->zgrid[0];
            X[a] = x - Lx * std::floor(x / Lx); Y[a] = y - Ly * std::floor(y / Ly); Z[a] = z - Lz * std::floor(z / Lz);
            Vector3d mom = p->getMomentum();
            PX[a] = mom.x; PY[a] = mom.y; PZ[a] = mom.z;
        }
        wrv(o, X.data(), n); wrv(o, Y.data(), n); wrv(o, Z.data(), n);
        wrv(o, PX.data(), n); wrv(o, PY.data(), n); wrv(o, PZ.data(), n);
    }
    std::vector<double> Eo(3 * N), Bo(3 * N), Jo(3 * N);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int ri = i + 2, rj = ny > 1 ? j + 2 : 0, rk = nz > 1 ? k + 2 : 0;
                long c = pidx(bx, i, j, k);
                if (solver == 0) {
                    Eo[c] = S->bunemanEx[ri][rj][rk]; Eo[N + c] = S->bunemanEy[ri][rj][rk]; Eo[2 * N + c] = S->bunemanEz[ri][rj][rk];
                    Bo[c] = S->bunemanBx[ri][rj][rk]; Bo[N + c] = S->bunemanBy[ri][rj][rk]; Bo[2 * N + c] = S->bunemanBz[ri][rj][rk];
                    Jo[c] = S->bunemanJx[ri][rj][rk]; Jo[N + c] = S->bunemanJy[ri][rj][rk]; Jo[2 * N + c] = S->bunemanJz[ri][rj][rk];
                } else {
                    for (int d = 0; d < 3; ++d) { Eo[d * N + c] = S->Efield[ri][rj][rk][d]; Bo[d * N + c] = S->Bfield[ri][rj][rk][d]; }
                }
            }
    wrv(o, Eo.data(), 3 * N); wrv(o, Bo.data(), 3 * N);
    if (solver == 0) wrv(o, Jo.data(), 3 * N);
    if (solver == 1 && dump) {
        wrv(o, dJ.data(), 3 * N); wrv(o, dMu.data(), 9 * N); wrv(o, dRho.data(), N);
        wrv(o, dPi.data(), 9 * N); wrv(o, dRhs.data(), 3 * N); wrv(o, dEt.data(), 3 * N);
    }
    if (density) {
        // momentum_collecting.cpp:760-1020 on the final state; every particle
        // is of type 0 here, whose folds run only for a populated type
        // (momentum_exchange.cpp:1056)
        S->types[0].particlesPerBin = 1;
        S->updateParticleCorrelationMaps();
        S->updateDensityParameters();
        std::vector<double> C(N), En(N), V(3 * N), R(N);
        for (int t = 0; t < ns; ++t) {
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        int ri = i + 2, rj = ny > 1 ? j + 2 : 0, rk = nz > 1 ? k + 2 : 0;
                        long c = pidx(bx, i, j, k);
                        C[c] = S->particleConcentrations[t][ri][rj][rk];
                        En[c] = S->particleEnergies[t][ri][rj][rk];
                        for (int d = 0; d < 3; ++d) V[d * N + c] = S->particleBulkVelocities[t][ri][rj][rk][d];
                        R[c] = S->chargeDensity[ri][rj][rk];
                    }
            wrv(o, C.data(), N); wrv(o, En.data(), N); wrv(o, V.data(), 3 * N);
        }
        wrv(o, R.data(), N);
    }
    fclose(o);
    return 0;
}
