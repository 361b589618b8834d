// diag.cuh -- diagnostics pass of updateDensityParameters
// (PIC++/momentum_collecting.cpp:760-1020): per species concentration,
// energy density and bulk velocity on cells, and the charge density.
#pragma once
#include "common.cuh"

namespace pic {

// Cell-weight deposit of one species: conc += w S / V, energy += w gamma m
// S / V, mom[3] += w p S / V (FP64 global atomics; a diagnostic, run every
// output interval).
template <typename T>
__global__ void __launch_bounds__(256) k_density_deposit(GridP g, PartView<T> p, double m, double w,
                                                         double* __restrict__ conc, double* __restrict__ energy,
                                                         double* __restrict__ mom) {
    const double ivol = 1.0 / (g.dx * g.dy * g.dz);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < p.n;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, p.cell[n], i, j, k);
        const double px = double(p.px[n]), py = double(p.py[n]), pz = double(p.pz[n]);
        const double gam = sqrt((px * px + py * py + pz * pz) / (m * m) + 1.0);
        const double wv = w * ivol;
        int X[2], Y[2], Z[2];
        T wx[2], wy[2], wz[2];
        cell_w(p.ox[n], i, g.nx, X, wx); cell_w(p.oy[n], j, g.ny, Y, wy); cell_w(p.oz[n], k, g.nz, Z, wz);
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) {
                    if ((!g.y3 && b) || (!g.z3 && c)) continue;
                    const long long id = lin(g, X[a], Y[b], Z[c]);
                    const double s = double(wx[a]) * double(wy[b]) * double(wz[c]) * wv;
                    atomicAdd(&conc[id], s);
                    atomicAdd(&energy[id], s * gam * m);
                    atomicAdd(&mom[id], s * px);
                    atomicAdd(&mom[g.N + id], s * py);
                    atomicAdd(&mom[2 * g.N + id], s * pz);
                }
    }
}

}  // namespace pic
