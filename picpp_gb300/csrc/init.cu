// init.cu -- pic_fill_species: seeded synthetic particle loading on the
// device, for workloads too large to build on the host (hundreds of millions
// of particles).  No reference counterpart: the reference's initialisers
// (PIC++/initialization.cpp:8145-8574) are replaced by this generator and by
// picpp_gb300/initstate.py, which implement the same distribution.
//
// Particle p of the species sits in cell p / ppc; its in-cell offsets are
// uniform; its momentum is drawn from a Maxwell-Juttner law of temperature
// theta (inverse transform on a tabulated CDF of u = |p|/mc, isotropic
// direction) and, when drift_gamma > 1, boosted along +-x with the flipping
// method (Zenitani 2015, Phys. Plasmas 22, 042116).  Random numbers come from
// splitmix64 of (seed, species, particle, draw), so the result does not
// depend on the launch configuration.
#include <cmath>
#include <vector>

#include "../../include/picpp_gb300.h"
#include "common.cuh"
#include "kernels.hpp"

namespace {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ double urand(unsigned long long seed, long long p, int draw) {
    unsigned long long h = splitmix64(seed ^ splitmix64((unsigned long long)p * 16ull + (unsigned long long)draw));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);   // [0, 1)
}

// rowx: cells per x row that receive particles, from cell x0 on (nx from
// 0, or fewer in a wall box whose two ghost columns stay empty); nx: the
// storage row length.
template <typename T>
__global__ void k_fill(pic::PartView<T> p, long long ppc, unsigned long long seed, const double* __restrict__ cdf_u,
                       const double* __restrict__ cdf, int ntab, double mass, double drift_gamma, int alternate,
                       int rowx, int nx, int x0) {
    const double beta = drift_gamma > 1.0 ? sqrt(1.0 - 1.0 / (drift_gamma * drift_gamma)) : 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < p.n; n += (long long)gridDim.x * blockDim.x) {
        const long long q = n / ppc;   // the q-th filled cell
        p.cell[n] = (int)((q / rowx) * nx + x0 + q % rowx);
        p.id[n] = (int)n;
        double o[3];
        for (int a = 0; a < 3; ++a) {
            o[a] = urand(seed, n, a);
            T t = T(o[a]);
            if (t >= T(1)) t = T(1) - T(1) / T(1 << 24);
            (a == 0 ? p.ox : a == 1 ? p.oy : p.oz)[n] = t;
        }
        double u = 0.0;
        if (ntab > 1) {
            // inverse CDF by bisection on the table, then linear interpolation
            double r = urand(seed, n, 3);
            int lo = 0, hi = ntab - 1;
            while (hi - lo > 1) {
                int mid = (lo + hi) >> 1;
                if (cdf[mid] <= r) lo = mid; else hi = mid;
            }
            double c0 = cdf[lo], c1 = cdf[hi];
            double f = c1 > c0 ? (r - c0) / (c1 - c0) : 0.0;
            u = cdf_u[lo] + f * (cdf_u[hi] - cdf_u[lo]);
        }
        double ct = 2.0 * urand(seed, n, 4) - 1.0;
        double ph = 2.0 * 3.14159265358979323846 * urand(seed, n, 5);
        double st = sqrt(fmax(0.0, 1.0 - ct * ct));
        double ux = u * ct, uy = u * st * cos(ph), uz = u * st * sin(ph);
        if (beta > 0.0) {
            double sign = alternate > 0 ? ((n & 1) ? -1.0 : 1.0) : (alternate < 0 ? -1.0 : 1.0);
            double g = sqrt(1.0 + ux * ux + uy * uy + uz * uz);
            if (-beta * sign * (ux / g) > urand(seed, n, 6)) ux = -ux;
            ux = drift_gamma * (ux + sign * beta * g);
        }
        p.px[n] = T(ux * mass);
        p.py[n] = T(uy * mass);
        p.pz[n] = T(uz * mass);
    }
}

}  // namespace

namespace pic {

// Host side: the CDF of u under f(u) ~ u^2 exp(-(gamma-1)/theta).
std::vector<double> juttner_table(double theta, int n, std::vector<double>& us) {
    std::vector<double> cdf(n, 0.0);
    us.assign(n, 0.0);
    double umax = std::sqrt((1.0 + 40.0 * theta) * (1.0 + 40.0 * theta) - 1.0) + 1e-12;
    double prev = 0.0;
    for (int a = 0; a < n; ++a) {
        double u = umax * a / (n - 1);
        double g = std::sqrt(1.0 + u * u);
        double pdf = u * u * std::exp(-(g - 1.0) / theta);
        us[a] = u;
        if (a > 0) cdf[a] = cdf[a - 1] + 0.5 * (pdf + prev) * (us[a] - us[a - 1]);
        prev = pdf;
    }
    for (int a = 0; a < n; ++a) cdf[a] /= cdf[n - 1];
    return cdf;
}

template <typename T>
void launch_fill(cudaStream_t s, PartView<T> p, long long ppc, unsigned long long seed, const double* u, const double* c,
                 int ntab, double mass, double drift_gamma, int alternate, int rowx, int nx, int x0) {
    k_fill<T><<<grid_for(p.n, 256, 32), 256, 0, s>>>(p, ppc, seed, u, c, ntab, mass, drift_gamma, alternate, rowx, nx, x0);
}
template void launch_fill<float>(cudaStream_t, PartView<float>, long long, unsigned long long, const double*,
                                 const double*, int, double, double, int, int, int, int);
template void launch_fill<double>(cudaStream_t, PartView<double>, long long, unsigned long long, const double*,
                                  const double*, int, double, double, int, int, int, int);

}  // namespace pic
