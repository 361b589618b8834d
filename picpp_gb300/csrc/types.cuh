// types.cuh -- plain structs shared by host launchers and kernels.
#pragma once
#include "common.cuh"

namespace pic {

constexpr int kMaxSpecies = 8;

// Reference ghosted-axis geometry for the pressure-tensor path
// (implicit_grid.cuh): interior cell c of an axis with n > 1 is index c + 2,
// the axis holds n + 4 cells; a single-cell axis keeps index 0.
struct GhostAxes {
    int cex, cey, cez;     // cell extents
    int gx, gy, gz;        // ghost offsets (2 or 0)
};

// Tiles of the tile-major sort key and of the per-tile particle kernels.
struct TileGeom {
    int tx, ty, tz;      // tile extents
    int ntx, nty, ntz;   // tiles per axis
    int lx, ly, lz;      // log2 of the extents when all three are powers of two, else -1
};

// Shared-memory blocks of the fused explicit kernel (boris_tile.cuh).
struct TileShape {
    int fx, fy, fz;   // staged field block (tile + 1 halo each side on active axes)
    int jx, jy, jz;   // current block (tile + 2 halo each side on active axes)
    int hx, hy, hz;   // halo widths of the field block (1 or 0)
    int gx, gy, gz;   // halo widths of the current block (2 or 0)
    long long jcells; // jx*jy*jz
};

template <typename TP>
struct SpeciesSet {
    PartView<TP> p[kMaxSpecies];
    TP q[kMaxSpecies], m[kMaxSpecies], w[kMaxSpecies];
    const int* off[kMaxSpecies];   // per-species sort offsets (nkeys + 1)
    // per species: the particles the fused explicit kernel leaves to its
    // deferred pass, one bit each -- dwords words of push-later bits, then
    // dwords words of deposit-later bits
    unsigned* defer[kMaxSpecies];
    long long dwords[kMaxSpecies];
    int ns;
};

// Species of the tiled implicit deposit (implicit_tile.cuh).
template <typename T>
struct ImpSpecies {
    PartView<T> p[kMaxSpecies];
    double q[kMaxSpecies], m[kMaxSpecies], w[kMaxSpecies];
    const int* off[kMaxSpecies];   // sort offsets by key (nkeys + 1)
    unsigned* defer[kMaxSpecies];  // the tiled mover's deferred particles, one bit each
    int ns;
};

// Shared accumulator blocks of the tiled implicit deposit: node block
// extent t + 2h + 1 and cell block extent t + 2h + 2 on active axes, 1 on a
// single-cell axis.
struct ImpBlock {
    int h;
    int nbx, nby, nbz, NB;
    int cbx, cby, cbz, CB;
    int stage;   // 1: E (node block) and B (cell block) staged in shared memory too (h = 0 only)
};

// Coefficients of the matrix-free Maxwell operator (implicit_grid.cuh).
struct OpCoef {
    double K;
    double kd2[3];      // K / d^2
    double kx4[3][3];   // K / (4 da dd)
    int has[3];
};

}  // namespace pic
