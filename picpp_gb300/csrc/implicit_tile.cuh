// implicit_tile.cuh -- moment deposition of the implicit path over tiles of
// cells (updateElectroMagneticParameters, PIC++/momentum_collecting.cpp
// 365-584, with the pressure tensor at the particle's own cells).
//
// Particles are ordered by the tile-major cell key (sort.cuh).  One CTA owns
// a tile and accumulates, in shared memory,
//   * on nodes (tile + h halo + 1):  J-hat (3) and mu (9), 8 nodes/particle;
//   * on cells (tile + h halo + 2):  rho-hat (1) and Pi (6 of the symmetric
//     9), 8 of the 27 cells around the particle's cell.
// A warp takes one cell key at a time and walks its particles 32 at a time.
// Lanes holding the same (current) cell share one stencil base, so their
// 96 node and 189 cell products (27 slots, zero weight outside the
// particle's octant) are summed over the run before one shared-memory atomic
// per sum: with FP32 accumulators as small TF32 tensor-core products at FP32
// accuracy (tc_run_sums), with FP64 accumulators by a butterfly
// transpose-reduction (after five exchange rounds lane L holds the warp total
// of product L of a 32-product pass).  Runs of only a few lanes add their
// products directly; particles more than h cells
// outside the tile add theirs to the FP64 grids with global atomics.  The
// tile's block is finally added to the FP64 grids (global atomics only on
// block entries, 22 per node/cell).
#pragma once
#include "implicit_particles.cuh"

namespace pic {

#ifndef PIC_IMP_THREADS
#define PIC_IMP_THREADS 256   // threads per CTA of the tiled implicit deposit (2 CTAs/SM, 128 registers)
#endif
#ifndef PIC_MOVER_THREADS
#define PIC_MOVER_THREADS 256   // threads per CTA of the tiled implicit mover (2 CTAs/SM)
#endif
constexpr int kImpThreads = PIC_IMP_THREADS;
// FP64 particles keep 256 threads (128 registers): their accumulators spill at 64
template <typename T>
__host__ __device__ constexpr int imp_threads() { return sizeof(T) == sizeof(float) ? kImpThreads : 256; }
constexpr int kMoverThreads = PIC_MOVER_THREADS;
constexpr int kXposeMin = 4;   // fewest lanes of one cell that take the transpose-reduction (FP64)
constexpr int kTcMin = 1;      // fewest lanes of one cell that take the tensor-core run sums (FP32)


// Symmetric pressure components kept in shared memory, q = 0..5:
// (a, b) = (0,0) (0,1) (0,2) (1,1) (1,2) (2,2).
__host__ __device__ constexpr int sym_a(int q) { return q < 3 ? 0 : (q < 5 ? 1 : 2); }
__host__ __device__ constexpr int sym_b(int q) { return q < 3 ? q : (q < 5 ? q - 2 : 2); }

// Butterfly transpose-reduction of one 32-product pass: returns, in lane L,
// the sum over the warp of v[L].
template <typename A>
__device__ __forceinline__ A xpose_sum(A v[32], int lane) {
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const bool up = (lane & w) != 0;
#pragma unroll
        for (int i = 0; i < w; ++i) {
            const A send = up ? v[i] : v[i + w];
            const A keep = up ? v[i + w] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, w);
        }
    }
    return v[0];
}

// Node / cell weights of one axis (node_w and cell_w of common.cuh, in the
// three-slot form c-1, c, c+1 for cells).
template <typename T>
__device__ __forceinline__ void axis_weights(T u, bool act, T wn[2], T wc[3]) {
    if (!act) { wn[0] = T(1); wn[1] = T(0); wc[0] = T(0); wc[1] = T(1); wc[2] = T(0); return; }
    if (u < T(0.5)) { wn[0] = T(0.5) + (T(0.5) - u); wn[1] = T(1) - wn[0]; }
    else            { wn[1] = T(0.5) + (u - T(0.5)); wn[0] = T(1) - wn[1]; }
    if (u < T(0.5)) { wc[1] = T(0.5) + u; wc[0] = T(1) - wc[1]; wc[2] = T(0); }
    else            { wc[1] = T(0.5) + (T(1) - u); wc[2] = T(1) - wc[1]; wc[0] = T(0); }
}

// Local index of global cell index c on an axis of n cells relative to a
// tile starting at x0, chosen within [-h, t - 1 + h] when a periodic image
// lies there; false if none does.
__device__ __forceinline__ bool local_axis(int c, int x0, int t, int h, int n, int& l) {
    l = c - x0;
    if (l >= -h && l <= t - 1 + h) return true;
    if (l - n >= -h && l - n <= t - 1 + h) { l -= n; return true; }
    if (l + n >= -h && l + n <= t - 1 + h) { l += n; return true; }
    return false;
}

// Trilinear gather from a staged block: base = block index of the lower
// corner, (sx, sy, sz) strides (0 on a single-cell axis), weights of the
// upper corners.
template <typename T>
__device__ __forceinline__ T tri_block(const T* __restrict__ F, int base, int sx, int sy, int sz, T wx, T wy, T wz) {
    const T ux = T(1) - wx, uy = T(1) - wy, uz = T(1) - wz;
    return uz * (uy * (ux * F[base] + wx * F[base + sx]) + wy * (ux * F[base + sy] + wx * F[base + sy + sx])) +
           wz * (uy * (ux * F[base + sz] + wx * F[base + sz + sx]) +
                 wy * (ux * F[base + sz + sy] + wx * F[base + sz + sy + sx]));
}

// The same trilinear form on a block of float4 nodes or cells (x, y, z, unused):
// one 16-byte load per corner for all three components, each component
// evaluated in exactly tri_block's order.
__device__ __forceinline__ void tri_block4(const float4* __restrict__ F, int base, int sx, int sy, int sz, float wx,
                                           float wy, float wz, float out[3]) {
    const float ux = 1.f - wx, uy = 1.f - wy, uz = 1.f - wz;
    const float4 f000 = F[base], f100 = F[base + sx], f010 = F[base + sy], f110 = F[base + sy + sx];
    const float4 f001 = F[base + sz], f101 = F[base + sz + sx], f011 = F[base + sz + sy], f111 = F[base + sz + sy + sx];
    out[0] = uz * (uy * (ux * f000.x + wx * f100.x) + wy * (ux * f010.x + wx * f110.x)) +
             wz * (uy * (ux * f001.x + wx * f101.x) + wy * (ux * f011.x + wx * f111.x));
    out[1] = uz * (uy * (ux * f000.y + wx * f100.y) + wy * (ux * f010.y + wx * f110.y)) +
             wz * (uy * (ux * f001.y + wx * f101.y) + wy * (ux * f011.y + wx * f111.y));
    out[2] = uz * (uy * (ux * f000.z + wx * f100.z) + wy * (ux * f010.z + wx * f110.z)) +
             wz * (uy * (ux * f001.z + wx * f101.z) + wy * (ux * f011.z + wx * f111.z));
}

// ---- tensor-core reduction of one run (FP32 accumulators) -------------------
// The 96 node sums  N[q][c] = sum_p QN_p[q] wn_p[c]  and 189 cell sums
// C[s][q] = sum_p wc_p[s] QC_p[q]  of a run of particles are small matrix
// products with the particles as the inner dimension.  Each lane writes its
// particle's raw quantities (rv 3, alpha 9, per-axis node weights 2 x 3,
// per-axis cell weights 3 x 3) to a per-warp scratch of 32 rows; the warp
// then runs m16n8k8 TF32 MMAs, eight particles per MMA, in the 3 x TF32 form
// (x = hi + lo, products hi*hi + hi*lo + lo*hi, FP32 accumulation), which
// keeps the sums at FP32 accuracy.  The per-species factors (cq, cm) are
// applied to the sums.
constexpr int kScrRow = 27;         // scratch floats per particle
constexpr int kScrParticles = 32;   // scratch rows per warp

// x = hi + lo + e with hi, lo in the 19-bit TF32 format (low 13 bits zero),
// both truncated: x - hi is exact in FP32 (at most 13 significant bits) and
// |e| < 2^-21 |x|.  Three integer/FP32 operations per split.
__device__ __forceinline__ void tf32_split(float x, unsigned& hi, unsigned& lo) {
    hi = __float_as_uint(x) & 0xffffe000u;
    lo = __float_as_uint(x - __uint_as_float(hi)) & 0xffffe000u;
}

// D (16x8, FP32) += A (16x8, TF32, row) * B (8x8, TF32, col)
__device__ __forceinline__ void mma_tf32(float d[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// D += A * B at FP32 accuracy from pre-split B
__device__ __forceinline__ void mma_tf32x3(float d[4], const float a[4], const unsigned bh[2], const unsigned bl[2]) {
    unsigned ah[4], al[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) tf32_split(a[i], ah[i], al[i]);
    mma_tf32(d, al, bh);
    mma_tf32(d, ah, bl);
    mma_tf32(d, ah, bh);
}

// The scratch-row columns a lane reads in tc_run_sums, which depend on the
// lane only: byte k of sx / sy / sz is the column of the x / y / z weight
// of cell slot g + 8k (g = lane / 4); bytes of nb: the node weight columns
// 12 + gx, 14 + gy, 16 + gz and the rv columns ia, ib of pressure
// component g - 1.  Built once per CTA into a shared table.
struct TcLane {
    unsigned sx, sy, sz, nb;
};
__device__ __forceinline__ TcLane tc_lane(int lane) {
    const int g = lane >> 2;
    TcLane t{0u, 0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int sl = g + 8 * k;
        t.sx |= (unsigned)(18 + sl % 3) << (8 * k);
        t.sy |= (unsigned)(21 + (sl / 3) % 3) << (8 * k);
        t.sz |= (unsigned)(sl < 27 ? 24 + sl / 9 : 24) << (8 * k);
    }
    const int ia = g >= 1 && g <= 6 ? sym_a(g - 1) : 0, ib = g >= 1 && g <= 6 ? sym_b(g - 1) : 0;
    t.nb = (unsigned)(12 + (g & 1)) | (unsigned)(14 + ((g >> 1) & 1)) << 8 | (unsigned)(16 + (g >> 2)) << 16 |
           (unsigned)(ia | ib << 4) << 24;
    return t;
}
__device__ __forceinline__ int tc_byte(unsigned w, int k) { return (int)((w >> (8 * k)) & 0xffu); }

// Sums of one run over the warp, added to dn and dc: mem = lanes in the run;
// row = this lane's raw quantities (used only when the lane is in the run);
// tl = this lane's TcLane.  Lane (g = lane/4, t = lane%4) holds
// dn[i] = N[g + 8(i/2)][2t + i%2] and dc[4k + i] = C[16k + g + 8(i/2)][2t + i%2].
__device__ __forceinline__ void tc_run_sums(float* __restrict__ scr, int lane, bool me, unsigned mem,
                                            const float row[kScrRow], float dn[4], float dc[8], const TcLane tl) {
    const int g = lane >> 2, tq = lane & 3;
    const int cnx = tc_byte(tl.nb, 0), cny = tc_byte(tl.nb, 1), cnz = tc_byte(tl.nb, 2);
    const int ia = tc_byte(tl.nb, 3) & 15, ib = tc_byte(tl.nb, 3) >> 4;
    int sox[4], soy[4], soz[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        sox[k] = tc_byte(tl.sx, k);
        soy[k] = tc_byte(tl.sy, k);
        soz[k] = tc_byte(tl.sz, k);
    }
    {
        float* r = scr + lane * kScrRow;
#pragma unroll
        for (int f = 0; f < kScrRow; ++f) r[f] = me ? row[f] : 0.f;
    }
    __syncwarp();
#pragma unroll 1
    for (int s2 = 0; s2 < 4; ++s2) {
        if (((mem >> (8 * s2)) & 0xffu) == 0) continue;
        const float* P0 = scr + (8 * s2 + tq) * kScrRow;
        const float* P1 = P0 + 4 * kScrRow;
        unsigned bh[2], bl[2];
        float a[4];
        // nodes: A[q][p] = (rv, alpha)[q], q = g and g + 8 (< 12); B[p][c] = node weight of corner c = g
        tf32_split(P0[cnx] * P0[cny] * P0[cnz], bh[0], bl[0]);
        tf32_split(P1[cnx] * P1[cny] * P1[cnz], bh[1], bl[1]);
        a[0] = P0[g];
        a[1] = g < 4 ? P0[g + 8] : 0.f;
        a[2] = P1[g];
        a[3] = g < 4 ? P1[g + 8] : 0.f;
        mma_tf32x3(dn, a, bh, bl);
        // cells: A[s][p] = slot weight, s = 16k + g (+ 8); B[p][q] = 1, rv_a rv_b (q = g < 7)
        tf32_split(g == 0 ? 1.f : (g < 7 ? P0[ia] * P0[ib] : 0.f), bh[0], bl[0]);
        tf32_split(g == 0 ? 1.f : (g < 7 ? P1[ia] * P1[ib] : 0.f), bh[1], bl[1]);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int j0 = 2 * k, j1 = 2 * k + 1;   // slots 16k + g and 16k + g + 8
            const bool v1 = 16 * k + g + 8 < 27;
            a[0] = P0[sox[j0]] * P0[soy[j0]] * P0[soz[j0]];
            a[1] = v1 ? P0[sox[j1]] * P0[soy[j1]] * P0[soz[j1]] : 0.f;
            a[2] = P1[sox[j0]] * P1[soy[j0]] * P1[soz[j0]];
            a[3] = v1 ? P1[sox[j1]] * P1[soy[j1]] * P1[soz[j1]] : 0.f;
            mma_tf32x3(dc + 4 * k, a, bh, bl);
        }
    }
    __syncwarp();
}

// Adds the run sums of tc_run_sums (lane layout as there) to the shared
// blocks at node base nb and cell base cb, times the species factors.
__device__ __forceinline__ void add_run_sums(float* __restrict__ sN, float* __restrict__ sC, int NB, int CB, int nb,
                                             int cb, int oxn, int oyn, int ozn, int oxc, int oyc, int ozc, int lane,
                                             const float dn[4], const float dc[8], float cq, float cm) {
    const int gq = lane >> 2, tq = lane & 3;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int q = gq + 8 * (i >> 1), c = 2 * tq + (i & 1);
        if (q < 12 && dn[i] != 0.f)
            atomicAdd(&sN[q * NB + nb + (c & 1) * oxn + ((c >> 1) & 1) * oyn + (c >> 2) * ozn], dn[i] * (q < 3 ? cq : cm));
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int sl = 16 * (i >> 2) + gq + 8 * ((i >> 1) & 1), q = 2 * tq + (i & 1);
        if (sl < 27 && q < 7 && dc[i] != 0.f)
            atomicAdd(&sC[q * CB + cb + (sl % 3) * oxc + ((sl / 3) % 3) * oyc + (sl / 9) * ozc], dc[i] * cq);
    }
}

// Deposited quantities of one particle from its raw row: QN = (rv cq, alpha cm),
// QC = (cq, cq rv_a rv_b) over the symmetric pressure components.
template <typename A, typename T>
__device__ __forceinline__ void run_quantities(const T row[kScrRow], double cq, double cm, A QN[12], A QC[7]) {
    const A rv[3] = {A(row[0]), A(row[1]), A(row[2])};
#pragma unroll
    for (int d = 0; d < 3; ++d) QN[d] = rv[d] * A(cq);
#pragma unroll
    for (int d = 0; d < 9; ++d) QN[3 + d] = A(row[3 + d]) * A(cm);
    QC[0] = A(cq);
#pragma unroll
    for (int q = 0; q < 6; ++q) QC[1 + q] = A(cq) * (rv[sym_a(q)] * rv[sym_b(q)]);
}

// Node (8 corners) and cell (27 slots) weights from the per-axis weights of a row.
template <typename A, typename T>
__device__ __forceinline__ void run_weights(const T row[kScrRow], A wn[8], A wc[27]) {
#pragma unroll
    for (int c = 0; c < 8; ++c) wn[c] = A(row[12 + (c & 1)] * row[14 + ((c >> 1) & 1)] * row[16 + (c >> 2)]);
#pragma unroll
    for (int q = 0; q < 27; ++q) wc[q] = A(row[18 + q % 3] * row[21 + (q / 3) % 3] * row[24 + q / 9]);
}

// Direct shared-memory adds of one particle of a short run (rolled loops:
// rare, so kept small next to the hot code).
template <typename T>
__device__ __forceinline__ T pick2(const T* w, int i) { return i ? w[1] : w[0]; }
template <typename T>
__device__ __forceinline__ T pick3(const T* w, int i) { return i == 0 ? w[0] : (i == 1 ? w[1] : w[2]); }

template <typename A, typename T>
__device__ __forceinline__ void imp_deposit_direct(const T row[kScrRow], double cq, double cm, A* __restrict__ sN,
                                                   A* __restrict__ sC, int NB, int CB, int nb, int cb, int oxn, int oyn,
                                                   int ozn, int oxc, int oyc, int ozc) {
    A QN[12], QC[7];
    run_quantities<A, T>(row, cq, cm, QN, QC);
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
        const A w = A(pick2(row + 12, c & 1) * pick2(row + 14, (c >> 1) & 1) * pick2(row + 16, c >> 2));
        if (w == A(0)) continue;
        const int o = nb + (c & 1) * oxn + ((c >> 1) & 1) * oyn + (c >> 2) * ozn;
#pragma unroll
        for (int q = 0; q < 12; ++q) atomicAdd(&sN[q * NB + o], QN[q] * w);
    }
#pragma unroll 1
    for (int sl = 0; sl < 27; ++sl) {
        const A w = A(pick3(row + 18, sl % 3) * pick3(row + 21, (sl / 3) % 3) * pick3(row + 24, sl / 9));
        if (w == A(0)) continue;
        const int o = cb + (sl % 3) * oxc + ((sl / 3) % 3) * oyc + (sl / 9) * ozc;
#pragma unroll
        for (int q = 0; q < 7; ++q) atomicAdd(&sC[q * CB + o], QC[q] * w);
    }
}

// All 8 node and 8 cell contributions of one particle to the FP64 grids
// (particles outside the tile's block; rare).
template <typename T>
__device__ __noinline__ void imp_deposit_global(const GridP g, int i, int j, int k, T ox, T oy, T oz,
                                                const double* QN, const double* QC, double* __restrict__ J,
                                                double* __restrict__ mu, double* __restrict__ rho,
                                                double* __restrict__ Pi) {
    int X[2], Y[2], Z[2];
    T wx[2], wy[2], wz[2];
    node_w(ox, i, g.nx, X, wx); node_w(oy, j, g.ny, Y, wy); node_w(oz, k, g.nz, Z, wz);
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                double wgt = double(wx[a]) * double(wy[b]) * double(wz[c]);
                if (wgt == 0.0) continue;
                long long id = lin(g, X[a], Y[b], Z[c]);
                for (int d = 0; d < 3; ++d) atomicAdd(&J[d * g.N + id], QN[d] * wgt);
                for (int d = 0; d < 9; ++d) atomicAdd(&mu[d * g.N + id], QN[3 + d] * wgt);
            }
    cell_w(ox, i, g.nx, X, wx); cell_w(oy, j, g.ny, Y, wy); cell_w(oz, k, g.nz, Z, wz);
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                double wgt = double(wx[a]) * double(wy[b]) * double(wz[c]);
                if (wgt == 0.0) continue;
                long long id = lin(g, X[a], Y[b], Z[c]);
                atomicAdd(&rho[id], QC[0] * wgt);
                for (int s = 0; s < 6; ++s) {
                    double v = QC[1 + s] * wgt;
                    atomicAdd(&Pi[(3 * sym_a(s) + sym_b(s)) * g.N + id], v);
                    if (sym_a(s) != sym_b(s)) atomicAdd(&Pi[(3 * sym_b(s) + sym_a(s)) * g.N + id], v);
                }
            }
}

// Global trilinear gathers of E (nodes) and B (cells), out of line for the
// staged kernel, where a particle outside its tile cannot occur after a sort.
// The grid in and the six components out by value: an address taken of the
// caller's arrays would send their every store to the stack.
template <typename T>
struct EB6 {
    T e[3], b[3];
};
template <typename T>
__device__ __noinline__ EB6<T> gather_eb_global(const GridP g, int i, int j, int k, T ox, T oy, T oz,
                                                const T* __restrict__ E, const T* __restrict__ B) {
    EB6<T> r;
    gather_node<T, T>(g, i, j, k, ox, oy, oz, E, r.e);
    gather_cell<T, T>(g, i, j, k, ox, oy, oz, B, r.b);
    return r;
}

// E and B come in the particle precision (FP32 copies for the FP32 path:
// no FP64 conversion per gather).  kStaged: E and B staged in shared memory
// next to the accumulators (right after a sort, h = 0); a separate
// instantiation keeps the hot loop's code small.
template <typename T, typename A, bool kStaged>
__global__ void __launch_bounds__(imp_threads<T>(), 2) k_implicit_deposit_tile(GridP g, TileGeom t, ImpBlock bk,
                                                                       ImpSpecies<T> S, const T* __restrict__ E,
                                                                       const T* __restrict__ B,
                                                                       double* __restrict__ J, double* __restrict__ mu,
                                                                       double* __restrict__ rho,
                                                                       double* __restrict__ Pi) {
    extern __shared__ __align__(16) unsigned char imp_smem[];
    A* sN = reinterpret_cast<A*>(imp_smem);   // [12][NB]
    A* sC = sN + 12 * bk.NB;                  // [7][CB]
    T* sE = reinterpret_cast<T*>(sC + 7 * bk.CB);   // [3][NB] when staged
    T* sB = sE + 3 * bk.NB;                          // [3][CB] when staged
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int T3 = t.tx * t.ty * t.tz;
    const int ntiles = t.ntx * t.nty * t.ntz;
    const double PI_D = 3.14159265358979323846;
    const double ivol = 1.0 / (g.dx * g.dy * g.dz);
    const bool ax = g.nx > 1, ay = g.y3, az = g.z3;
    const int hx = ax ? bk.h : 0, hy = ay ? bk.h : 0, hz = az ? bk.h : 0;
    const int nsy = bk.nbx, nsz = bk.nbx * bk.nby;
    const int csy = bk.cbx, csz = bk.cbx * bk.cby;
    const int oxn = ax ? 1 : 0, oyn = ay ? nsy : 0, ozn = az ? nsz : 0;   // corner strides
    const int oxc = ax ? 1 : 0, oyc = ay ? csy : 0, ozc = az ? csz : 0;   // slot strides
    const int tot = 12 * bk.NB + 7 * bk.CB;
    constexpr bool kTc = sizeof(A) == sizeof(float);   // FP32 accumulators: tensor-core run sums
    float* scr0 = reinterpret_cast<float*>(imp_smem + (size_t)tot * sizeof(A) +
                                           (kStaged ? (size_t)3 * (bk.NB + bk.CB) * sizeof(T) : 0));
    float* scr = scr0 + warp * (kScrParticles * kScrRow);
    // the lane table of tc_run_sums follows the scratch rows of all warps
    TcLane* s_lane = reinterpret_cast<TcLane*>(scr0 + nwarps * (kScrParticles * kScrRow));
    if (kTc && threadIdx.x < 32) s_lane[threadIdx.x] = tc_lane(threadIdx.x);

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int ti = tile % t.ntx, tj = (tile / t.ntx) % t.nty, tk = tile / (t.ntx * t.nty);
        const int x0 = ti * t.tx, y0 = tj * t.ty, z0 = tk * t.tz;
        for (int e = threadIdx.x; e < tot; e += blockDim.x) sN[e] = A(0);
        if (kStaged) {   // with h = 0 the blocks cover exactly the stencils of the tile's own cells
            for (int e = threadIdx.x; e < bk.NB; e += blockDim.x) {
                const int lx = e % bk.nbx, ly = (e / bk.nbx) % bk.nby, lz = e / (bk.nbx * bk.nby);
                const long long id = linw(g, x0 + lx, y0 + ly, z0 + lz);
#pragma unroll
                for (int c = 0; c < 3; ++c) sE[c * bk.NB + e] = E[c * g.N + id];
            }
            for (int e = threadIdx.x; e < bk.CB; e += blockDim.x) {
                const int lx = e % bk.cbx, ly = (e / bk.cbx) % bk.cby, lz = e / (bk.cbx * bk.cby);
                const long long id = linw(g, x0 - (ax ? 1 : 0) + lx, y0 - (ay ? 1 : 0) + ly, z0 - (az ? 1 : 0) + lz);
#pragma unroll
                for (int c = 0; c < 3; ++c) sB[c * bk.CB + e] = B[c * g.N + id];
            }
        }
        __syncthreads();
        for (int s = 0; s < S.ns; ++s) {
            const PartView<T> p = S.p[s];
            const int* __restrict__ off = S.off[s];
            const double qs = S.q[s], ms = S.m[s], ws = S.w[s];
            const T beta = T(0.5 * qs * g.dt / ms);
            const double cq = qs * ws * ivol;
            const double cm = -(ws * g.theta * g.dt * g.dt * 2 * PI_D * qs * qs / ms) * ivol;
            for (int lc = warp; lc < T3; lc += nwarps) {
                const int kk = tile * T3 + lc;
                const int b0 = off[kk], b1 = off[kk + 1];
                // Right after a sort the particles of this key lie in the key's cell:
                // the tensor-core sums of all its chunks accumulate and reach the
                // block once.
                constexpr bool kCellAcc = kStaged && kTc;
                float an[4] = {0.f, 0.f, 0.f, 0.f}, ac[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                bool acc_any = false;
                int nbK = 0, cbK = 0;
                if constexpr (kCellAcc) {
                    const int li = lc % t.tx, lj = (lc / t.tx) % t.ty, lk = lc / (t.tx * t.ty);
                    nbK = (lk + hz) * nsz + (lj + hy) * nsy + (li + hx);
                    cbK = (lk + hz) * csz + (lj + hy) * csy + (li + hx);
                }
                for (int c0 = b0; c0 < b1; c0 += 32) {
                    const int n = c0 + lane;
                    const bool valid = n < b1;
                    // raw quantities: rv (3), alpha (9), node weights x/y/z (2 each), cell weights x/y/z (3 each)
                    T row[kScrRow];
#pragma unroll
                    for (int f = 0; f < kScrRow; ++f) row[f] = T(0);
                    int cell = -1, nb = 0, cb = 0;
                    bool inb = false;
                    if (valid) {
                        cell = p.cell[n];
                        int i, j, k;
                        decode(g, cell, i, j, k);
                        const T ox = p.ox[n], oy = p.oy[n], oz = p.oz[n];
                        T mom[3] = {p.px[n], p.py[n], p.pz[n]};
                        T gam, v[3];
                        gamma_vel<T>(mom, T(ms), gam, v);
                        T* nw = row + 12;
                        T* cw = row + 18;
                        axis_weights<T>(ox, ax, nw, cw);
                        axis_weights<T>(oy, ay, nw + 2, cw + 3);
                        axis_weights<T>(oz, az, nw + 4, cw + 6);
                        int li = 0, lj = 0, lk = 0;
                        inb = local_axis(i, x0, t.tx, hx, g.nx, li) && local_axis(j, y0, t.ty, hy, g.ny, lj) &&
                              local_axis(k, z0, t.tz, hz, g.nz, lk);
                        if (inb) {
                            nb = (lk + hz) * nsz + (lj + hy) * nsy + (li + hx);
                            cb = (lk + hz) * csz + (lj + hy) * csy + (li + hx);
                        }
                        T e[3], bf[3];
                        if (kStaged && inb) {
                            // node pair (c, c+1); cell pair (c-1, c) below the centre, (c, c+1) above
                            const int cbase = cb + (ox < T(0.5) ? 0 : oxc) + (oy < T(0.5) ? 0 : oyc) + (oz < T(0.5) ? 0 : ozc);
                            const T ux = ox < T(0.5) ? cw[1] : cw[2];
                            const T uy = oy < T(0.5) ? cw[4] : cw[5];
                            const T uz = oz < T(0.5) ? cw[7] : cw[8];
#pragma unroll
                            for (int c = 0; c < 3; ++c) {
                                e[c] = tri_block<T>(sE + c * bk.NB, nb, oxn, oyn, ozn, nw[1], nw[3], nw[5]);
                                bf[c] = tri_block<T>(sB + c * bk.CB, cbase, oxc, oyc, ozc, ux, uy, uz);
                            }
                        } else if (kStaged) {
                            const EB6<T> r = gather_eb_global<T>(g, i, j, k, ox, oy, oz, E, B);
#pragma unroll
                            for (int c = 0; c < 3; ++c) { e[c] = r.e[c]; bf[c] = r.b[c]; }
                        } else {
                            gather_node<T, T>(g, i, j, k, ox, oy, oz, E, e);
                            gather_cell<T, T>(g, i, j, k, ox, oy, oz, B, bf);
                        }
                        T al[9];
                        alpha_tensor<T>(beta, v, gam, e, bf, al);
                        const T vg[3] = {v[0] * gam, v[1] * gam, v[2] * gam};
#pragma unroll
                        for (int a = 0; a < 3; ++a) row[a] = al[3 * a] * vg[0] + al[3 * a + 1] * vg[1] + al[3 * a + 2] * vg[2];
#pragma unroll
                        for (int d = 0; d < 9; ++d) row[3 + d] = al[d];
                        if (!inb) {
                            A QN[12], QC[7];
                            run_quantities<A, T>(row, cq, cm, QN, QC);
                            double qn[12], qc[7];
#pragma unroll
                            for (int d = 0; d < 12; ++d) qn[d] = double(QN[d]);
#pragma unroll
                            for (int d = 0; d < 7; ++d) qc[d] = double(QC[d]);
                            imp_deposit_global<T>(g, i, j, k, ox, oy, oz, qn, qc, J, mu, rho, Pi);
                        }
                    }
                    unsigned pending = __ballot_sync(0xffffffffu, valid && inb);
                    if constexpr (kCellAcc) {
                        const bool mine = valid && inb && nb == nbK;
                        const unsigned mm = __ballot_sync(0xffffffffu, mine);
                        if (mm) {
                            tc_run_sums(scr, lane, mine, mm, row, an, ac, s_lane[lane]);
                            acc_any = true;
                        }
                        pending &= ~mm;
                    }
                    while (pending) {
                        const int leader = __ffs(pending) - 1;
                        const int lcell = __shfl_sync(0xffffffffu, cell, leader);
                        const bool me = ((pending >> lane) & 1u) && cell == lcell;
                        const unsigned mem = __ballot_sync(0xffffffffu, me);
                        pending &= ~mem;
                        if (__popc(mem) >= (kTc ? kTcMin : kXposeMin)) {
                            const int nbL = __shfl_sync(0xffffffffu, nb, leader);
                            const int cbL = __shfl_sync(0xffffffffu, cb, leader);
                            if constexpr (kTc) {
                                float dn[4] = {0.f, 0.f, 0.f, 0.f}, dc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                                tc_run_sums(scr, lane, me, mem, row, dn, dc, s_lane[lane]);
                                add_run_sums(sN, sC, bk.NB, bk.CB, nbL, cbL, oxn, oyn, ozn, oxc, oyc, ozc, lane, dn, dc,
                                             float(cq), float(cm));
                            } else {
                                A QN[12], QC[7], wn[8], wc[27];
                                run_quantities<A, T>(row, cq, cm, QN, QC);
                                run_weights<A, T>(row, wn, wc);
                                A vv[32];
#pragma unroll
                                for (int r = 0; r < 3; ++r) {
#pragma unroll
                                    for (int x = 0; x < 32; ++x) vv[x] = me ? QN[4 * r + x / 8] * wn[x % 8] : A(0);
                                    const A sum = xpose_sum<A>(vv, lane);
                                    const int q = 4 * r + lane / 8, c = lane % 8;
                                    if (sum != A(0))
                                        atomicAdd(&sN[q * bk.NB + nbL + (c & 1) * oxn + ((c >> 1) & 1) * oyn + (c >> 2) * ozn],
                                                  sum);
                                }
#pragma unroll
                                for (int r = 0; r < 6; ++r) {
#pragma unroll
                                    for (int x = 0; x < 32; ++x) {
                                        const int idx = 32 * r + x;
                                        vv[x] = (idx < 189 && me) ? QC[idx / 27] * wc[idx % 27] : A(0);
                                    }
                                    const A sum = xpose_sum<A>(vv, lane);
                                    const int idx = 32 * r + lane;
                                    if (idx < 189 && sum != A(0)) {
                                        const int q = idx / 27, sl = idx % 27;
                                        atomicAdd(&sC[q * bk.CB + cbL + (sl % 3) * oxc + ((sl / 3) % 3) * oyc + (sl / 9) * ozc],
                                                  sum);
                                    }
                                }
                            }
                        } else if (me) {
                            imp_deposit_direct<A, T>(row, cq, cm, sN, sC, bk.NB, bk.CB, nb, cb, oxn, oyn, ozn, oxc, oyc, ozc);
                        }
                    }
                }
                if constexpr (kCellAcc) {
                    if (acc_any)
                        add_run_sums(sN, sC, bk.NB, bk.CB, nbK, cbK, oxn, oyn, ozn, oxc, oyc, ozc, lane, an, ac, float(cq),
                                     float(cm));
                }
            }
        }
        __syncthreads();
        // flush the block into the FP64 grids
        for (int e = threadIdx.x; e < bk.NB; e += blockDim.x) {
            const int lx = e % bk.nbx, ly = (e / bk.nbx) % bk.nby, lz = e / (bk.nbx * bk.nby);
            const long long id = linw(g, x0 - hx + lx, y0 - hy + ly, z0 - hz + lz);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const A v = sN[d * bk.NB + e];
                if (v != A(0)) atomicAdd(&J[d * g.N + id], double(v));
            }
#pragma unroll
            for (int d = 0; d < 9; ++d) {
                const A v = sN[(3 + d) * bk.NB + e];
                if (v != A(0)) atomicAdd(&mu[d * g.N + id], double(v));
            }
        }
        for (int e = threadIdx.x; e < bk.CB; e += blockDim.x) {
            const int lx = e % bk.cbx, ly = (e / bk.cbx) % bk.cby, lz = e / (bk.cbx * bk.cby);
            const long long id = linw(g, x0 - hx - (ax ? 1 : 0) + lx, y0 - hy - (ay ? 1 : 0) + ly,
                                      z0 - hz - (az ? 1 : 0) + lz);
            const A r = sC[e];
            if (r != A(0)) atomicAdd(&rho[id], double(r));
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const A v = sC[(1 + q) * bk.CB + e];
                if (v == A(0)) continue;
                atomicAdd(&Pi[(3 * sym_a(q) + sym_b(q)) * g.N + id], double(v));
                if (sym_a(q) != sym_b(q)) atomicAdd(&Pi[(3 * sym_b(q) + sym_a(q)) * g.N + id], double(v));
            }
        }
        __syncthreads();
    }
}

}  // namespace pic

namespace pic {

constexpr int kMoverHalo = 2;   // cells of field halo staged around a mover tile

// Field blocks of the tiled mover: nodes (E^n, E^theta) over tile + 2H + 1,
// cells (B^n) over tile + 2H + 2 on active axes.
struct MoverBlock {
    int nbx, nby, nbz, NB;
    int cbx, cby, cbz, CB;
};

// moveParticle (PIC++/mover.cpp:194-491), one CTA per tile of tile-ordered
// particles: E^n and E^{n+theta} (nodes) and B^n (cells) of the tile and a
// two-cell halo are staged in shared memory in the particle precision, so
// the predictor and the up to three Picard gathers read shared memory.  A
// particle with a position whose stencil leaves the block is left untouched
// and its bit set in S.defer: k_implicit_push_deferred moves it from the
// FP64 grids (the kernel itself calls nothing out of line, which would cost
// its hot loop register spills).  Same arithmetic as k_implicit_push.
template <typename T, bool kWall>
__global__ void __launch_bounds__(kMoverThreads, 2) k_implicit_push_tile(GridP g, TileGeom t, MoverBlock mb, ImpSpecies<T> S,
                                                            const double* __restrict__ E, const double* __restrict__ B,
                                                            const double* __restrict__ Et) {
    extern __shared__ __align__(16) unsigned char mv_smem[];
    // FP32: E^theta and B^n, gathered two or three times per particle, as
    // float4 nodes / cells (one 16-byte load per corner); E^n, gathered
    // once, as three scalar planes.  FP64: three scalar planes each.
    constexpr bool kVec = sizeof(T) == sizeof(float);
    float4* sEt4 = reinterpret_cast<float4*>(mv_smem);   // [NB] (FP32)
    float4* sB4 = sEt4 + mb.NB;                           // [CB] (FP32)
    T* sE = kVec ? reinterpret_cast<T*>(sB4 + mb.CB) : reinterpret_cast<T*>(mv_smem);   // [3][NB]
    T* sEt = sE + 3 * mb.NB;                 // [3][NB] (FP64)
    T* sB = sEt + 3 * mb.NB;                 // [3][CB] (FP64)
    // after the field blocks: every thread's next particle, copied with
    // cp.async while it moves the current one ([6][threads] values, then
    // [threads] cells)
    const size_t fld = kVec ? ((size_t)mb.NB + mb.CB) * 16 + 3 * (size_t)mb.NB * sizeof(float)
                            : (6 * (size_t)mb.NB + 3 * (size_t)mb.CB) * sizeof(T);
    T* sPre = reinterpret_cast<T*>(mv_smem + ((fld + 15) & ~size_t(15)));
    int* sPreCell = reinterpret_cast<int*>(sPre + 6 * blockDim.x);
    auto stage = [&](const PartView<T>& pv, int m) {
        const int me = threadIdx.x, bdim = blockDim.x;
        cp_async<4>(&sPreCell[me], pv.cell + m);
        cp_async<sizeof(T)>(&sPre[0 * bdim + me], pv.ox + m);
        cp_async<sizeof(T)>(&sPre[1 * bdim + me], pv.oy + m);
        cp_async<sizeof(T)>(&sPre[2 * bdim + me], pv.oz + m);
        cp_async<sizeof(T)>(&sPre[3 * bdim + me], pv.px + m);
        cp_async<sizeof(T)>(&sPre[4 * bdim + me], pv.py + m);
        cp_async<sizeof(T)>(&sPre[5 * bdim + me], pv.pz + m);
    };
    const int ntiles = t.ntx * t.nty * t.ntz;
    const int T3 = t.tx * t.ty * t.tz;
    const bool ax = g.nx > 1, ay = g.y3, az = g.z3;
    const int hx = ax ? kMoverHalo : 0, hy = ay ? kMoverHalo : 0, hz = az ? kMoverHalo : 0;
    const int nsx = ax ? 1 : 0, nsy = ay ? mb.nbx : 0, nsz = az ? mb.nbx * mb.nby : 0;
    const int csx = ax ? 1 : 0, csy = ay ? mb.cbx : 0, csz = az ? mb.cbx * mb.cby : 0;
    const T dt = T(g.dt), eta = T(g.eta), edt = T(g.eta * g.dt);
    const T id[3] = {T(g.idx), T(g.idy), T(g.idz)};
    const int nn[3] = {g.nx, g.ny, g.nz};
    const T dxT = T(g.dx);
    const T redt = T((1.0 - g.eta) * g.dt);
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int ti = tile % t.ntx, tj = (tile / t.ntx) % t.nty, tk = tile / (t.ntx * t.nty);
        const int x0 = ti * t.tx, y0 = tj * t.ty, z0 = tk * t.tz;
        __syncthreads();   // previous tile's particles are done with the blocks
        for (int e = threadIdx.x; e < mb.NB; e += blockDim.x) {
            const int lx = e % mb.nbx, ly = (e / mb.nbx) % mb.nby, lz = e / (mb.nbx * mb.nby);
            const long long gid = linw(g, x0 - hx + lx, y0 - hy + ly, z0 - hz + lz);
#pragma unroll
            for (int c = 0; c < 3; ++c) sE[c * mb.NB + e] = T(E[c * g.N + gid]);
            if constexpr (kVec) {
                sEt4[e] = make_float4(float(Et[gid]), float(Et[g.N + gid]), float(Et[2 * g.N + gid]), 0.f);
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c) sEt[c * mb.NB + e] = T(Et[c * g.N + gid]);
            }
        }
        for (int e = threadIdx.x; e < mb.CB; e += blockDim.x) {
            const int lx = e % mb.cbx, ly = (e / mb.cbx) % mb.cby, lz = e / (mb.cbx * mb.cby);
            const long long gid = linw(g, x0 - hx - (ax ? 1 : 0) + lx, y0 - hy - (ay ? 1 : 0) + ly,
                                       z0 - hz - (az ? 1 : 0) + lz);
            if constexpr (kVec) {
                sB4[e] = make_float4(float(B[gid]), float(B[g.N + gid]), float(B[2 * g.N + gid]), 0.f);
            } else {
#pragma unroll
                for (int c = 0; c < 3; ++c) sB[c * mb.CB + e] = T(B[c * g.N + gid]);
            }
        }
        __syncthreads();
        for (int s = 0; s < S.ns; ++s) {
            const PartView<T> p = S.p[s];
            const double qs = S.q[s], ms = S.m[s];
            const T beta = T(0.5 * qs * g.dt / ms);
            const T qdt = T(qs * g.dt);
            const T mm = T(ms);
            const int b0 = S.off[s][tile * T3], b1 = S.off[s][(tile + 1) * T3];
            if (b0 + (int)threadIdx.x < b1) stage(p, b0 + threadIdx.x);
            cp_async_commit();
            for (int n = b0 + threadIdx.x; n < b1; n += blockDim.x) {
                cp_async_wait_all();   // this thread's particle n (its own slot)
                const int bdim = blockDim.x, me = threadIdx.x;
                const int cell_n = sPreCell[me];
                const T pu[3] = {sPre[0 * bdim + me], sPre[1 * bdim + me], sPre[2 * bdim + me]};
                const T pm[3] = {sPre[3 * bdim + me], sPre[4 * bdim + me], sPre[5 * bdim + me]};
                if (n + bdim < b1) stage(p, n + bdim);
                cp_async_commit();
                int ci[3];
                decode(g, cell_n, ci[0], ci[1], ci[2]);
                // A position (cell c, offset u) is located once: its node and cell
                // stencils in the staged block (bases, upper weights), shared by the
                // two or three gathers there; a stencil that leaves the block
                // gathers from the FP64 grids.
                struct Loc {
                    bool inb;
                    int nbase, cbase;
                    T wn[3], wc[3];
                };
                // from tile-local cells l (the block holds l in [-h, t - 1 + h])
                auto locate_l = [&](const int l[3], const T u[3], Loc& L) {
                    L.inb = l[0] >= -hx && l[0] <= t.tx - 1 + hx && l[1] >= -hy && l[1] <= t.ty - 1 + hy &&
                            l[2] >= -hz && l[2] <= t.tz - 1 + hz;
                    if (!L.inb) return;
                    int lo[3];
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        T w2[2];
                        int idx[2];
                        node_w<T>(u[a], l[a], nn[a], idx, w2);
                        L.wn[a] = w2[1];
                        cell_w<T>(u[a], l[a], nn[a], idx, w2);
                        L.wc[a] = w2[1];
                        // lower cell of the pair: c - 1 below the centre, c above
                        lo[a] = (nn[a] > 1 && u[a] < T(0.5)) ? l[a] - 1 : l[a];
                    }
                    L.nbase = (l[2] + hz) * nsz + (l[1] + hy) * nsy + (l[0] + hx) * nsx;
                    const int ex = ax ? 1 : 0, ey = ay ? 1 : 0, ez = az ? 1 : 0;
                    L.cbase = (lo[2] + hz + ez) * csz + (lo[1] + hy + ey) * csy + (lo[0] + hx + ex) * csx;
                };
                // from global cells c: the periodic image inside the block, if any
                auto locate = [&](const int c[3], const T u[3], Loc& L, int l[3]) {
                    if (!(local_axis(c[0], x0, t.tx, hx, g.nx, l[0]) && local_axis(c[1], y0, t.ty, hy, g.ny, l[1]) &&
                          local_axis(c[2], z0, t.tz, hz, g.nz, l[2]))) {
                        L.inb = false;
                        return;
                    }
                    locate_l(l, u, L);
                };
                // gathers at a located position inside the block
                auto gat = [&](const Loc& L, const T* __restrict__ blkN, bool node, T out[3]) {
                    if (node) {
#pragma unroll
                        for (int q = 0; q < 3; ++q)
                            out[q] = tri_block<T>(blkN + q * mb.NB, L.nbase, nsx, nsy, nsz, L.wn[0], L.wn[1], L.wn[2]);
                    } else {
#pragma unroll
                        for (int q = 0; q < 3; ++q)
                            out[q] = tri_block<T>(blkN + q * mb.CB, L.cbase, csx, csy, csz, L.wc[0], L.wc[1], L.wc[2]);
                    }
                };
                // E^theta (node) and B^n (cell): float4 blocks for FP32
                auto gatEt = [&](const Loc& L, T out[3]) {
                    if constexpr (kVec) tri_block4(sEt4, L.nbase, nsx, nsy, nsz, L.wn[0], L.wn[1], L.wn[2], out);
                    else gat(L, sEt, true, out);
                };
                auto gatB = [&](const Loc& L, T out[3]) {
                    if constexpr (kVec) tri_block4(sB4, L.cbase, csx, csy, csz, L.wc[0], L.wc[1], L.wc[2], out);
                    else gat(L, sB, false, out);
                };
                auto defer = [&]() { atomicOr(&S.defer[s][n >> 5], 1u << (n & 31)); };
                T u0[3] = {pu[0], pu[1], pu[2]};
                T mom0[3] = {pm[0], pm[1], pm[2]};
                T gam, v[3];
                gamma_vel<T>(mom0, mm, gam, v);
                T e[3], b[3], al[9];
                Loc L0;
                int l0[3];
                locate(ci, u0, L0, l0);
                if (!L0.inb) {
                    defer();
                    continue;
                }
                gat(L0, sE, true, e);
                gatB(L0, b);
                alpha_tensor<T>(beta, v, gam, e, b, al);
                gatEt(L0, e);
                T vxb[3] = {v[1] * b[2] - v[2] * b[1], -v[0] * b[2] + v[2] * b[0], v[0] * b[1] - v[1] * b[0]};
                T pnew[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) pnew[d] = mom0[d] + (e[d] + vxb[d]) * qdt;
                T vnew[3];
                evaluate_velocity<T>(pnew, mm, vnew);
                T mv[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) mv[d] = v[d] * (T(1) - eta) + vnew[d] * eta;
                if constexpr (kWall) {
                    if (wall_left_of<T>(ci[0], u0[0], (mv[0] * edt) * id[0])) {
                        wall_reflect_trial<T>(g, ci, u0, mv, vnew, mm, edt, redt, id, pnew);
                        p.px[n] = pnew[0]; p.py[n] = pnew[1]; p.pz[n] = pnew[2];
                        p.ox[n] = u0[0]; p.oy[n] = u0[1]; p.oz[n] = u0[2];
                        p.cell[n] = (int)lin(g, ci[0], ci[1], ci[2]);
                        continue;
                    }
                }
                T vh[3];
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    vh[a] = (al[3 * a] * gam) * v[0] + (al[3 * a + 1] * gam) * v[1] + (al[3 * a + 2] * gam) * v[2];
                const T momNorm = picard_norm<T>(mom0[0] * mom0[0] + mom0[1] * mom0[1] + mom0[2] * mom0[2]);
                T err = picard_norm<T>((mom0[0] - pnew[0]) * (mom0[0] - pnew[0]) + (mom0[1] - pnew[1]) * (mom0[1] - pnew[1]) +
                                 (mom0[2] - pnew[2]) * (mom0[2] - pnew[2]));
                const T dxN = picard_ref<T>(dxT);
                T cerr = dxN;
                T newDisp[3] = {mv[0] * edt, mv[1] * edt, mv[2] * edt};
                T prevDisp[3];
                int it = 0;
                bool reflected = false, left = false;
                while (picard_continue<T>(err, momNorm, cerr, dxN, it)) {
                    ++it;
                    const T prevMom[3] = {pnew[0], pnew[1], pnew[2]};
#pragma unroll
                    for (int d = 0; d < 3; ++d) prevDisp[d] = newDisp[d];
                    T re[3];
#pragma unroll
                    for (int a = 0; a < 3; ++a) re[a] = al[3 * a] * e[0] + al[3 * a + 1] * e[1] + al[3 * a + 2] * e[2];
#pragma unroll
                    for (int d = 0; d < 3; ++d) mv[d] = vh[d] + re[d] * beta;
#pragma unroll
                    for (int d = 0; d < 3; ++d) newDisp[d] = mv[d] * edt;
                    if constexpr (kWall) {
                        if (wall_left_of<T>(ci[0], u0[0], newDisp[0] * id[0])) {
                            wall_reflect_trial<T>(g, ci, u0, mv, vnew, mm, edt, redt, id, pnew);
                            reflected = true;
                            break;
                        }
                    }
                    // the trial position x^n + newDisp: the offsets as advance_axis
                    // forms them, the cell in tile-local terms (no periodic wrap)
                    T tu[3];
                    int tl[3];
                    Loc L1;
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const T sd = u0[d] + newDisp[d] * id[d];
                        const T fd = dev_floor(sd);
                        T ud = sd - fd;
                        int cd = l0[d] + (int)fd;
                        if (ud >= T(1)) { ud -= T(1); cd += 1; }
                        tl[d] = nn[d] > 1 ? cd : 0;
                        tu[d] = ud;
                    }
                    locate_l(tl, tu, L1);
                    if (!L1.inb) {
                        left = true;
                        break;
                    }
                    gatEt(L1, e);
                    gatB(L1, b);
                    const T mvxb[3] = {mv[1] * b[2] - mv[2] * b[1], -mv[0] * b[2] + mv[2] * b[0], mv[0] * b[1] - mv[1] * b[0]};
#pragma unroll
                    for (int d = 0; d < 3; ++d) pnew[d] = mom0[d] + (e[d] + mvxb[d]) * qdt;
                    err = picard_norm<T>((prevMom[0] - pnew[0]) * (prevMom[0] - pnew[0]) +
                                   (prevMom[1] - pnew[1]) * (prevMom[1] - pnew[1]) +
                                   (prevMom[2] - pnew[2]) * (prevMom[2] - pnew[2]));
                    cerr = picard_norm<T>((prevDisp[0] - newDisp[0]) * (prevDisp[0] - newDisp[0]) +
                                    (prevDisp[1] - newDisp[1]) * (prevDisp[1] - newDisp[1]) +
                                    (prevDisp[2] - newDisp[2]) * (prevDisp[2] - newDisp[2]));
                }
                if (left) {   // nothing written yet: the deferred pass moves it from the start
                    defer();
                    continue;
                }
                if (!reflected) {
                    if constexpr (kWall) {
                        const int o = wall_final_x<T>(g, ci[0], u0[0], (mv[0] * dt) * id[0]);
                        if (o == 2) { p.cell[n] = -1; continue; }   // escaped through the open boundary
                        if (o == 1) pnew[0] = -pnew[0];
#pragma unroll
                        for (int d = 1; d < 3; ++d) advance_axis<T>(u0[d], ci[d], (mv[d] * dt) * id[d], nn[d]);
                    } else {
#pragma unroll
                        for (int d = 0; d < 3; ++d) advance_axis<T>(u0[d], ci[d], (mv[d] * dt) * id[d], nn[d]);
                    }
                }
                p.px[n] = pnew[0]; p.py[n] = pnew[1]; p.pz[n] = pnew[2];
                p.ox[n] = u0[0]; p.oy[n] = u0[1]; p.oz[n] = u0[2];
                p.cell[n] = (int)lin(g, ci[0], ci[1], ci[2]);
            }
        }
    }
}

}  // namespace pic
