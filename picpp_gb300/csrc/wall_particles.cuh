// wall_particles.cuh -- the implicit movers' rules at a conductor wall at
// x = 0 and an open boundary at x = (nx - 2) dx (the box layout is described
// in wall.cuh).
#pragma once
#include "common.cuh"

namespace pic {

// Particle::setMomentumByV (particle.cpp:337-364): m v below v^2 < 1e-4
// (relativisticPrecision, constants.h:39), m gamma(v) v above.
template <typename T>
__device__ __forceinline__ void momentum_by_v(const T v[3], T m, T p[3]) {
    const T v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const T f = v2 < T(1e-4) ? m : m / dev_sqrt(T(1) - v2);
#pragma unroll
    for (int d = 0; d < 3; ++d) p[d] = v[d] * f;
}

// True when x^n + disp (disp in cells along x) lies left of the wall; c, u
// the cell and offset of x^n.  Exact in the offset arithmetic: only the
// cell shift is compared.
template <typename T>
__device__ __forceinline__ bool wall_left_of(int c, T u, T disp) {
    return c + (int)dev_floor(u + disp) < 0;
}

// Cell and offset of a position x >= 0 given in cells.
template <typename T>
__device__ __forceinline__ void wall_set_x(T X, int& c, T& u) {
    const T f = dev_floor(X);
    c = (int)f;
    u = X - f;
    if (u >= T(1)) { u -= T(1); c += 1; }
}

// The reflection of moveParticle at the wall from a trial position
// (mover.cpp:247-260 after the predictor, 312-330 in the Picard loop):
// x = -(x^n + eta dt vbar_x) + |vbar_x| (1 - eta) dt, y and z carried on by
// vbar (1 - eta) dt after eta dt, momentum from the predictor's velocity
// with |v_x|.  ci, u: cell and offset of x^n on entry, of the result on
// return.
template <typename T>
__device__ __forceinline__ void wall_reflect_trial(const GridP& g, int ci[3], T u[3], const T mv[3], const T vnew[3],
                                                   T m, T edt, T redt, const T id[3], T pout[3]) {
    const int nn[3] = {g.nx, g.ny, g.nz};
    const T X = -(T(ci[0]) + u[0] + (mv[0] * edt) * id[0]) + fabs(mv[0] * redt) * id[0];
    wall_set_x<T>(X, ci[0], u[0]);
#pragma unroll
    for (int d = 1; d < 3; ++d) {
        advance_axis<T>(u[d], ci[d], (mv[d] * edt) * id[d], nn[d]);
        advance_axis<T>(u[d], ci[d], (mv[d] * redt) * id[d], nn[d]);
    }
    const T vr[3] = {fabs(vnew[0]), vnew[1], vnew[2]};
    momentum_by_v<T>(vr, m, pout);
}

// The final x move x^{n+1} = x^n + dt vbar_x next to the wall
// (mover.cpp:435-458): returns 0 inside (c, u advanced), 1 mirrored at the
// wall (c, u set; p_x is to be reversed, reflectMomentumX), 2 escaped
// through the open boundary.
template <typename T>
__device__ __forceinline__ int wall_final_x(const GridP& g, int& c, T& u, T disp) {
    const T s = u + disp;
    const T fl = dev_floor(s);
    int cn = c + (int)fl;
    T un = s - fl;
    if (un >= T(1)) { un -= T(1); cn += 1; }
    if (cn < 0) {
        wall_set_x<T>(-(T(c) + s), c, u);
        return 1;
    }
    if (cn > g.nx - 2 || (cn == g.nx - 2 && un > T(0))) return 2;
    c = cn;
    u = un;
    return 0;
}

// The x move of moveParticleTristan in a wall box (mover.cpp:744-772),
// reflecting at node kTristanWallNode:
// x^{n+1} = x^n + disp (disp in cells) without a periodic wrap; a position
// left of the reflecting wall is mirrored there (bit 1 of the result: p_x
// is to be reversed, reflectMomentumX); a position beyond the open boundary
// x = (nx - 2) dx sets bit 2 (escaped: the particle deposits its current
// this step, then leaves).  c, u: cell and offset of x^n on entry, of the
// result on return.
template <typename T>
__device__ __forceinline__ int tristan_wall_x(const GridP& g, int& c, T& u, T disp) {
    const int W = kTristanWallNode;
    const T s = u + disp;
    const T fl = dev_floor(s);
    int cn = c + (int)fl;
    T un = s - fl;
    if (un >= T(1)) { un -= T(1); cn += 1; }
    int r = 0;
    if (cn < W) {   // x' = 2 W - x
        if (un > T(0)) { cn = 2 * W - cn - 1; un = T(1) - un; }
        else cn = 2 * W - cn;
        r = 1;
    }
    if (cn > g.nx - 2 || (cn == g.nx - 2 && un > T(0))) r |= 2;
    c = cn;
    u = un;
    return r;
}

// True for a particle that left a wall box through the open boundary: its
// position lies beyond x = (nx - 2) dx (the ghost column).
template <typename T>
__device__ __forceinline__ bool tristan_escaped(const GridP& g, int i, T u) {
    return i > g.nx - 2 || (i == g.nx - 2 && u > T(0));
}

}  // namespace pic
