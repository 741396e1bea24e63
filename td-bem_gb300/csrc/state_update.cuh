// The state update of one dof after a solve step (SolverT::ExtractField's placement,
// SolverT.cpp:396-409): the displacement history takes the prescribed value or the
// unknown, the traction history the prescribed traction times the load amplitude
// (0 where none), or the unknown where the displacement is prescribed, except at the
// last dof, whose prescribed traction stays (ExtractField's loop stops one short).
#pragma once

#include "tdbem_internal.cuh"

namespace tdbem {

__device__ __forceinline__ void update_state_dof(const StateUpdate& p, int D, int j, double x) {
    const bool u = p.is_u[j] != 0, f = p.is_f[j] != 0;
    p.u_hist[(size_t)p.s * D + j] = u ? p.ubc[j] : x;
    double tv = f ? p.fbc[j] * p.amp : 0.0;
    if (u && j < D - 1) tv = x;
    p.t_hist[(size_t)p.s * D + j] = tv;
}

}  // namespace tdbem
