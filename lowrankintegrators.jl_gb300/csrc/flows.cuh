// flows.cuh - build-time registry of the local flow maps of the instance
// engine.
//
// The reference accepts any flow map F(Y, t) as a Julia closure and evaluates
// it on the factored operand (src/integrators/unconventional.jl:51-79, the
// K_rhs / L_rhs / S_rhs hooks of :2-4,16-21).  A GPU engine cannot call host
// closures.  Flow maps that act column by column through a periodic
// three-point stencil along the rows,
//
//     F(Y)_ij = f(Y_{i-1,j}, Y_ij, Y_{i+1,j}, c_j; h, p0, p1),
//
// are instead functors registered here when the library is built.  The
// engine evaluates them tile by tile on Y = K V^T (flow_contract in
// engine.cuh) for the K, L and S substeps, without forming the n x m matrix.
//
// Adding a flow map:
//   1. write a struct with
//        template <typename T>
//        __device__ static T eval(T ym, T y0, T yp, T c, T ih2, T ihx, T p0, T p1);
//      (ym, y0, yp: Y at rows i-1, i, i+1 of column j, periodic; c: the
//      column's parameter c_j from operator B; ih2 = 1/h^2, ihx = 1/(2h);
//      p0, p1: the batch's two scalars.  T is float, double or the
//      double-float pair: use +, -, * and fma only);
//   2. append it to LRI_LOCAL_FLOWS with the next id and a name;
//   3. rebuild.  The op LRI_OP_LOCAL_FLOW with lri_batch_desc.flow = id
//      selects it; lri_flow_count / lri_flow_name list the registry.
#pragma once

#include <cuda_runtime.h>

namespace lri {

// F = (Dxx Y) diag(c) + p0 (Dx Y) .* Y + p1 Dx(Y .* Y): the periodic Burgers
// flow (c = viscosity per column; the reference test's form is p0 = -1,
// p1 = 0, test/data_agnostic_approximation.jl:16-33; the conservative form
// p0 = 0, p1 = -1/2).  Also the engine's LRI_OP_BURGERS_PERIODIC.
struct BurgersFlow {
  template <typename T>
  __device__ __forceinline__ static T eval(T ym, T y0, T yp, T c, T ih2, T ihx, T p0, T p1) {
    T f = c * (((ym + yp) - (y0 + y0)) * ih2);
    f = fma(p0 * ((yp - ym) * ihx), y0, f);
    return fma(p1, (yp * yp - ym * ym) * ihx, f);
  }
};

// F = (Dxx Y) diag(c) + p0 Y + p1 Y.^3: reaction-diffusion (Allen-Cahn for
// c = eps^2, p0 = 1, p1 = -1; linear diffusion with decay for p1 = 0).
struct ReactionDiffusionFlow {
  template <typename T>
  __device__ __forceinline__ static T eval(T ym, T y0, T yp, T c, T ih2, T ihx, T p0, T p1) {
    (void)ihx;
    T f = c * (((ym + yp) - (y0 + y0)) * ih2);
    f = fma(p0, y0, f);
    return fma(p1 * y0, y0 * y0, f);
  }
};

// id, functor, name
#define LRI_LOCAL_FLOWS(X)       \
  X(0, BurgersFlow, "burgers") \
  X(1, ReactionDiffusionFlow, "reaction_diffusion")

constexpr int kLocalFlowCount = 2;

// Calls f(Functor{}) for the registered flow `id` (nothing for an unknown id).
template <typename F>
__device__ __forceinline__ void with_local_flow(int id, F&& f) {
  switch (id) {
#define LRI_FLOW_CASE(ID, TYPE, NAME) \
  case ID:                            \
    f(TYPE{});                        \
    break;
    LRI_LOCAL_FLOWS(LRI_FLOW_CASE)
#undef LRI_FLOW_CASE
    default:
      break;
  }
}

}  // namespace lri
