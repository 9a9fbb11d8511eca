// Curved (non-affine) elements: the reference's quadrature formulation,
// element by element, for the elements whose high-order nodes leave the
// straight-sided lattice (curved.cu).
//
// Per curved element (slot s, element celem[s]), in the context's precision:
//   A    [Ng][D][D]         w_g det J(x_g) d(xi_r)/d(x_d): the stiffness
//                           integrand of Mesh.cpp:734-751 at element point g
//   Minv [Np][Np]           inverse of M = sum_g w_g det J_g phi_i phi_j
//                           (Mesh.cpp:691-724; FP64 Gauss-Jordan on the GPU)
//   F    [Nf][Ngf][D+1]     per face point: outward unit normal, w_g |J_f,g|
//                           (Mesh.cpp:209-260, :316-367, :536-568)
//   TB   [Nf][6]            3-D tangent and bitangent of the face, built from
//                           its first three quadrature points (Mesh.cpp:284-308)
// and per stage the right-hand side M^-T (S - F) of every curved element goes
// to crhs [NV][ncurved][Np]; the stage kernels take it in place of their
// affine operator result for those elements (StageArgs::cslot).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

struct dg_ctx;

namespace dgc {

// Classifies nothing itself: curved_flag [E] (device, 1 = curved) comes from
// the element-geometry pass. Builds the per-element data above and the slot
// table; returns DG_OK or a DG_ERR_* code with c->err set.
int setup_curved(dg_ctx* c, const double* xyz, const int64_t* en, const int* perm, const double* det_aff,
                 const int* curved_flag, cudaStream_t st);

// Right-hand side of every curved element from the stage input y_in (the
// context's precision) into c->crhs, on c->stream.
cudaError_t launch_curved(dg_ctx* c, const void* y_in);

}  // namespace dgc
