// Shared view of the device mesh for the finite-volume kernels, and the
// exact-rounding FP64 shorthands they use to reproduce the reference's
// operation order without FMA contraction.
#pragma once
#include <cuda_runtime.h>

#include "fc_internal.hpp"

#define DM __dmul_rn
#define DA __dadd_rn
#define DS __dsub_rn
#define DD __ddiv_rn

namespace fcfv {

struct MeshView {
  int nC, nI, nB, nF, nT;
  const int* __restrict__ owner;
  const int* __restrict__ neighbour;
  const int* __restrict__ cf_ptr;
  const int* __restrict__ cf_face;
  const int* __restrict__ bpatch;
  const int* __restrict__ bwall;
  const double* __restrict__ srdw;
  const double* __restrict__ dnw;
  const double* __restrict__ arx;
  const double* __restrict__ ary;
  const double* __restrict__ arz;
  const double* __restrict__ xf;
  const double* __restrict__ yf;
  const double* __restrict__ zf;
  const double* __restrict__ xc;
  const double* __restrict__ yc;
  const double* __restrict__ zc;
  const double* __restrict__ vol;
  const double* __restrict__ facint;
  const double* __restrict__ Df;
  const int* __restrict__ ijk;
  const int* __restrict__ jik;
  // periodic pairs (MeshDev): nIP = nI + nPer indexes pair q as slot-map
  // entry nI + q
  int nPer, nIP;
  const int* __restrict__ pface;
  const int* __restrict__ ptwin;
  const int* __restrict__ ppos;
  const int* __restrict__ pflag;
  const int* __restrict__ bpair;
  const int* __restrict__ af_ptr;
  const int* __restrict__ af_ent;
  const int* __restrict__ diag;
  const int* __restrict__ ia;
};

}  // namespace fcfv

fcfv::MeshView mesh_view(fc_ctx* ctx);
int fv_grad(fc_ctx* ctx, int scheme, const double* phi, double* g);
// the context's slope limiter applied to the SoA gradient g of phi (fc_limiter.cu)
int fv_limit(fc_ctx* ctx, const double* phi, double* g);
// node-based Gauss gradient of phi into the SoA g (fc_nodegrad.cu)
int fv_grad_node(fc_ctx* ctx, const double* phi, double* g);
// grad_gauss without the limiter (fc_fv.cu)
int fv_grad_gauss(fc_ctx* ctx, const double* phi, double* g);
