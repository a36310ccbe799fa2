// Field storage of a context (variables.f90 / sparse_matrix.f90 globals).
#pragma once
#include <string>
#include <vector>

#include "fc_internal.hpp"

struct FieldSlot {
  std::string name;
  DVec<double>* vec = nullptr;
  size_t n = 0;
  int kind = 0;  // 0 plain, 1 gradient (SoA on device, (3,n) at the boundary), 2 internal
};

struct FieldStore {
  DVec<double> u, v, w, p, pp, vis, den, t, flmass, visw;
  DVec<double> su, sv, sw, spu, spv, sp, apu, apv, apw;
  DVec<double> gu, gv, gw, gp, gt;  // gradients, SoA [3][numTotal]
  DVec<double> uo, vo, wo, uoo, voo, woo, uooo, vooo, wooo;  // old time levels (numTotal)
  DVec<double> rU, rV, rW;          // PISO: explicit momentum terms (numCells)
  // k-omega SST: k, omega, blending function F1 (numTotal), their gradients
  // (SoA), production, strain magnitude, wall distance (numCells), wall shear
  // stress and y+ (per wall face)
  DVec<double> te, ed, fsst, gte, ged, gen, mag, wd, tau, ypl;
  DVec<double> fscratch, cscratch, cscratch_big;
  DVec<double> dmat;                // least-squares cofactors, SoA [9][numCells]
  int dmat_scheme = 0;              // scheme the cofactors were built for (0: none)
  std::vector<FieldSlot> list;
};

FieldStore& ctx_fields(fc_ctx* ctx);
FieldSlot* find_field(fc_ctx* ctx, const std::string& name);
void fc_fields_release(fc_ctx* ctx);
