// ORACLE (test infrastructure only) -- C entry points used through ctypes by
// tests/, the smoke check and the CPU-baseline leg of bench.py.  Arrays cross
// this boundary 0-based in memory holding the reference's 1-based index
// values, exactly as a Fortran caller would pass them.
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "oracle.hpp"

using namespace orc;

namespace {

std::vector<double>* dbl_array(Case& c, const std::string& n, int& len, int& offset, int& stride) {
  offset = 1; stride = 1;
  if (n == "arx") { len = c.numFaces; return &c.arx; }
  if (n == "ary") { len = c.numFaces; return &c.ary; }
  if (n == "arz") { len = c.numFaces; return &c.arz; }
  if (n == "xf") { len = c.numFaces; return &c.xf; }
  if (n == "yf") { len = c.numFaces; return &c.yf; }
  if (n == "zf") { len = c.numFaces; return &c.zf; }
  if (n == "xc") { len = c.numCells; return &c.xc; }
  if (n == "yc") { len = c.numCells; return &c.yc; }
  if (n == "zc") { len = c.numCells; return &c.zc; }
  if (n == "vol") { len = c.numCells; return &c.vol; }
  if (n == "facint") { len = c.numInnerFaces; return &c.facint; }
  if (n == "Df") { len = c.numInnerFaces; return &c.Df; }
  if (n == "dnw") { len = c.nwal; return &c.dnw; }
  if (n == "srdw") { len = c.nwal; return &c.srdw; }
  if (n == "dns") { len = c.nsym; return &c.dns; }
  if (n == "srds") { len = c.nsym; return &c.srds; }
  if (n == "a") { len = c.nnz; return &c.a; }
  if (n == "su") { len = c.numCells; return &c.su; }
  if (n == "sv") { len = c.numCells; return &c.sv; }
  if (n == "sw") { len = c.numCells; return &c.sw; }
  if (n == "spu") { len = c.numCells; return &c.spu; }
  if (n == "spv") { len = c.numCells; return &c.spv; }
  if (n == "sp") { len = c.numCells; return &c.sp; }
  if (n == "apu") { len = c.numCells; return &c.apu; }
  if (n == "apv") { len = c.numCells; return &c.apv; }
  if (n == "apw") { len = c.numCells; return &c.apw; }
  if (n == "u") { len = c.numTotal; return &c.u; }
  if (n == "v") { len = c.numTotal; return &c.v; }
  if (n == "w") { len = c.numTotal; return &c.w; }
  if (n == "p") { len = c.numTotal; return &c.p; }
  if (n == "pp") { len = c.numTotal; return &c.pp; }
  if (n == "vis") { len = c.numTotal; return &c.vis; }
  if (n == "den") { len = c.numTotal; return &c.den; }
  if (n == "t") { len = c.numTotal; return &c.T; }
  if (n == "dTdxi") { len = 3 * c.numTotal; offset = 3; return &c.dTdxi; }
  if (n == "flmass") { len = c.numFaces; return &c.flmass; }
  if (n == "visw") { len = c.nwal; return &c.visw; }
  if (n == "d") { len = c.numCells; return &c.d; }
  if (n == "dUdxi") { len = 3 * c.numTotal; offset = 3; return &c.dUdxi; }
  if (n == "dVdxi") { len = 3 * c.numTotal; offset = 3; return &c.dVdxi; }
  if (n == "dWdxi") { len = 3 * c.numTotal; offset = 3; return &c.dWdxi; }
  if (n == "dPdxi") { len = 3 * c.numTotal; offset = 3; return &c.dPdxi; }
  if (n == "Dmat") { len = 9 * c.numCells; offset = 9; return &c.Dmat; }
  if (n == "te") { len = c.numTotal; return &c.te; }
  if (n == "ed") { len = c.numTotal; return &c.ed; }
  if (n == "fsst") { len = c.numTotal; return &c.fsst; }
  if (n == "dTEdxi") { len = 3 * c.numTotal; offset = 3; return &c.dTEdxi; }
  if (n == "dEDdxi") { len = 3 * c.numTotal; offset = 3; return &c.dEDdxi; }
  if (n == "gen") { len = c.numCells; return &c.gen; }
  if (n == "magStrain") { len = c.numCells; return &c.magStrain; }
  if (n == "walldist") { len = c.numCells; return &c.walldist; }
  if (n == "tau") { len = c.nwal; return &c.tau; }
  if (n == "ypl") { len = c.nwal; return &c.ypl; }
  if (n == "uo") { len = c.numTotal; return &c.uo; }
  if (n == "vo") { len = c.numTotal; return &c.vo; }
  if (n == "wo") { len = c.numTotal; return &c.wo; }
  if (n == "uoo") { len = c.numTotal; return &c.uoo; }
  if (n == "voo") { len = c.numTotal; return &c.voo; }
  if (n == "woo") { len = c.numTotal; return &c.woo; }
  if (n == "uooo") { len = c.numTotal; return &c.uooo; }
  if (n == "vooo") { len = c.numTotal; return &c.vooo; }
  if (n == "wooo") { len = c.numTotal; return &c.wooo; }
  if (n == "rU") { len = c.numCells; return &c.rU; }
  if (n == "rV") { len = c.numCells; return &c.rV; }
  if (n == "rW") { len = c.numCells; return &c.rW; }
  return nullptr;
}

std::vector<int>* int_array(Case& c, const std::string& n, int& len) {
  if (n == "ia") { len = c.numCells + 1; return &c.ia; }
  if (n == "ja") { len = c.nnz; return &c.ja; }
  if (n == "diag") { len = c.numCells; return &c.diag; }
  if (n == "ijk") { len = c.numInnerFaces + c.numPeriodic; return &c.ijk; }
  if (n == "jik") { len = c.numInnerFaces + c.numPeriodic; return &c.jik; }
  if (n == "owner") { len = c.numFaces; return &c.owner; }
  if (n == "neighbour") { len = c.numInnerFaces; return &c.neighbour; }
  return nullptr;
}

template <class T>
std::vector<T> pad1(const T* p, int n) {
  std::vector<T> v(n + 1);
  if (n > 0) std::memcpy(v.data() + 1, p, sizeof(T) * n);
  return v;
}

}  // namespace

extern "C" {

void* orc_case_new(int numNodes, int numCells, int numInnerFaces, int numBoundaryFaces, const double* x,
                   const double* y, const double* z, const int* nnodes, const int* nodes, const int* owner,
                   const int* neighbour, int numBoundaries, const int* bctype, const int* nfaces,
                   const int* startFace, const int* twin) {
  Case* c = new Case();
  setup_case(*c, numNodes, numCells, numInnerFaces, numBoundaryFaces, x, y, z, nnodes, nodes, owner, neighbour,
             numBoundaries, bctype, nfaces, startFace, twin);
  return c;
}

void orc_case_free(void* h) { delete (Case*)h; }

// out[9] = numCells, numInnerFaces, numBoundaryFaces, numFaces, numTotal, nnz, nwal, nsym, numPeriodic
int orc_case_sizes(void* h, int* out) {
  Case& c = *(Case*)h;
  out[0] = c.numCells; out[1] = c.numInnerFaces; out[2] = c.numBoundaryFaces; out[3] = c.numFaces;
  out[4] = c.numTotal; out[5] = c.nnz; out[6] = c.nwal; out[7] = c.nsym; out[8] = c.numPeriodic;
  return 0;
}

int orc_case_get(void* h, const char* name, double* out) {
  Case& c = *(Case*)h;
  int len, off, st;
  std::vector<double>* v = dbl_array(c, name, len, off, st);
  if (!v) return -1;
  if ((int)v->size() < len + off) return -1;
  std::memcpy(out, v->data() + off, sizeof(double) * len);
  return len;
}

int orc_case_set(void* h, const char* name, const double* in) {
  Case& c = *(Case*)h;
  int len, off, st;
  std::vector<double>* v = dbl_array(c, name, len, off, st);
  if (!v) return -1;
  if ((int)v->size() < len + off) v->resize(len + off, 0.0);
  std::memcpy(v->data() + off, in, sizeof(double) * len);
  return len;
}

int orc_case_get_int(void* h, const char* name, int* out) {
  Case& c = *(Case*)h;
  int len;
  std::vector<int>* v = int_array(c, name, len);
  if (!v) return -1;
  std::memcpy(out, v->data() + 1, sizeof(int) * len);
  return len;
}

int orc_case_set_param(void* h, const char* name, double val) {
  Case& c = *(Case*)h;
  std::string n(name);
  if (n == "densit") c.densit = val;
  else if (n == "viscos") c.viscos = val;
  else if (n == "urfU1") c.urfU[0] = val;
  else if (n == "urfU2") c.urfU[1] = val;
  else if (n == "urfU3") c.urfU[2] = val;
  else if (n == "gdsU") c.gdsU = val;
  else if (n == "urfP") c.urfP = val;
  else if (n == "cSchemeU") c.cSchemeU = (int)val;
  else if (n == "gradScheme") c.gradScheme = (int)val;
  else if (n == "pscheme") c.pscheme = (int)val;
  else if (n == "limiter") c.limiter = (int)val;
  else if (n == "tscheme") c.tscheme = (int)val;
  else if (n == "piso") c.piso = (int)val;
  else if (n == "ncorr") c.ncorr = (int)val;
  else if (n == "timestep") c.timestep = val;
  else if (n == "c2n") { c.c2n = (int)val; c.wCellToNode.clear(); c.wFaceToNode.clear(); }
  else if (n == "maxiterU") c.maxiterU = (int)val;
  else if (n == "maxiterP") c.maxiterP = (int)val;
  else if (n == "npcor") c.npcor = (int)val;
  else if (n == "pRefCell") c.pRefCell = (int)val;
  else if (n == "tolAbsU") c.tolAbsU = val;
  else if (n == "tolRelU") c.tolRelU = val;
  else if (n == "tolAbsP") c.tolAbsP = val;
  else if (n == "tolRelP") c.tolRelP = val;
  else if (n == "flomas") c.flomas = val;
  else if (n == "pranl") c.pranl = val;
  else if (n == "sigt") c.sigt = val;
  else if (n == "urfT") c.urfT = val;
  else if (n == "gdsT") c.gdsT = val;
  else if (n == "cSchemeT") c.cSchemeT = (int)val;
  else if (n == "maxiterT") c.maxiterT = (int)val;
  else if (n == "tolAbsT") c.tolAbsT = val;
  else if (n == "tolRelT") c.tolRelT = val;
  else if (n == "urfVis") c.urfVis = val;
  else if (n.size() > 1 && (n.back() == 'K' || n.back() == 'W') && n.compare(0, n.size() - 1, "urf") == 0)
    (n.back() == 'K' ? c.turbK : c.turbW).urf = val;
  else if (n == "gdsK" || n == "gdsW") (n.back() == 'K' ? c.turbK : c.turbW).gds = val;
  else if (n == "cSchemeK" || n == "cSchemeW") (n.back() == 'K' ? c.turbK : c.turbW).cScheme = (int)val;
  else if (n == "maxiterK" || n == "maxiterW") (n.back() == 'K' ? c.turbK : c.turbW).maxiter = (int)val;
  else if (n == "tolAbsK" || n == "tolAbsW") (n.back() == 'K' ? c.turbK : c.turbW).tolAbs = val;
  else if (n == "tolRelK" || n == "tolRelW") (n.back() == 'K' ? c.turbK : c.turbW).tolRel = val;
  else return -1;
  return 0;
}

int orc_case_set_solver(void* h, const char* which, const char* solver) {
  Case& c = *(Case*)h;
  if (std::string(which) == "U") c.lSolverU = solver;
  else if (std::string(which) == "P") c.lSolverP = solver;
  else if (std::string(which) == "T") c.lSolverT = solver;
  else if (std::string(which) == "K") c.turbK.lSolver = solver;
  else if (std::string(which) == "W") c.turbW.lSolver = solver;
  else return -1;
  return 0;
}

// bcDFraction(7, ib) of the temperature equation, ib 1-based
int orc_case_set_bcdfrac_t(void* h, int ib, double val) {
  Case& c = *(Case*)h;
  if (ib < 1 || ib > c.numBoundaries) return -1;
  c.bcDFracT[ib] = val;
  return 0;
}

double orc_case_get_scalar(void* h, const char* name) {
  Case& c = *(Case*)h;
  std::string n(name);
  if (n.size() == 6 && n.compare(0, 5, "resor") == 0) return c.resor[n[5] - '0'];
  if (n == "cumulativeContErr") return c.cumulativeContErr;
  return 0.0;
}

// scheme: 0 gauss, 1 lstsq, 2 lstsq_dm, 3 node-based Gauss.  phi: numTotal; dphi: 3*numTotal
int orc_grad(void* h, int scheme, double* phi, double* dphi) {
  Case& c = *(Case*)h;
  std::vector<double> p = pad1(phi, c.numTotal);
  std::vector<double> g(3 * (size_t)(c.numTotal + 1), 0.0);
  grad_scheme(c, scheme, p, g);
  slope_limiter(c, p, g);
  std::memcpy(dphi, g.data() + 3, sizeof(double) * 3 * c.numTotal);
  return 0;
}

int orc_prepare_lsq(void* h, int scheme) {
  Case& c = *(Case*)h;
  c.gradScheme = scheme;
  if (lsq_matrix_of(scheme) == 1) create_matrix_lsq(c);
  else if (lsq_matrix_of(scheme) == 2) create_matrix_lsq_dm(c);
  return 0;
}

// a <- laplacian matrix, su accumulated (the caller sets su beforehand)
int orc_laplacian(void* h, const double* mu, const double* phi, unsigned long long mask) {
  Case& c = *(Case*)h;
  std::vector<double> m = pad1(mu, c.numCells), p = pad1(phi, c.numTotal);
  laplacian(c, m, p, mask);
  return 0;
}

int orc_gradp_and_sources(void* h, int which_pp) {
  Case& c = *(Case*)h;
  gradp_and_sources(c, which_pp ? c.pp : c.p);
  return 0;
}

int orc_init_flmass(void* h) { init_flmass(*(Case*)h); return 0; }
int orc_update_velocity_at_boundary(void* h) { updateVelocityAtBoundary(*(Case*)h); return 0; }
int orc_calcuvw(void* h) { return calcuvw(*(Case*)h); }
int orc_calcp_simple(void* h) { return calcp_simple(*(Case*)h); }
int orc_calculate_temperature(void* h, int solve) { return calculate_temperature(*(Case*)h, solve != 0); }
int orc_wall_distance(void* h) { return wall_distance_poisson(*(Case*)h); }
int orc_calc_strain(void* h) { calc_strain(*(Case*)h); return 0; }
int orc_calcsc_sst(void* h, int ifi) { return calcsc_sst(*(Case*)h, ifi); }
int orc_modify_mu_eff_sst(void* h) { modify_mu_eff_sst(*(Case*)h); return 0; }
int orc_kw_sst(void* h) { return modify_viscosity_k_omega_sst(*(Case*)h); }

// gamma, source: numCells (0-based memory); a <- A, su <- source * vol
int orc_cd_assemble(void* h, const double* gamma, const double* source) {
  Case& c = *(Case*)h;
  cd_assemble(c, pad1(gamma, c.numCells), pad1(source, c.numCells));
  return 0;
}

// out (numCells) = dJ/dgamma for phi, lambda (numCells)
int orc_cd_gradient(void* h, const double* phi, const double* lambda, double* out) {
  Case& c = *(Case*)h;
  std::vector<double> o;
  cd_gradient(c, pad1(phi, c.numCells), pad1(lambda, c.numCells), o);
  std::memcpy(out, o.data() + 1, sizeof(double) * c.numCells);
  return 0;
}

// one SIMPLE outer iteration (main.f90:159-165); resor4 gets resor(1..4);
// elapsed_s gets the wall time of the iteration
int orc_time_shift(void* h) { time_shift(*(Case*)h); return 0; }
int orc_calcp_piso(void* h) { return calcp_piso(*(Case*)h); }

// calcuvw + calcp_piso (main.f90:159-165 with PISO)
int orc_piso_iteration(void* h, double* resor4) {
  Case& c = *(Case*)h;
  int st = calcuvw(c);
  int st2 = calcp_piso(c);
  if (resor4) for (int k = 0; k < 4; ++k) resor4[k] = c.resor[k + 1];
  return st < st2 ? st : st2;
}

int orc_simple_iteration(void* h, double* resor4, double* elapsed_s) {
  Case& c = *(Case*)h;
  auto t0 = std::chrono::steady_clock::now();
  int st = calcuvw(c);
  int st2 = calcp_simple(c);
  auto t1 = std::chrono::steady_clock::now();
  if (resor4) for (int k = 0; k < 4; ++k) resor4[k] = c.resor[k + 1];
  if (elapsed_s) *elapsed_s = std::chrono::duration<double>(t1 - t0).count();
  return st < st2 ? st : st2;
}

// Standalone solvers on caller arrays (1-based index values).
// info[0]=itr_used, info[1]=res0 (L1), info[2]=final resl, info[3]=factor
int orc_solve(const char* solver, int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag,
              double* fi, const double* rhs, double* res0, int itr_max, double tol_abs, double tol_rel,
              double* info) {
  std::vector<int> IA = pad1(ia, n + 1), JA = pad1(ja, nnz), DG = pad1(diag, n);
  std::vector<double> A = pad1(a, nnz), X = pad1(fi, n), B = pad1(rhs, n);
  std::vector<double> r(n + 1), ro(n + 1), p(n + 1), u(n + 1), z(n + 1), v(n + 1), d(n + 1);
  SolveInfo si;
  double resor = res0 ? *res0 : 0.0;
  std::string s(solver);
  int st = 0;
  if (s == "gauss-seidel") gauss_seidel(n, nnz, IA.data(), JA.data(), A.data(), DG.data(), X.data(), B.data(), resor, itr_max, tol_abs, tol_rel, r.data(), si);
  else if (s == "dpcg") dpcg(n, nnz, IA.data(), JA.data(), A.data(), DG.data(), X.data(), B.data(), resor, itr_max, tol_abs, tol_rel, r.data(), p.data(), z.data(), si);
  else if (s == "iccg") iccg(n, nnz, IA.data(), JA.data(), A.data(), DG.data(), X.data(), B.data(), resor, itr_max, tol_abs, tol_rel, r.data(), p.data(), z.data(), d.data(), si);
  else if (s == "bicgstab") bicgstab(n, nnz, IA.data(), JA.data(), A.data(), DG.data(), X.data(), B.data(), resor, itr_max, tol_abs, tol_rel, r.data(), ro.data(), p.data(), u.data(), z.data(), v.data(), d.data(), si);
  else if (s == "pmgmres") {
    std::vector<int> ua(DG);
    st = pmgmres_ilu(n, nnz, IA.data(), JA.data(), A.data(), ua.data(), X.data(), B.data(), resor, itr_max, 4, tol_abs, tol_rel, si);
  } else return -1;
  std::memcpy(fi, X.data() + 1, sizeof(double) * n);
  if (res0) *res0 = resor;
  if (info) { info[0] = si.itr_used; info[1] = si.res0; info[2] = si.resl; info[3] = si.factor; }
  return st;
}

int orc_dic_setup(int n, const int* ia, const int* ja, const double* a, const int* diag, double* d, int dilu) {
  int nnz = ia[n] - 1;
  std::vector<int> IA = pad1(ia, n + 1), JA = pad1(ja, nnz), DG = pad1(diag, n);
  std::vector<double> A = pad1(a, nnz), D(n + 1);
  if (dilu) dilu_setup(n, IA.data(), JA.data(), A.data(), DG.data(), D.data());
  else dic_setup(n, IA.data(), JA.data(), A.data(), DG.data(), D.data());
  std::memcpy(d, D.data() + 1, sizeof(double) * n);
  return 0;
}

int orc_precond_apply(int n, const int* ia, const int* ja, const double* a, const int* diag, const double* d,
                      const double* r, double* z) {
  int nnz = ia[n] - 1;
  std::vector<int> IA = pad1(ia, n + 1), JA = pad1(ja, nnz), DG = pad1(diag, n);
  std::vector<double> A = pad1(a, nnz), D = pad1(d, n), R = pad1(r, n), Z(n + 1);
  diag_precond_apply(n, IA.data(), JA.data(), A.data(), DG.data(), D.data(), R.data(), Z.data());
  std::memcpy(z, Z.data() + 1, sizeof(double) * n);
  return 0;
}

int orc_spmv(int n, const int* ia, const int* ja, const double* a, const double* x, double* y, int transpose) {
  int nnz = ia[n] - 1;
  std::vector<int> IA = pad1(ia, n + 1), JA = pad1(ja, nnz);
  std::vector<double> A = pad1(a, nnz), X = pad1(x, n), Y(n + 1);
  if (transpose) atx_cr(n, IA.data(), JA.data(), A.data(), X.data(), Y.data());
  else ax_cr(n, IA.data(), JA.data(), A.data(), X.data(), Y.data());
  std::memcpy(y, Y.data() + 1, sizeof(double) * n);
  return 0;
}

int orc_ilu0(int n, const int* ia, const int* ja, const double* a, const int* diag, double* l, int* ua_out) {
  int nnz = ia[n] - 1;
  std::vector<int> IA = pad1(ia, n + 1), JA = pad1(ja, nnz), UA = pad1(diag, n);
  std::vector<double> A = pad1(a, nnz), L(nnz + 2);
  int st = ilu_cr(n, IA.data(), JA.data(), A.data(), UA.data(), L.data());
  std::memcpy(l, L.data() + 1, sizeof(double) * nnz);
  if (ua_out) std::memcpy(ua_out, UA.data() + 1, sizeof(int) * n);
  return st;
}

}  // extern "C"
