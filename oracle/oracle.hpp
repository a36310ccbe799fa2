// ORACLE -- test infrastructure only.  A CPU restatement (FP64, no FMA
// contraction: built with -ffp-contract=off) of the reference Fortran routines
// of freeCappuccino's per-iteration path, statement order preserved, so that
// the GPU library can be checked against it.  Nothing in the product links or
// calls this code; only tests/, the smoke check and the CPU-baseline leg of
// bench.py do.
//
// Parity status: the reference is Fortran and no Fortran compiler exists in
// the build container, so the reference itself cannot be run; this
// restatement is pinned by the reference's own known-answer programs
// (test/test_linear_solvers_spsolve.f90 5x5 systems,
// test/testFieldOperations linear-field gradient on its 20x20x1 polyMesh)
// and by the properties its code guarantees (see tests/).
//
// Arrays inside the oracle are 1-based: every vector has a dummy element 0 so
// that loops read exactly like the Fortran.  (3,n) arrays are stored as
// g[3*i + k-1], k = 1..3.
#pragma once
#include <string>
#include <vector>

namespace orc {

// Single-precision literals of the reference promoted to double
// (parameters.f90:6 small=1e-20, linear_solvers.f90:238,447 s0=1.e20).
static const double kSmall = (double)1e-20f;
static const double kS0 = (double)1.e20f;
static const double kTiny30 = (double)1e-30f;   // interpolation.f90:556 (+1e-30)

enum { BC_WALL = 1, BC_INLET = 2, BC_OUTLET = 3, BC_SYMMETRY = 4, BC_PRESSURE = 5, BC_EMPTY = 6, BC_PERIODIC = 7 };

// settings of one turbulence scalar (TurbModelData.f90 TurbScalar; the
// default tolAbs 1e-10 is a default-real literal)
struct TurbScalar {
  double urf = 0.7, gds = 1.0;
  int cScheme = 2;  // linearUpwind
  std::string lSolver = "bicgstab";
  int maxiter = 10;
  double tolAbs = (double)1e-10f, tolRel = 0.01;
};

struct Case {
  // sizes (geometry.f90:17-24)
  int numNodes = 0, numCells = 0, numInnerFaces = 0, numBoundaryFaces = 0, numFaces = 0, numTotal = 0;
  int numBoundaries = 0;
  std::vector<int> bctype, nfaces, startFace, iBndValueStart;  // 1-based per boundary
  int nwal = 0, nsym = 0;
  // periodic pairs (geometry.f90:24, :82, :250-258): nper pairs, numPeriodic
  // faces on the 'periodic' sides, startFaceTwin(iPer) 1-based by pair
  int nper = 0, numPeriodic = 0;
  std::vector<int> startFaceTwin;
  // mesh (1-based)
  std::vector<double> x, y, z;
  std::vector<int> nnodes, node;  // node[(iface)*6 + k] k=1..6 -> stored at node[iface*6 + k-1]
  std::vector<int> owner, neighbour;
  // geometry
  std::vector<double> arx, ary, arz, xf, yf, zf, xc, yc, zc, vol, facint, Df;
  std::vector<double> dns, srds, dnw, srdw;
  // CSR (sparse_matrix.f90:10-18), 1-based values
  int nnz = 0;
  std::vector<int> ia, ja, diag, ijk, jik;
  // matrix / sources (sparse_matrix.f90:21-25)
  std::vector<double> a, su, sv, sw, spu, spv, sp, apu, apv, apw;
  // fields (variables.f90)
  std::vector<double> u, v, w, p, pp, flmass, vis, den, visw;
  std::vector<double> dUdxi, dVdxi, dWdxi, dPdxi;  // 3*(numTotal+1)
  std::vector<double> Dmat;                        // 9*(numCells+1)  (gradients.f90:12)
  int dmatScheme = 0;                              // gradient scheme Dmat was built for (0: none)
  // solver work vectors (linear_solvers.f90:33)
  std::vector<double> res, reso, pk, zk, d, uk, vk;
  // parameters of the SIMPLE path
  int gradScheme = 0;  // 0 gauss, 1 lstsq, 2 lstsq_dm
  int limiter = 0;     // gradients.f90:13: 0 none, 1 Barth-Jespersen, 2 Venkatakrishnan, 3 'R3', 4 multidimensional
  // node_interpolation.f90: c2n 0 'psl' (pseudo-Laplacian, the default), 1 'ids' (inverse distance)
  int c2n = 0;
  // transient momentum and PISO (velocity.f90:133-290, :565-570;
  // calcp_piso.f90; time_shift.f90): tscheme 0 steady, 1 bdf (Euler),
  // 2 bdf2, 3 bdf3
  int tscheme = 0, piso = 0, ncorr = 1;
  double timestep = 1.0;
  std::vector<double> uo, vo, wo, uoo, voo, woo, uooo, vooo, wooo;  // numTotal+1
  std::vector<double> rU, rV, rW;                                   // numCells+1
  std::vector<double> h;                                            // nnz+1
  std::vector<double> wCellToNode, wFaceToNode;  // 1-based, in the module's running order
  int pscheme = 0;     // 0 linear, 1 central, 2 weighted
  double densit = 1.0, viscos = 0.01;
  double urfU[3] = {0.8, 0.8, 0.8}, gdsU = 1.0, urfP = 0.3;
  int cSchemeU = 1;    // interpolation scheme id (see face_value)
  int maxiterU = 5, maxiterP = 20, npcor = 1, pRefCell = 1;
  double tolAbsU = 1e-15, tolRelU = 0.01, tolAbsP = 1e-15, tolRelP = 0.025;
  std::string lSolverU = "bicgstab", lSolverP = "iccg";
  double resor[13] = {0};
  double cumulativeContErr = 0.0;
  // temperature transport (ScalarEqns/temperature.f90:15-25, parameters.f90:30)
  std::vector<double> T, dTdxi;        // numTotal+1, 3*(numTotal+1)
  std::vector<double> bcDFracT;        // bcDFraction(7,ib), 1-based per boundary
  double pranl = 0.7, sigt = 1.0, urfT = 0.9, gdsT = 1.0;
  int cSchemeT = 2;                    // interpolation scheme id (linearUpwind)
  int maxiterT = 10;
  double tolAbsT = 1e-13, tolRelT = 0.02;
  std::string lSolverT = "bicgstab";
  double flomas = 0.0;
  int verbose = 0;
  // k-omega SST (k_omega_SST.f90, calc_strain_and_vorticity.f90,
  // wall_distance.f90): te = k, ed = omega
  std::vector<double> te, ed, fsst;         // numTotal+1
  std::vector<double> dTEdxi, dEDdxi;       // 3*(numTotal+1)
  std::vector<double> gen, magStrain, walldist;  // numCells+1
  std::vector<double> tau, ypl;             // nwal+1
  TurbScalar turbK, turbW;                  // TurbModel%Scalar(1), (2)
  double urfVis = 1.0;                      // TurbModel%urfVis
};

inline double& G(std::vector<double>& g, int k, int i) { return g[3 * (size_t)i + (k - 1)]; }

// mesh + geometry + CSR
// twin: per patch, the 0-based startFace of a 'periodic' patch's twin (the
// fifth field of its boundary-file line), ignored for other patches; NULL
// when the mesh has no periodic patches
void setup_case(Case& c, int numNodes, int numCells, int numInnerFaces, int numBoundaryFaces,
                const double* x, const double* y, const double* z, const int* nnodes, const int* nodes,
                const int* owner, const int* neighbour, int numBoundaries, const int* bctype,
                const int* nfaces, const int* startFace, const int* twin = nullptr);
void geometry(Case& c);
void face_mapping(Case& c);
void create_csr(Case& c);

// linear solvers (linear_solvers.f90); arrays 1-based raw pointers
struct SolveInfo { int itr_used = 0; double res0 = 0, resl = 0, factor = 0, resor = 0; int early = 0; };
void gauss_seidel(int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag, double* fi,
                  const double* rhs, double& resor, int itr_max, double tol_abs, double tol_rel, double* res,
                  SolveInfo& si);
void dpcg(int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag, double* fi,
          const double* rhs, double& resor, int itr_max, double tol_abs, double tol_rel, double* res, double* pk,
          double* zk, SolveInfo& si);
void iccg(int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag, double* fi,
          const double* rhs, double& resor, int itr_max, double tol_abs, double tol_rel, double* res, double* pk,
          double* zk, double* d, SolveInfo& si);
void bicgstab(int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag, double* fi,
              const double* rhs, double& resor, int itr_max, double tol_abs, double tol_rel, double* res,
              double* reso, double* pk, double* uk, double* zk, double* vk, double* d, SolveInfo& si);
int pmgmres_ilu(int n, int nz_num, const int* ia, const int* ja, const double* a, int* ua, double* x,
                const double* rhs, double& resor, int itr_max, int mr, double tol_abs, double tol_rel, SolveInfo& si);
void dic_setup(int n, const int* ia, const int* ja, const double* a, const int* diag, double* d);
void dilu_setup(int n, const int* ia, const int* ja, const double* a, const int* diag, double* d);
void diag_precond_apply(int n, const int* ia, const int* ja, const double* a, const int* diag, const double* d,
                        const double* r, double* z);
void ax_cr(int n, const int* ia, const int* ja, const double* a, const double* x, double* w);
void atx_cr(int n, const int* ia, const int* ja, const double* a, const double* x, double* w);
int ilu_cr(int n, const int* ia, const int* ja, const double* a, int* ua, double* l);
void lus_cr(int n, const int* ia, const int* ja, const double* l, const int* ua, const double* r, double* z);
int csrsolve(Case& c, const std::string& solver, std::vector<double>& fi, const std::vector<double>& rhs,
             double& res0, int itr_max, double tol_abs, double tol_rel, SolveInfo& si);

// gradients (gradients.f90)
void grad_gauss(Case& c, const std::vector<double>& u, std::vector<double>& dudxi);
void create_matrix_lsq(Case& c);
void grad_lsq(Case& c, const std::vector<double>& phi, std::vector<double>& dphidxi, bool exact = false);
void create_matrix_lsq_dm(Case& c);
void grad_lsq_dm(Case& c, const std::vector<double>& phi, std::vector<double>& dphidxi, bool exact = false);
// least-squares matrix of a gradient scheme: 1 (LSQ, LSQ exact), 2 (LSQ_DM, LSQ_DM exact), 0 none
inline int lsq_matrix_of(int scheme) { return scheme == 1 || scheme == 4 ? 1 : scheme == 2 || scheme == 5 ? 2 : 0; }
void prepare_lsq(Case& c, int scheme);
void grad_scheme(Case& c, int scheme, const std::vector<double>& phi, std::vector<double>& dphidxi);
void grad(Case& c, const std::vector<double>& phi, std::vector<double>& dphidxi);
void slope_limiter(Case& c, const std::vector<double>& phi, std::vector<double>& dphidxi);
void set_interpolation_weights(Case& c);
void interpolate_to_nodes(Case& c, const std::vector<double>& phiC, std::vector<double>& phiN);
void grad_node_based_gauss(Case& c, const std::vector<double>& u, std::vector<double>& dudxi);
void time_shift(Case& c);
int calcp_piso(Case& c);

// operators
void laplacian(Case& c, const std::vector<double>& mu, const std::vector<double>& phi, unsigned long long dirichlet_mask);

// SIMPLE path
void gradp_and_sources(Case& c, std::vector<double>& p);
void bpres(Case& c, std::vector<double>& p, int istage);
void updateVelocityAtBoundary(Case& c);
void updateBoundary(Case& c, std::vector<double>& phi);
// scalar face fluxes (scalar_fluxes.f90), shared by the temperature and the
// turbulence equations
void facefluxsc(Case& c, int i, int ijp, int ijn, double xf, double yf, double zf, double arx, double ary, double arz,
                double fm, double lambda, double gam, int scheme, const std::vector<double>& fi,
                std::vector<double>& dfidxi, double dcoef, double& cap, double& can, double& suadd);
void facefluxsc_bnd(Case& c, int ijp, double xf, double yf, double zf, double arx, double ary, double arz, double fm,
                    std::vector<double>& dfidxi, double dcoef, double& cap, double& can, double& suadd);
void facefluxsc_periodic(Case& c, int i, int ijp, int ijn, double xf, double yf, double zf, double arx, double ary,
                         double arz, double fm, double gam, const std::vector<double>& fi,
                         std::vector<double>& dfidxi, double dcoef, double& cap, double& can, double& suadd);
// k-omega SST (oracle_turb.cpp)
int wall_distance_poisson(Case& c);
void calc_strain(Case& c);
int calcsc_sst(Case& c, int ifi);
void modify_mu_eff_sst(Case& c);
int modify_viscosity_k_omega_sst(Case& c);
void init_flmass(Case& c);
int calcuvw(Case& c);
int calcp_simple(Case& c);
// calculate_temperature (ScalarEqns/temperature.f90:35-385), steady, no
// turbulence: assemble (a, su), solve, update boundaries, clip.  With
// solve == false only the assembly (through the under-relaxation) is done.
int calculate_temperature(Case& c, bool solve);
void continuityErrors(Case& c);
// Steady convection-diffusion of a passive scalar with the implicit part of
// facefluxsc (scalar_fluxes.f90:32-141, :256-337): upwind convection,
// diffusion gamma_f Df with gamma_f = gamma_P (1 - facint) + gamma_N facint,
// phi = 0 on every boundary face (sp += gamma_P |S|^2 / (d.S)), main
// diagonal = sp - sum of the row's off-diagonals (temperature.f90:359-361).
// a <- A, su <- source * vol.  gamma, source: 1-based, numCells.
void cd_assemble(Case& c, const std::vector<double>& gamma, const std::vector<double>& source);
// dJ/dgamma_c = -lambda^T (dA/dgamma_c) phi, the reverse face loop of
// cd_assemble: out (1-based, numCells)
void cd_gradient(Case& c, const std::vector<double>& phi, const std::vector<double>& lambda, std::vector<double>& out);
double face_value(Case& c, int ijp, int ijn, double xf, double yf, double zf, double lambda,
                  const std::vector<double>& u, std::vector<double>& dUdxi, int scheme);

}  // namespace orc
