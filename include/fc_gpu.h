/*
 * fc_gpu.h -- C ABI of the GB300 (sm_103a) implementation of freeCappuccino's
 * per-iteration hot path: face-based flux assembly into CSR, cell gradients and
 * the built-in sparse Krylov solvers.
 *
 * Conventions shared by every entry point
 *  - Every call returns an int status: 0 = OK, >0 = warning, <0 = error
 *    (FC_* codes below).  No call aborts the process; the text of the last
 *    error of a context is returned by fc_last_error().
 *  - Index arrays handed over from the Fortran side are 1-based exactly as the
 *    reference stores them (ia, ja, diag, owner, neighbour, face nodes).
 *  - Fields follow the reference layout: numTotal = numCells+numBoundaryFaces
 *    values, cell values first, then one value per boundary face
 *    (geometry.f90:282).  Gradients are (3,numTotal) column-major, i.e. xyz
 *    interleaved per cell (variables.f90:10).
 *  - Host pointers are copied; pointers to device memory are used in place.
 *  - One fc_ctx per host thread; calls on one context are stream ordered and
 *    not thread safe.
 */
#ifndef FC_GPU_H
#define FC_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FC_OK                0
#define FC_WARN_MAXITER      1   /* solver stopped at itr_max (the reference continues silently) */
#define FC_ERR_BAD_INPUT    -1   /* invalid argument / inconsistent sizes / bad index */
#define FC_ERR_CUDA         -2   /* CUDA runtime error */
#define FC_ERR_NAN          -3   /* NaN or Inf met in a residual norm */
#define FC_ERR_BREAKDOWN    -4   /* Krylov breakdown (zero denominator) */
#define FC_ERR_TIMEOUT      -5   /* a bounded device spin-wait ran out */
#define FC_ERR_STATE        -6   /* call made in the wrong state (e.g. no mesh set) */
#define FC_ERR_UNSUPPORTED  -7   /* option not implemented */
#define FC_ERR_ZERO_PIVOT   -8   /* zero pivot in ILU(0) (ilu_cr stops the program) */
#define FC_ERR_NOMEM        -9   /* device allocation failed */

/* ---- boundary condition types (bctype strings of the native mesh) ------- */
#define FC_BC_WALL       1   /* 'wall'     */
#define FC_BC_INLET      2   /* 'inlet'    */
#define FC_BC_OUTLET     3   /* 'outlet'   */
#define FC_BC_SYMMETRY   4   /* 'symmetry' */
#define FC_BC_PRESSURE   5   /* 'pressure' */
#define FC_BC_EMPTY      6   /* 'empty'    */
#define FC_BC_PERIODIC   7   /* 'periodic': paired with an 'empty' twin patch (startFaceTwin) */

/* ======================================================================== */
/* Host-side mesh (native polyMesh format of read_mesh_native,              */
/* geometry.f90:118-410).  These calls need no GPU.                          */
/* ======================================================================== */
typedef struct fc_mesh fc_mesh;

#define FC_NOMAX 6   /* max nodes per face, geometry.f90:40 */

/* Structured nx*ny*nz hex box on [0,lx]x[0,ly]x[0,lz].  Interior vertices are
 * moved by U(-perturb*h, +perturb*h) per axis (seeded).  tets!=0 splits every
 * hex into 6 tetrahedra.  side_bctype[6] gives the FC_BC_* type of the
 * patches xmin,xmax,ymin,ymax,zmin,zmax (NULL: all walls); a FC_BC_PERIODIC
 * side is paired with the opposite side, which must be FC_BC_EMPTY.  Inner faces are
 * ordered by (owner,neighbour), owner<neighbour, area vector owner->neighbour;
 * boundary faces are grouped by patch in the order above. */
int fc_mesh_box(int nx, int ny, int nz, double lx, double ly, double lz,
                double perturb, unsigned long long seed, int tets,
                const int* side_bctype, fc_mesh** out);

/* Build from arrays in the reference's native layout (1-based owner,
 * neighbour and face nodes; nodes has FC_NOMAX entries per face; startFace is
 * the 0-based face offset of each patch as in the 'boundary' file). */
int fc_mesh_from_arrays(int numNodes, int numCells, int numInnerFaces, int numBoundaryFaces,
                        const double* x, const double* y, const double* z,
                        const int* nnodes, const int* nodes,
                        const int* owner, const int* neighbour,
                        int numBoundaries, const int* bctype, const int* nfaces,
                        const int* startFace, fc_mesh** out);

/* Periodic pairs (geometry.f90:250-258): a FC_BC_PERIODIC patch names its
 * twin by the twin's 0-based startFace (the fifth field of the patch's line
 * in the boundary file).  The twin is another patch of the same size typed
 * FC_BC_EMPTY; at most three pairs.  fc_mesh_set_twin sets it for a mesh
 * built from arrays; fc_mesh_twins gives it per patch (-1: not periodic). */
int fc_mesh_set_twin(fc_mesh* m, int patch, int startFaceTwin);
int fc_mesh_twins(const fc_mesh* m, int* startFaceTwin);

/* Read / write the native files points, faces, owner, neighbour, boundary,
 * size of a polyMesh directory (read_mesh_native, geometry.f90:165-410). */
int fc_mesh_read_native(const char* dir, fc_mesh** out);
int fc_mesh_write_native(const fc_mesh* m, const char* dir);
/* Read / write OpenFOAM-format ASCII polyMesh files (read_mesh_openfoam,
 * geometry.f90:846-1400): points, faces, owner, neighbour with FoamFile
 * headers and 0-based indices, sizes from the owner file's note line and
 * confirmed by every list; boundary in the reference's one-line-per-patch
 * format (a header line, then name type nFaces startFace) or in OpenFOAM's
 * dictionary form (type wall / symmetryPlane / symmetry / empty / cyclic
 * give the role, a generic patch takes it from its name: inlet, outlet,
 * pressure, ...).  The writer uses the reference's format. */
int fc_mesh_read_openfoam(const char* dir, fc_mesh** out);
int fc_mesh_write_openfoam(const fc_mesh* m, const char* dir);

/* info[6] = numNodes, numCells, numInnerFaces, numBoundaryFaces, numFaces, numBoundaries */
int fc_mesh_info(const fc_mesh* m, int* info);
/* Copy the mesh out (any pointer may be NULL). */
int fc_mesh_export(const fc_mesh* m, double* x, double* y, double* z,
                   int* nnodes, int* nodes, int* owner, int* neighbour,
                   int* bctype, int* nfaces, int* startFace);
void fc_mesh_free(fc_mesh* m);

/* ======================================================================== */
/* Context                                                                  */
/* ======================================================================== */
typedef struct fc_ctx fc_ctx;

#define FC_PREC_FP64   0   /* everything in FP64, as the reference */
#define FC_PREC_MIXED  1   /* FP32 matrix/preconditioner/Krylov vectors inside FP64 iterative refinement */
/* ICCG solves as in FC_PREC_MIXED, but the FP32 inner solve runs on a
 * multicolour ordering of the rows: its DIC factor is built and applied one
 * colour at a time (bandwidth-bound passes instead of the natural order's long
 * chain of levels).  The preconditioner differs from the reference's, the
 * stopping test and the FP64 refinement do not.  The other solvers run in
 * FP64 as in FC_PREC_FP64. */
#define FC_PREC_MIXED_COLOURED 2
/* A diagnostic of precision's share in FC_PREC_MIXED_COLOURED: the same
 * multicolour preconditioner, refinement loop and stopping test, with the
 * inner solve in FP64.  No counterpart in the reference. */
#define FC_PREC_COLOURED_FP64 3

int fc_init(int device, fc_ctx** out);
void fc_finalize(fc_ctx* ctx);
const char* fc_last_error(const fc_ctx* ctx);
/* level 1: print the reference's solver report line after every solve */
int fc_set_verbosity(fc_ctx* ctx, int level);
/* FC_PREC_MIXED(_COLOURED): inner FP32 solves to the relative tolerance inner_tol
 * (<=0: 1e-4), at most inner_itmax iterations each (<=0: itr_max); the
 * refinement loop stops on the reference's criterion in FP64. */
int fc_set_precision(fc_ctx* ctx, int mode, double inner_tol, int inner_itmax);
long long fc_kernel_launches(const fc_ctx* ctx);  /* kernels launched so far by this context */
/* device allocations plus frees made by the library so far, over all
 * contexts (a diagnostic: no reference counterpart) */
long long fc_device_alloc_count(void);
/* Fills every device allocation the library makes from now on with the byte
 * value (0..255; -1, the default, leaves new memory as the allocator gives
 * it), over all contexts.  0xFF makes every float and double NaN, so that a
 * read of memory nothing has written shows up in the results.  Testing only:
 * no reference counterpart. */
int fc_debug_fill_allocations(int byte);
int fc_stream_sync(fc_ctx* ctx);
void* fc_stream(fc_ctx* ctx);                     /* the cudaStream_t every call is ordered on */
int fc_event_record(fc_ctx* ctx, int which);      /* which: 0 start, 1 stop (on the context stream) */
int fc_event_elapsed_ms(fc_ctx* ctx, float* ms);

/* ======================================================================== */
/* Linear solvers                                                           */
/* ======================================================================== */
typedef struct {
  int status;            /* FC_* of this solve */
  int itr_used;          /* Krylov iterations (inner iterations in FC_PREC_MIXED) */
  int outer_iterations;  /* refinement steps (FC_PREC_MIXED) */
  int early_exit;        /* 1: initial residual below tol_abs, nothing done */
  double res0_l1;        /* initial residual, L1 norm */
  double resor;          /* res0_l1 / factor: the normalised residual the reference reports */
  double resl;           /* final residual, L1 norm (|g(k+1)| for pmgmres) */
  double factor;         /* sum|a_ii x_i| + small after the first iteration */
  double ms;             /* device time of the solve */
} fc_solve_info;

/* Drop-in for csrsolve (src/linearSolvers/linear_solvers.f90:40-91) with the
 * matrix passed explicitly, as the individual solvers take it
 * (linear_solvers.f90:96,206,364,548,789).  solver: "iccg" (DIC-PCG),
 * "bicgstab" (DILU-BiCGStab), "dpcg" (Jacobi-PCG), "gauss-seidel",
 * "pmgmres" (GMRES(4)+ILU(0)).  ia(n+1), ja(nnz), diag(n) are 1-based; fi
 * (in/out), rhs, a may be host or device memory.  *res0 receives the
 * normalised initial residual (left unchanged on the early exit, as in the
 * reference).  The pattern analysis is cached per (ia, ja, diag) address and
 * size; call fc_csr_pattern_forget() after changing a pattern in place.
 * Returns FC_OK, FC_WARN_MAXITER, or an error. */
int fc_csrsolve(fc_ctx* ctx, const char* solver, int n, int nnz, const int* ia, const int* ja,
                const double* a, const int* diag, double* fi, const double* rhs, double* res0,
                int itr_max, double tol_abs, double tol_rel, const char* chvar, int verbose,
                fc_solve_info* info);
int fc_csr_pattern_forget(fc_ctx* ctx);

/* Diagonal factors of the DIC (iccg, linear_solvers.f90:439-445) or DILU
 * (bicgstab, :613-624) preconditioner, d_i stored inverted as there. */
int fc_precond_setup(fc_ctx* ctx, const char* kind, int n, int nnz, const int* ia, const int* ja,
                     const double* a, const int* diag, double* d_out);
/* z = M^-1 q with the same preconditioner (forward sweep, z/(d+small),
 * backward sweep: linear_solvers.f90:458-475). */
int fc_precond_apply(fc_ctx* ctx, const char* kind, int n, int nnz, const int* ia, const int* ja,
                     const double* a, const int* diag, const double* q, double* z_out);
/* y = A x (ax_cr, linear_solvers.f90:1173) or y = A^T x (atx_cr, :1079). */
int fc_spmv(fc_ctx* ctx, int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag,
            const double* x, double* y, int transpose);
/* Statistics of the schedule-ordered sweep structure of the mesh system
 * (which=0) or of the cached fc_csrsolve pattern (which=1): out[11] = tiles,
 * levels, widest step of a tile, ring depth, estimated forward-sweep us,
 * ring-served entries, pushed entries, cross-tile entries (both triangles),
 * stage depth, most steps of a tile, rows of a step held in the stage
 * buffers (0: whole steps; the further rows of a wider step are read from
 * global memory). */
int fc_sweep_stats(fc_ctx* ctx, int which, double* out);
/* Caps the rows of a sweep step in the pattern analyses that follow (rows
 * >= 1; 0 restores the default).  A level of a tile wider than the cap is
 * split into consecutive steps; the preconditioner is unchanged.  By default
 * a level too wide for the shared-memory staging (e.g. on 6 million
 * tetrahedra) stays one step whose first rows are staged (see
 * fc_set_sweep_stage_rows), and the analysis splits levels by itself only
 * for batched systems or when too few rows would be staged.  Tuning and
 * testing only: no counterpart in the reference. */
int fc_set_sweep_cap(fc_ctx* ctx, int rows);
/* Sets the tile count (thread blocks of the ordered sweeps, at most one per
 * SM) of the pattern analyses that follow; 0 restores the default, the
 * candidate count with the smallest critical-path estimate.  The
 * preconditioner and the iterates do not depend on it.  Tuning and testing
 * only: no counterpart in the reference. */
int fc_set_sweep_tiles(fc_ctx* ctx, int tiles);
/* Sets the rows of a step that the stage buffers hold in the pattern
 * analyses that follow (0 restores the default: whole steps where they fit,
 * else as many rows as fit); the further rows of a wider step read their
 * records from global memory.  Results do not depend on it.  Tuning and
 * testing only: no counterpart in the reference. */
int fc_set_sweep_stage_rows(fc_ctx* ctx, int rows);
/* Appends one JSON line per solve to the file at path (NULL or "": stop):
 * the entry point, solver, variable, rows, precision mode, status,
 * iterations, refinement steps, early exit, res0 (L1), final residual,
 * resor, factor and device ms, the numbers of the reference's report line
 * (linear_solvers.f90:540-541) in machine-readable form.  Solves through
 * fc_csrsolve, the mesh system (SIMPLE, temperature, fc_solve_field), the
 * batched solves and the adjoint are logged.  No counterpart in the
 * reference. */
int fc_set_solve_log(fc_ctx* ctx, const char* path);
/* Colours of the multicolour ordering FC_PREC_MIXED_COLOURED uses for the
 * same systems (which as above); builds the ordering if no solve has yet.
 * Diagnostics only: no counterpart in the reference. */
int fc_mixed_colours(fc_ctx* ctx, int which, int* ncol);

/* ---- Batched solves of independent systems (no reference counterpart: the
 * reference makes one csrsolve call per system, linear_solvers.f90:40-91,
 * e.g. u, v and w in calcuvw, velocity.f90:638, :693, :748).  Every problem
 * keeps its own pattern analysis; one persistent launch solves them all, its
 * grid split into one group of blocks per problem, each group with its own
 * sweep tiles (one per block), barrier, reductions and stopping test.  In
 * FC_PREC_FP64 (and FC_PREC_MIXED_COLOURED, which mixes ICCG only) a
 * problem's iterates are those of a single bicgstab solve on the same tiles;
 * in FC_PREC_MIXED the inner solves are FP32 BiCGStab on the natural
 * ordering inside FP64 refinement, per problem.
 *   fc_batch_add:   1-based CSR pattern (host or device), optional row
 *                   coordinates xyz (3n: x..., y..., z...) for the tiling;
 *                   returns the problem index (>= 0) or an error.
 *   fc_batch_plan:  tiles NULL: the tuned plan cached for these problem
 *                   sizes, else the planner's cost model; or explicit tiles
 *                   per problem (sum <= SMs).  Builds the sweep schedules.
 *   fc_batch_tiles: the current plan.
 *   fc_batch_solve: solver "bicgstab"; a[p], x[p] (in/out), rhs[p] host or
 *                   device arrays; info[p] per problem (ms = the group's
 *                   device time).  Returns the worst status.
 *   fc_batch_tune:  measured solves from x0 (x0 is not modified) to refine
 *                   the model per problem, at most `rounds` plans; keeps the
 *                   fastest, caches it for these sizes, *best_ms its time. */
typedef struct fc_batch fc_batch;
int fc_batch_create(fc_ctx* ctx, fc_batch** out);
int fc_batch_destroy(fc_batch* b);
int fc_batch_add(fc_batch* b, int n, int nnz, const int* ia, const int* ja, const int* diag, const double* xyz);
int fc_batch_plan(fc_batch* b, const int* tiles);
int fc_batch_tiles(fc_batch* b, int* tiles);
int fc_batch_solve(fc_batch* b, const char* solver, const double* const* a, double* const* x,
                   const double* const* rhs, int itr_max, double tol_abs, double tol_rel, fc_solve_info* info);
int fc_batch_tune(fc_batch* b, const char* solver, const double* const* a, const double* const* x0,
                  const double* const* rhs, int itr_max, double tol_abs, double tol_rel, int rounds,
                  double* best_ms);
/* Tracing of the FP64 ICCG kernel (no counterpart in the reference): with
 * on != 0 the solves run a traced instantiation that records per block the
 * SM cycles of each phase and, for the forward and backward sweep of the
 * first iteration, four stamps per step of every tile.  fc_trace_get:
 * out[11] = cycles summed over the blocks for setup, forward sweep, sweep
 * barrier, backward sweep, dot product, p update, SpMV, x/r update; then the
 * blocks that ran, the blocks of the launch (B) and the stamps per tile (K);
 * timeline (optional, 2*B*K*8 entries) receives the stamps as
 * [sweep][tile][step][8]: the compute warps' start of the step, the moment
 * its staged data had landed, the staging thread's start of its copies
 * (clock64 of the tile's SM), the step start on the global timer, then
 * thread 0's next-step loads issued, its row's dependencies ready, its value
 * computed and its stores issued (clock64).  With
 * tracing on, the multicolour inner solve of FC_PREC_MIXED_COLOURED launches
 * its kernels from the host instead of its CUDA graph, so that a profiler
 * sees each launch. */
int fc_set_tracing(fc_ctx* ctx, int on);
int fc_trace_get(fc_ctx* ctx, double* out, unsigned long long* timeline);
/* ILU(0) factors of ilu_cr (linear_solvers.f90:1267-1385) in the CSR slots. */
int fc_ilu0(fc_ctx* ctx, int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag,
            double* l_out);

/* Jacobi-preconditioned CG solve that allocates nothing.  It has no
 * counterpart in the reference.  It is for callers that may not allocate
 * device memory while they solve: cudaMalloc/cudaFree synchronise the whole
 * device and stall the caller's other streams, and a caller whose pool
 * allocator already holds the free memory cannot get more.  Its work vectors
 * live in a fixed scratch area in static device memory of the library
 * (3 * FC_NOALLOC_MAX_N doubles + a small control block, one per device,
 * held until the process exits); n > FC_NOALLOC_MAX_N is rejected with
 * FC_ERR_BAD_INPUT.  The iteration is fc_csrsolve's "dpcg" on the same grid
 * (one block per SM), so both give the same iterates.
 *  - ia(n+1), ja(nnz), diag(n) 0-based with ia[0] == 0 and ia[n] == nnz;
 *    a, x (in/out), b: DEVICE memory of the current device; stream: a
 *    cudaStream_t of that device (NULL = legacy default stream).
 *  - the first call on each device looks up the scratch address
 *    (cudaGetSymbolAddress with that device current).
 *  - calls that overlap in time on the same device (other threads, other
 *    streams) race on the one scratch area: serialise them.
 *  - blocks until the solve has finished (it synchronises the stream), so it
 *    cannot be captured into a CUDA graph; info->ms is not measured (0).
 *  - errmsg (may be NULL) receives a one-line reason on failure.
 * Returns FC_OK, FC_WARN_MAXITER or an error, as fc_csrsolve. */
#define FC_NOALLOC_MAX_N (1 << 20)
int fc_dpcg_noalloc(void* stream, int n, int nnz, const int* ia, const int* ja, const double* a,
                    const int* diag, double* x, const double* b, int itr_max, double tol_abs, double tol_rel,
                    fc_solve_info* info, char* errmsg, int errlen);

/* ======================================================================== */
/* Mesh, fields and finite-volume operators on the device                   */
/* ======================================================================== */
/* Upload the mesh and build everything derived from it once: cell -> face
 * lists, the geometry of read_mesh_native (geometry.f90:416-665, computed on
 * the device), the periodic face mapping (face_mapping, geometry.f90:
 * 1848-1997: the twin faces' owners, centres and area vectors reordered to
 * their pairs), the CSR pattern and face -> CSR slot maps of
 * create_CSR_matrix (sparse_matrix.f90:86-296, periodic pairs included), and
 * zeroed fields.  Replaces read_mesh + create_CSR_matrix + create_fields
 * (main.f90:105-107).  A mesh whose periodic mapping is not one to one, or
 * that couples two cells twice, is rejected. */
int fc_set_mesh(fc_ctx* ctx, const fc_mesh* m);
/* Geometry arrays by the reference's names: "arx","ary","arz","xf","yf","zf"
 * (numFaces), "xc","yc","zc","vol" (numCells), "facint","Df" (numInnerFaces). */
int fc_get_geometry(fc_ctx* ctx, const char* name, double* out);
/* CSR pattern (ia, ja, diag) and icell_jcell_csr_index / jcell_icell_csr_index
 * (numInnerFaces + numPeriodic entries: inner faces, then the periodic pairs
 * in patch and face order), 1-based; any output may be NULL. */
int fc_get_csr_pattern(fc_ctx* ctx, int* n, int* nnz, int* ia, int* ja, int* diag, int* ijk, int* jik);
/* Wall-clock seconds of the phases of the last fc_set_mesh, in this order:
 * FC_SETUP_TOPOLOGY (host checks, cell -> face lists, topology upload),
 * FC_SETUP_GEOMETRY (device geometry), FC_SETUP_PERIODIC (face mapping),
 * FC_SETUP_CSR (device CSR pattern and slot maps, with their download),
 * FC_SETUP_TILING (the sweep tile count: trial schedules of the candidate
 * counts), FC_SETUP_SCHEDULE (the schedule-ordered sweep structure, with
 * every step-width cap tried), FC_SETUP_ANALYSIS (the rest of the pattern
 * analysis: checks, transpose slots, level sets, uploads), FC_SETUP_FIELDS
 * (field allocation).  seconds holds FC_SETUP_PHASES values. */
#define FC_SETUP_TOPOLOGY 0
#define FC_SETUP_GEOMETRY 1
#define FC_SETUP_PERIODIC 2
#define FC_SETUP_CSR 3
#define FC_SETUP_TILING 4
#define FC_SETUP_SCHEDULE 5
#define FC_SETUP_ANALYSIS 6
#define FC_SETUP_FIELDS 7
#define FC_SETUP_PHASES 8
int fc_get_setup_times(fc_ctx* ctx, double* seconds);

/* Fields by the reference's variable names: "u","v","w","p","pp","vis","den","t"
 * (numTotal), "flmass" (numFaces), "visw" (number of wall faces), "su","sv",
 * "sw","spu","spv","sp","apu","apv","apw" (numCells), "dUdxi","dVdxi",
 * "dWdxi","dPdxi","dTdxi" (3*numTotal, (3,numTotal) layout) and "a" (nnz, the
 * global matrix).  count must equal the field length. */
int fc_field_set(fc_ctx* ctx, const char* name, const double* values, long long count);
int fc_field_get(fc_ctx* ctx, const char* name, double* out, long long count);
/* Several fields at once with one stream synchronisation: the device-to-host
 * step before a restart dump (write_restart_files,
 * src/io/write_restart_files.f90, stays on the host; after readfiles the
 * fields go back with fc_field_set).  counts[k] as fc_field_get's count. */
int fc_download_fields(fc_ctx* ctx, int nfields, const char* const* names, double* const* out,
                       const long long* counts);
int fc_field_fill(fc_ctx* ctx, const char* name, double value);
double* fc_field_ptr(fc_ctx* ctx, const char* name);  /* device address, NULL if unknown */

#define FC_GRAD_GAUSS   0   /* grad_gauss    gradients.f90:1607 */
#define FC_GRAD_LSQ     1   /* grad_lsq      gradients.f90:782  */
#define FC_GRAD_LSQ_DM  2   /* grad_lsq_dm   gradients.f90:1334 */
#define FC_GRAD_NODE_GAUSS 3 /* grad_node_based_gauss gradients.f90:1491, node values of node_interpolation.f90 */
/* Least-squares gradients with the correct 3x3 solve (no reference
 * counterpart): grad_lsq / grad_lsq_dm compute the y component with the
 * wrong adjugate row (b1*D4 - b2*D5 - b3*D6, gradients.f90:887,1480), and
 * grad_lsq_dm weights boundary faces at xf(i) of the face counter
 * (gradients.f90:1459).  The _EXACT schemes take the adjugate's y row,
 * -b1*D2 + b2*D4 - b3*D8, and (dm) the face's own centre, so that linear
 * fields have exact gradients.  Same matrices as FC_GRAD_LSQ / _DM. */
#define FC_GRAD_LSQ_EXACT    4
#define FC_GRAD_LSQ_DM_EXACT 5
/* Cell-to-node interpolation of the node-based gradient (the `c2n` of
 * node_interpolation.f90:36): FC_C2N_PSL pseudo-Laplacian (the default,
 * :265-631) or FC_C2N_IDS inverse distance (:88-260).  The weights are built
 * on the first node-based gradient after a mesh or method change. */
#define FC_C2N_PSL 0
#define FC_C2N_IDS 1
int fc_set_node_interpolation(fc_ctx* ctx, int method);
/* grad(phi, dPhidxi) (gradients.f90:106-163): phi numTotal values, dphi
 * (3,numTotal); host or device memory.  The context's limiter applies. */
int fc_grad(fc_ctx* ctx, int scheme, const double* phi, double* dphi);
/* The namelist's `limiter` (gradients.f90:13, applied by grad_scalar_field
 * after every gradient, :141-160): every gradient of the context (fc_grad,
 * the velocity and temperature gradients of calcuvw and
 * calculate_temperature) is limited by it.  The pressure gradient of
 * gradp_and_sources is not, as in the reference. */
#define FC_LIMITER_NONE   0  /* 'none' / 'no-limit'                       */
#define FC_LIMITER_BJ     1  /* 'Barth-Jespersen'   gradients.f90:288-366 */
#define FC_LIMITER_VENKAT 2  /* 'Venkatakrishnan'   gradients.f90:373-451 */
#define FC_LIMITER_R      3  /* 'R3' (its active line is R4) :456-535     */
#define FC_LIMITER_MD     4  /* 'multidimensional'  gradients.f90:541-656 */
int fc_set_gradient_limiter(fc_ctx* ctx, int kind);
/* laplacian(mu, phi) (laplacian.f90:1-105): fills the global matrix "a" and
 * accumulates the Dirichlet terms into "su" (not cleared, as there).  Bit b
 * of dirichlet_mask enables the boundary term on patch b; ~0ULL reproduces
 * the reference, which applies it on every patch. */
int fc_laplacian(fc_ctx* ctx, const double* mu, const double* phi, unsigned long long dirichlet_mask);
/* csrsolve(solver, fi, rhs, res0, ...) on the global matrix with the fields
 * x_field (in/out) and rhs_field, exactly the reference's call convention. */
int fc_solve_field(fc_ctx* ctx, const char* solver, const char* x_field, const char* rhs_field, double* res0,
                   int itr_max, double tol_abs, double tol_rel, const char* chvar, fc_solve_info* info);

/* ======================================================================== */
/* SIMPLE path (velocity.f90 calcuvw, calcp_simple.f90, nablap.f90)          */
/* ======================================================================== */
/* convection schemes of face_value (interpolation.f90:28-113, :489-650) */
#define FC_SCHEME_CDS                     0   /* 'cds'          */
#define FC_SCHEME_CENTRAL                 1   /* 'central'      */
#define FC_SCHEME_LINEAR_UPWIND           2   /* 'linearUpwind' */
#define FC_SCHEME_KAPPA                   3   /* 'kappa'        */
#define FC_SCHEME_MUSCL                  10
#define FC_SCHEME_UMIST                  11
#define FC_SCHEME_KOREN                  12
#define FC_SCHEME_SMART                  13
#define FC_SCHEME_AVLSMART               14   /* 'avl-smart' */
#define FC_SCHEME_CHARM                  15
#define FC_SCHEME_VANLEER                16
#define FC_SCHEME_OSPRE                  17
#define FC_SCHEME_MINMOD                 18
#define FC_SCHEME_BOUNDED_LINEAR_UPWIND  19   /* 'boundedLinearUpwind'   */
#define FC_SCHEME_BOUNDED_LINEAR_UPWIND02 20  /* 'boundedLinearUpwind02' */
#define FC_SCHEME_BOUNDED_CENTRAL        21   /* 'boundedCentral'        */
#define FC_SCHEME_FROMM                  22
#define FC_SCHEME_CUI                    23
#define FC_SCHEME_QUICK                  24
#define FC_SCHEME_SPL13                  25

/* The namelist parameters of the SIMPLE path (read_input.f90; defaults in
 * velocity.f90:24-33 and pressure.f90:28-33). */
typedef struct {
  double densit, viscos;      /* density, molecular viscosity */
  double urfU[3], gdsU, urfP; /* under-relaxation, deferred-correction blend */
  int cSchemeU;               /* FC_SCHEME_* for the momentum convection */
  int gradScheme;             /* FC_GRAD_* */
  int pscheme;                /* pressure interpolation: 0 'linear', 1 'central', 2 'weighted' */
  int maxiterU, maxiterP, npcor, pRefCell;
  double tolAbsU, tolRelU, tolAbsP, tolRelP;
  char lSolverU[16], lSolverP[16];  /* csrsolve names */
  double flomas;              /* inlet mass flow (init.f90:179-195) */
} fc_simple_params;

int fc_simple_set_params(fc_ctx* ctx, const fc_simple_params* prm);
/* inner-face mass fluxes from the face-interpolated velocity (init.f90:167-176) */
int fc_init_flmass(fc_ctx* ctx);
int fc_update_velocity_at_boundary(fc_ctx* ctx);
/* gradp_and_sources(p) (nablap.f90:19-208) on field "p" or "pp": su,sv,sw and dPdxi */
int fc_gradp_and_sources(fc_ctx* ctx, const char* field);
/* calcuvw (velocity.f90:50-750): momentum assembly (periodic pairs by
 * facefluxuvw_periodic, :1038-1179) and the three solves; resor[3] receives
 * the normalised initial residuals of U, V, W. */
int fc_calcuvw(fc_ctx* ctx, double* resor);
/* on != 0: calcuvw solves U, V and W together (when lSolverU is bicgstab) in
 * one batched launch (fc_batch_*) on three copies of the mesh pattern, each
 * with its own diagonal and source as velocity.f90:611-748 forms them; the
 * resulting fields, residuals and matrix state are those of the three
 * sequential solves up to the rounding of the solvers' reductions.  Default
 * off.  No counterpart in the reference. */
int fc_simple_set_batched_momentum(fc_ctx* ctx, int on);
/* calcp_simple (calcp_simple.f90:1-470); *resor4 = resor(4) of continuityErrors. */
int fc_calcp_simple(fc_ctx* ctx, double* resor4);
/* one outer SIMPLE iteration (main.f90:159-165); resor[4] as the reference
 * logs them; FC_ERR_NAN when max(resor(1:3)) > 1e30 (main.f90:202-207). */
int fc_simple_iteration(fc_ctx* ctx, double* resor);

/* ---- Transient momentum and PISO (velocity.f90:133-290, :565-570;
 * calcp_piso.f90:86-489; time_shift.f90; main.f90:132-165).
 *   scheme: the unsteady term of calcuvw, FC_TIME_BDF (Euler), FC_TIME_BDF2
 *   or FC_TIME_BDF3, on the old levels "uo", "uoo", "uooo" (and v, w);
 *   FC_TIME_STEADY for none.  Crank-Nicolson is not supported.
 *   piso != 0: calcuvw keeps its explicit terms in "rU", "rV", "rW" for
 *   fc_calcp_piso; ncorr PISO correctors, npcor pressure solves per
 *   corrector (fc_simple_params.npcor), urfP.  PISO with BDF2/BDF3 is
 *   rejected: the reference extrapolates the mass fluxes and pressure from
 *   old levels (velocity.f90:146-162) that its time_shift never updates.
 *   Incompressible, with periodic pairs as SIMPLE, without pressure
 *   boundaries.
 * fc_time_shift: time_shift.f90 for the velocity levels.
 * fc_calcp_piso: calcp_piso; *resor4 as continuityErrors sets resor(4).
 * fc_piso_iteration: calcuvw + calcp_piso, resor[4], and the divergence
 * stop of main.f90:202-207. */
#define FC_TIME_STEADY 0
#define FC_TIME_BDF    1
#define FC_TIME_BDF2   2
#define FC_TIME_BDF3   3
typedef struct {
  double timestep;
  int scheme;   /* FC_TIME_* */
  int piso;     /* 1: PISO (keep rU, rV, rW) */
  int ncorr;    /* PISO correctors */
} fc_transient_params;
int fc_transient_set_params(fc_ctx* ctx, const fc_transient_params* prm);
int fc_time_shift(fc_ctx* ctx);
int fc_calcp_piso(fc_ctx* ctx, double* resor4);
int fc_piso_iteration(fc_ctx* ctx, double* resor);

/* The outer loops of main.f90:132-267: numstep time steps (time_shift first
 * when the context is transient), in each up to maxit iterations of calcuvw
 * + calcp_simple (or calcp_piso in PISO mode) + calculate_temperature (when
 * temperature != 0), until max(resor(1:3)) < tolerance.  A transient run
 * then goes on with the next time step; a steady one stops there, as
 * converged.  Stops with FC_ERR_NAN when the iterations diverge
 * (max(resor(1:3)) > 1e30).  *steps, *iterations: done; resor[4]: the last
 * iteration's resor(1:4). */
typedef struct {
  int numstep;
  int maxit;
  double tolerance;
  int temperature;
} fc_run_params;
int fc_run(fc_ctx* ctx, const fc_run_params* prm, int* steps, int* iterations, double* resor);

/* ---------------------------------------------------------------------------
 * Scalar transport: the temperature equation (ScalarEqns/temperature.f90).
 * --------------------------------------------------------------------------- */

/* The namelist parameters of calculate_temperature (temperature.f90:14-25,
 * parameters.f90:30; read_input.f90:86-88,152).  viscos and gradScheme are
 * the global ones the reference shares with the momentum equations. */
typedef struct {
  double viscos;              /* molecular viscosity */
  double pranl;               /* Prandtl number of the fluid */
  double sigt;                /* turbulent Prandtl number (1.0 by default) */
  double urfT, gdsT;          /* under-relaxation (0.9), deferred-correction blend (1.0) */
  int cSchemeT;               /* FC_SCHEME_* (linearUpwind by default) */
  int gradScheme;             /* FC_GRAD_* */
  int maxiterT;               /* csrsolve itr_max (10) */
  double tolAbsT, tolRelT;    /* csrsolve tolerances (1e-13, 0.02) */
  char lSolverT[16];          /* csrsolve name ('bicgstab') */
} fc_temperature_params;

/* Sets the parameters and bcDFraction(7,1:numBoundaries) of the mesh's
 * patches: 1.0 marks an isothermal wall (Dirichlet on T), 0.0 an adiabatic
 * one; other values leave a wall without a temperature condition, as in the
 * reference.  bc_dfraction may be NULL (all 0, geometry.f90:226).  Replaces
 * the namelist read and the bcDFraction setup of field_initialization.f90. */
int fc_temperature_set_params(fc_ctx* ctx, const fc_temperature_params* prm, const double* bc_dfraction);
/* calculate_temperature (temperature.f90:35-385) for the steady case without
 * turbulent heat fluxes: grad(T), the facefluxsc assembly of the matrix and
 * sources (scalar_fluxes.f90:32-141, :147-251 for periodic pairs, :256-337),
 * the boundary conditions,
 * under-relaxation, csrsolve(lSolverT, T, su, resor(7), ...), updateBoundary(T)
 * and the clip to small when min(T) < 0.  With solve == 0 the call stops after
 * the under-relaxation and leaves the system in the mesh's matrix and "su".
 * *resor7 (may be NULL) receives resor(7).  Fields: "t", "dTdxi", "vis",
 * "flmass"; a 'wallQFlux' patch type does not exist in the reference's mesh
 * setup (srdw covers 'wall' patches only) and is not accepted. */
int fc_calculate_temperature(fc_ctx* ctx, int solve, double* resor7);

/* ---- Turbulence: the k-omega SST model (TurbulenceModels/k_omega_SST.f90),
 * high-Re form (LowRe = .false.), steady, without buoyancy.  The settings of
 * one transported scalar (TurbModelData.f90 TurbScalar): */
typedef struct {
  double urf, gds;       /* under-relaxation, deferred-correction factor */
  int cScheme;           /* interpolation scheme id, as cSchemeU */
  char lSolver[16];      /* csrsolve solver name */
  int maxiter;
  double tolAbs, tolRel;
} fc_turb_scalar;
typedef struct {
  fc_turb_scalar k, omega;  /* TurbModel%Scalar(1) and (2) */
  double urfVis;            /* TurbModel%urfVis, eddy-viscosity under-relaxation */
  int gradScheme;           /* FC_GRAD_* of grad(k) and grad(omega), the case's gradient scheme */
} fc_turbulence_params;
/* Defaults of TurbModelData.f90: urf 0.7, gds 1, linearUpwind, bicgstab,
 * maxiter 10, tolAbs 1e-10 (a default-real literal), tolRel 0.01; urfVis 1;
 * Gauss gradients.  viscos and densit come from fc_simple_set_params. */
int fc_turbulence_set_params(fc_ctx* ctx, const fc_turbulence_params* prm);
/* wall_distance_poisson (mesh/wall_distance.f90:29-118): the field
 * "walldist" (numCells) from lap(phi) = -1 solved by ICCG with the
 * reference's laplacian (phi = 0 on every patch; 500 iterations, tolAbs
 * 1e-12, tolRel 1e-10, both default-real literals), non-wall boundary values
 * from the owners, d = -|grad phi| + sqrt(|grad phi|^2 + 2 phi).  The
 * matrix "a" and "su" are overwritten / added to, as there. */
int fc_wall_distance(fc_ctx* ctx);
/* modify_viscosity_turbulence (modify_viscosity_turbulence.f90:25-45) with
 * TurbModel%name = 'k_omega_sst': Gauss gradients of u, v, w ("dUdxi"...),
 * the strain magnitude ("magStrain", calc_strain_and_vorticity.f90), the k
 * and omega equations (calcsc, k_omega_SST.f90:91-785: production with its
 * limiter, the blending function "fsst", cross diffusion, sigma-blended
 * diffusion, inlet/outlet/pressure and periodic faces, wall functions:
 * the wall-cell production of k and omega fixed in wall cells, csrsolve,
 * updateBoundary, the clip to small) and the eddy viscosity "vis" with its
 * wall values "visw", "ypl", "tau" (modify_mu_eff, :790-958).  Fields: "te"
 * (k), "ed" (omega), "fsst" (read by the k equation before the omega
 * equation recomputes it; the reference reads it uninitialised on the first
 * call, zero here), "gen", "walldist" (fc_wall_distance), "u", "v", "w",
 * "vis", "den", "flmass", "visw".  resor56 (may be NULL) receives resor(5)
 * and resor(6). */
int fc_kw_sst(fc_ctx* ctx, double* resor56);

/* ---- The case namelist &input_parameters (read_input.f90:28-227) for the
 * keys this path uses, starting from the reference's module defaults
 * (velocity.f90:24-33, pressure.f90:28-33, temperature.f90:14-25; default-real
 * literals such as urfU = 0.7 promoted as the reference promotes them).
 * The gradient flags select FC_GRAD_* as grad_scalar_field does; ltransient
 * with bdf / bdf2 / bdf3, SIMPLE / PISO, ncorr, npcor, numstep, maxit,
 * tolerance and timestep fill the transient and loop settings.  lstsq_qr,
 * CN, compressible and const_mflux are rejected (errmsg says which); keys
 * of other modules are skipped.  fc_namelist_read needs no GPU.
 * fc_apply_settings passes them to a context (simple, transient, limiter
 * and, with calcT, temperature parameters); fc_run then runs the loops. */
typedef struct {
  fc_simple_params simple;
  fc_temperature_params temperature;
  fc_transient_params transient;
  fc_run_params run;
  int limiter;                /* FC_LIMITER_* */
  int calcU, calcP, calcT;
  int mesh_foam;              /* mesh_format 'foamMesh' (else 'nativeMesh') */
  char title[72];
} fc_case_settings;
int fc_namelist_read(const char* path, fc_case_settings* out, char* errmsg, int errlen);
int fc_apply_settings(fc_ctx* ctx, const fc_case_settings* s);

/* ---------------------------------------------------------------------------
 * Discrete adjoint of steady scalar convection-diffusion.  No counterpart in
 * the reference; the operator is the implicit part of its facefluxsc
 * (scalar_fluxes.f90:32-141, :256-337) with temperature.f90's main diagonal.
 * --------------------------------------------------------------------------- */

/* A(gamma) phi = source * vol on the current mesh: upwind convection of the
 * face fluxes in field "flmass", diffusion gamma_f Df with gamma_f the
 * face-interpolated cell diffusivity (facint), phi = 0 on every boundary face
 * (coefficient gamma_P |S|^2 / (d.S)), no deferred or non-orthogonal
 * correction.  gamma, source: numCells values, host or device.  The matrix
 * goes to the mesh's matrix, the right-hand side to field "su". */
int fc_cd_assemble(fc_ctx* ctx, const double* gamma, const double* source);
/* Solves the assembled system with BiCGStab from phi = 0 to the relative
 * tolerance (the reference's L1 test); phi (numCells, host or device, may be
 * NULL) receives the solution, which is also kept for fc_cd_adjoint. */
int fc_cd_solve(fc_ctx* ctx, double* phi, int itr_max, double tol_rel, fc_solve_info* info);
/* Given dJ/dphi (numCells) for the last solution: solves A^T lambda = dJ/dphi
 * (BiCGStab on the transposed values, same pattern) and returns
 * dJ/dgamma_c = -lambda^T (dA/dgamma_c) phi from a reverse face loop that
 * recomputes the face coefficients.  lambda, dJdgamma may be NULL. */
int fc_cd_adjoint(fc_ctx* ctx, const double* dJdphi, double* lambda, double* dJdgamma, int itr_max, double tol_rel,
                  fc_solve_info* info);

#ifdef __cplusplus
}
#endif
#endif /* FC_GPU_H */
