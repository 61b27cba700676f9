/*
 * mrhyde_gb300.h -- C ABI of the GB300-native (sm_103a) workset finite-element assembly path.
 *
 * The entry points replace, for one GPU, the calls MrHyDE's SolverManager makes into its
 * AssemblyManager and its own Krylov loop (paths relative to the MrHyDE source tree):
 *
 *   mrg_problem_create    AssemblyManager ctor + createGroups + DiscretizationInterface setup +
 *                         LinearAlgebraInterface::setupLinearAlgebra graph
 *                         (src/managers/assembly/assemblyManager_construct.hpp:14-180,
 *                          src/managers/assembly/assemblyManager_groups.hpp:14-286,
 *                          src/interfaces/linear_algebra/linearAlgebraInterface_construct.hpp:214-265)
 *   mrg_get_graph         the overlapped CrsGraph the scatter targets (getLocalMatrixDevice row_map/entries,
 *                         src/managers/assembly/assemblyManager_jacres.hpp:145-151)
 *   mrg_assemble          AssemblyManager::assembleJacRes / assembleRes
 *                         (src/managers/assembly/assemblyManager.hpp:237-259, :330-380;
 *                          body src/managers/assembly/assemblyManager_jacres.hpp:121-630, :669-880)
 *   mrg_set_dirichlet     SolverManager::setDirichlet (src/managers/solver/solverManager_util.hpp:60-140)
 *   mrg_get_side_points   the "side ip" points at which MrHyDE's FunctionManager evaluates boundary data
 *   mrg_set_face_bc       "Neumann conditions" / "weak Dirichlet" sides: thermal::boundaryResidual
 *                         (src/physics/thermal.cpp:170-260) in the boundary workset loop of assembleJacRes
 *                         (src/managers/assembly/assemblyManager_jacres.hpp:485-603)
 *   mrg_spmv              Tpetra CrsMatrix::apply as used by SolverManager::PCG
 *                         (src/managers/solver/solverManager_solvers.hpp:852, :884)
 *   mrg_solve_pcg         SolverManager::PCG (src/managers/solver/solverManager_solvers.hpp:812-901)
 *   mrg_newton            SolverManager::nonlinearSolver (src/managers/solver/solverManager_solvers.hpp:290-643)
 *
 * Contract (mirrors the reference's Tpetra contract, jacres:145-151 and solverManager_solvers.hpp:345-355):
 *   - The caller owns u, r, the CSR arrays and the CSR values, all in device memory.
 *   - Assembly ADDS INTO r and J ("sum-into", like CrsMatrix::sumIntoValues) unless MRG_ASM_OVERWRITE is
 *     given, which is exactly "J.setAllToScalar(0); r.putScalar(0);" fused into the assembly.
 *   - Dirichlet rows are not scattered; afterwards J(d,d) = 1 (replace), as setJacobianConstraints does.
 *   - J values must be laid out on the graph returned by mrg_get_graph (canonical structured numbering,
 *     sorted columns).
 *   - All work is enqueued on the caller's stream; nothing synchronises the host except the calls that
 *     return host-visible results (mrg_solve_pcg / mrg_newton statistics).  mrg_assemble can be captured
 *     in a CUDA graph once a first call has created its workspace (the Q2 FP32 Jacobian allocates its
 *     tensor-core workspace on first use); a time-out inside the tensor-core kernel is reported by a
 *     later Q2 FP32 Jacobian call instead of synchronising.
 *   - Every call returns an mrg_status; no C++ exception crosses the ABI.  mrg_last_error() gives text.
 *   - A handle is thread-compatible (one host thread at a time per handle).
 */
#ifndef MRHYDE_GB300_H
#define MRHYDE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* mrg_stream_t; /* identical to cudaStream_t; NULL = legacy default stream */
typedef struct mrg_problem mrg_problem;

typedef enum mrg_status {
  MRG_OK = 0,
  MRG_EINVAL = 1,   /* bad argument (null pointer, size out of range, unsupported combination) */
  MRG_ENOMEM = 2,   /* device allocation failed */
  MRG_ECUDA = 3,    /* a CUDA runtime call failed */
  MRG_ETIMEOUT = 4, /* a bounded device-side wait gave up */
  MRG_ENOTSUP = 5,  /* feature of the reference not built here (adjoint, sensitivities, ...) */
  MRG_ENOCONV = 6,  /* iterative solver did not reach its tolerance */
  MRG_ENUMERIC = 7  /* NaN/Inf detected in input or iteration (e.g. non-SPD matrix in PCG) */
} mrg_status;

/* Physics forms (the reference's "thermal" module, src/physics/thermal.cpp:71-165). */
enum {
  MRG_THERMAL = 0,         /* -div(kappa_cell grad u) = f                    */
  MRG_DIFFUSION_1PU2 = 1   /* -div((1 + u^2) grad u) = f, "thermal diffusion: 1+T^2" */
};
/* Source term forms ("thermal source" function). */
enum { MRG_SRC_CONST = 0, MRG_SRC_SINPROD = 1 /* amp * prod_d sin(freq * x_d) */ };
/* Dirichlet faces of the structured box. */
enum {
  MRG_FACE_XLO = 1, MRG_FACE_XHI = 2, MRG_FACE_YLO = 4, MRG_FACE_YHI = 8,
  MRG_FACE_ZLO = 16, MRG_FACE_ZHI = 32, MRG_FACE_ALL = 63
};
/* Dirichlet value forms. */
enum { MRG_DBC_CONST = 0, MRG_DBC_NODE = 1 /* per-DOF host array of length n_dofs */ };

typedef struct mrg_mesh_desc {
  int32_t dim;    /* 2 (quadrilaterals) or 3 (hexahedra) */
  int32_t order;  /* Lagrange order, 1 or 2 (equispaced nodes, HGRAD_{QUAD,HEX}_C1 / _Cn) */
  int32_t nx, ny, nz;
  double lo[3], hi[3];
  /* Optional host array [(nx+1)(ny+1)(nz+1) * dim] of vertex coordinates (x fastest).  NULL = uniform
     box.  When given, cells may be non-affine and the exact per-cell AD path is used. */
  const double* vertex_coords;
} mrg_mesh_desc;

typedef struct mrg_physics_desc {
  int32_t kind;            /* MRG_THERMAL or MRG_DIFFUSION_1PU2 */
  int32_t source_kind;     /* MRG_SRC_* */
  double source_amp, source_freq;
  double kappa_const;      /* used when kappa_cell is NULL */
  const double* kappa_cell;/* optional host array [n_cells] */
  uint32_t dirichlet_faces;/* MRG_FACE_* bitmask */
  int32_t dirichlet_kind;  /* MRG_DBC_* */
  double dirichlet_const;
  const double* dirichlet_node; /* host [n_dofs], read at the fixed DOFs (MRG_DBC_NODE) */
  int32_t quad_order;      /* 0 -> 2*order (discretizationInterface_construct.hpp:111) */
  int32_t reserved;
} mrg_physics_desc;

typedef struct mrg_problem_info {
  int64_t n_dofs, n_cells, nnz, n_fixed;
  int32_t nodes_per_cell, qp_per_cell;
  int32_t path;            /* MRG_PATH_* chosen at creation */
  int32_t reserved;
} mrg_problem_info;

enum {
  MRG_PATH_FACTORED = 1,   /* identical affine cells: K_e = kappa_c * K_ref, row-gather assembly */
  MRG_PATH_CELL = 2,       /* per-cell geometry + forward-AD tangents in registers, colored scatter */
  MRG_PATH_TENSOR = 3,     /* identical affine hexahedra, Q2 or nonlinear Q1: sum-factorised FP64 residual,
                              row-gather Jacobian (each (row, cell) pair one row of a constant-operand GEMM) */
  MRG_PATH_STORED = 4      /* thermal Q1 hexahedra of general geometry: each cell's kappa-free stiffness (FP64
                              and FP32) and the node loads computed once at creation (the reference's stored
                              per-cell basis data, "storage proportion" 1.0; 432 bytes a cell and 8 a node),
                              row-gather assembly.  MRG_ASM_FORCE_CELL or MRG_ASM_ATOMIC select the per-cell
                              AD kernels instead */
};

/* mrg_assemble flags */
enum {
  MRG_ASM_RES = 1u,            /* residual r += -res.val()                       */
  MRG_ASM_JAC = 2u,            /* Jacobian J += res.dx()                         */
  MRG_ASM_J_FP32 = 4u,         /* J_vals is float[] (mixed precision), else double[] */
  MRG_ASM_OVERWRITE = 8u,      /* fused J.setAllToScalar(0), r.putScalar(0)      */
  MRG_ASM_FIX_ZERO_ROWS = 16u, /* "fix zero rows" (jacres:609-628)               */
  MRG_ASM_FORCE_CELL = 256u,   /* force the per-cell AD path (testing)           */
  MRG_ASM_ATOMIC = 512u,       /* per-cell AD path with atomic scatter instead of the 8-colour scatter */
  MRG_ASM_ADJOINT = 1024u,     /* not supported -> MRG_ENOTSUP                   */
  MRG_ASM_SENS = 2048u,        /* not supported -> MRG_ENOTSUP                   */
  MRG_ASM_TENSOR_CORES = 4096u,/* Q2 FP32 Jacobian: element contractions on tcgen05 tensor cores (3xTF32);
                                  the default for Q2 FP32 Jacobians, kept for explicitness */
  MRG_ASM_CUDA_CORES = 8192u,  /* Q2 FP32 Jacobian: force the CUDA-core contraction instead */
  MRG_ASM_NATIVE_FP64 = 16384u /* Q1 factored path: every kappa sum, product and residual FMA as an FP64
                                  instruction.  By default each S(off) is the exact sum (64-bit fixed point
                                  on the integer pipes) rounded once to FP64, for every row whose kappa lie
                                  within 2^7 of each other, and on cubic cells the axis-neighbour entries,
                                  whose coefficient is +0, and their residual terms take no FP64
                                  instruction (the same values: +0 * S, NaN from a non-finite S or u) */
};

/* ---- problem lifetime ------------------------------------------------------------------------- */
int mrg_problem_create(const mrg_mesh_desc* mesh, const mrg_physics_desc* phys, mrg_problem** out);
/* Same as mrg_problem_create with the handle's device memory allocated (stream-ordered) and uploaded
   on `stream`; nothing synchronises other streams, so problems can be created while other solves run
   (the serving loop).  mrg_problem_create is this call on the legacy default stream. */
int mrg_problem_create_on_stream(const mrg_mesh_desc* mesh, const mrg_physics_desc* phys, mrg_stream_t stream,
                                 mrg_problem** out);
/* Waits for the last stream the handle's work was enqueued on, then frees its memory in stream order. */
int mrg_problem_destroy(mrg_problem* p);
int mrg_problem_get_info(const mrg_problem* p, mrg_problem_info* info);

/* ---- structure (device output buffers, enqueued on stream) ------------------------------------ */
int mrg_get_graph(const mrg_problem* p, int64_t* row_ptr /*[n_dofs+1]*/, int32_t* col_idx /*[nnz]*/,
                  mrg_stream_t stream);
int mrg_get_dof_map(const mrg_problem* p, int32_t* lids /*[n_cells*nodes_per_cell]*/, mrg_stream_t stream);
int mrg_get_fixed_dofs(const mrg_problem* p, int32_t* dofs /*[n_fixed]*/, double* values /*[n_fixed] or NULL*/,
                       mrg_stream_t stream);

/* ---- coefficients and Dirichlet data --------------------------------------------------------- */
int mrg_set_kappa(mrg_problem* p, const double* kappa_dev /*[n_cells]*/, mrg_stream_t stream);
int mrg_set_dirichlet(const mrg_problem* p, double* u_dev /*[n_dofs]*/, mrg_stream_t stream);

/* ---- boundary terms on mesh faces (thermal.cpp:170-260) -------------------------------------- *
 * Faces are numbered 0..2*dim-1 = x-, x+, y-, y+, z-, z+ (bit f of MRG_FACE_*).  Side points of a face are
 * ordered by face cell (first tangential cell index fastest) and then by point of the cell's side rule
 * (the problem's 1-D Gauss rule on the tangential axes, first tangential axis fastest).
 *   MRG_BC_NEUMANN         r_i += int_face g phi_i                        (residual only)
 *   MRG_BC_WEAK_DIRICHLET  Nitsche terms with penalty 10/h, h = face measure^(1/(dim-1)), form_param 1:
 *                          res_i += 10/h k (u - g) phi_i - k (grad u . n) phi_i - k (u - g) (grad phi_i . n)
 *                          (k = kappa_c, or 1 + u^2), in r (as -res) and in J.
 * Box cells and general cells (vertex_coords): on general cells each face cell's side weights, outward
 * normals and h come from its own geometry, computed when the condition is set.  At most 4 points per
 * axis in the side rule (MRG_ENOTSUP otherwise).  A face with a strong Dirichlet condition cannot also
 * carry one of these (MRG_EINVAL). */
enum { MRG_BC_NONE = 0, MRG_BC_NEUMANN = 1, MRG_BC_WEAK_DIRICHLET = 2 };
/* *npts = number of side points of the face; xyz (host, [npts][3], z = 0 in 2-D) may be NULL. */
int mrg_get_side_points(const mrg_problem* p, int32_t face, int64_t* npts, double* xyz);
/* g: host array with one value per side point (NULL = 0).  MRG_BC_NONE removes the face's condition. */
int mrg_set_face_bc(mrg_problem* p, int32_t face, int32_t kind, const double* g);

/* ---- assembly -------------------------------------------------------------------------------- */
int mrg_assemble(mrg_problem* p, const double* u_dev, double* r_dev, void* J_vals_dev, uint32_t flags,
                 mrg_stream_t stream);
/* Residual only: AssemblyManager::assembleRes (assemblyManager_jacres.hpp:669-880), called by the Newton
 * loop before each Jacobian (solverManager_solvers.hpp:380).  mrg_assemble with MRG_ASM_RES and no J;
 * flags may add MRG_ASM_OVERWRITE and the path switches (MRG_ASM_JAC and MRG_ASM_J_FP32 are ignored). */
int mrg_assemble_residual(mrg_problem* p, const double* u_dev, double* r_dev, uint32_t flags, mrg_stream_t stream);

/* ---- linear algebra on the assembled system -------------------------------------------------- */
/* y = J x on the canonical graph; J_fp32 != 0 means J_vals is float[]. */
int mrg_spmv(const mrg_problem* p, const void* J_vals_dev, int32_t J_fp32, const double* x_dev, double* y_dev,
             mrg_stream_t stream);

typedef struct mrg_solve_stats {
  int32_t iterations;       /* PCG iterations (summed over refinement / Newton steps) */
  int32_t outer_iterations; /* Newton / refinement iterations                        */
  double rel_residual;      /* final ||r||_2/||r0||_2 (PCG) or ||F||_inf/||F0||_inf (Newton) */
  double abs_residual;
  int32_t status;           /* mrg_status of the solve                                */
  int32_t reserved;
} mrg_solve_stats;

/* PCG on J x = b (x holds the initial guess).  Same iteration and stopping test as the reference
   (rel. 2-norm); Jacobi preconditioning unless mrg_set_preconditioner chose multigrid.  Synchronises
   `stream` once at the end to return stats. */
int mrg_solve_pcg(mrg_problem* p, const void* J_vals_dev, int32_t J_fp32, const double* b_dev, double* x_dev,
                  double rtol, int32_t maxiter, mrg_solve_stats* stats, mrg_stream_t stream);

/* Jacobi-preconditioned BiCGStab on J x = b for nonsymmetric Jacobians (x holds the initial guess).
   The reference offers the same method as "Belos solver: BiCGStab"
   (src/interfaces/linear_algebra/linearAlgebraInterface_solvers.hpp:108-110).  J_fp32: FP32 matrix,
   solved for the correction in FP32 vectors.  Synchronises `stream` once at the end. */
int mrg_solve_bicgstab(mrg_problem* p, const void* J_vals_dev, int32_t J_fp32, const double* b_dev, double* x_dev,
                       double rtol, int32_t maxiter, mrg_solve_stats* stats, mrg_stream_t stream);

enum { MRG_KRYLOV_AUTO = 0, MRG_KRYLOV_PCG = 1, MRG_KRYLOV_BICGSTAB = 2 };

/* Preconditioner of the CG used by mrg_solve_pcg and by mrg_newton's CG branch.
     MRG_PREC_JACOBI  diagonal scaling: the reference's SolverManager::PCG (default)
     MRG_PREC_GMG     geometric multigrid V(2,2)-cycle on the structured grid: Galerkin coarse operators,
                      Chebyshev-Jacobi smoothing, dense coarsest solve -- the structured-grid counterpart
                      of the reference's MueLu multigrid option for Belos
                      (src/interfaces/linear_algebra/linearAlgebraInterface_solvers.hpp:15-160).
                      Q1 and Q2 problems (a Q2 level 0 is coarsened to Q1 first; MRG_ENOTSUP for higher
                      orders).  Runs in the precision of the Jacobian.
                      In FP32 the levels of at most 1024 rows run as one single-CTA kernel per cycle.
     MRG_PREC_GMG_SPLIT  the same cycle with every step of every level its own launch (bit-identical
                      results; for comparison) */
enum { MRG_PREC_JACOBI = 0, MRG_PREC_GMG = 1, MRG_PREC_GMG_SPLIT = 2 };
int mrg_set_preconditioner(mrg_problem* p, int32_t kind);

typedef struct mrg_newton_opts {
  double nl_tol;        /* relative inf-norm tolerance ("nonlinear TOL")                       */
  int32_t max_iters;    /* "max nonlinear iters"                                                */
  int32_t mixed;        /* 1: FP32 Jacobian + FP32 inner Krylov, FP64 residual and update       */
  double lin_tol;       /* Krylov relative tolerance (FP64 path) or inner tolerance (mixed)     */
  int32_t lin_maxiter;
  int32_t reuse_jacobian; /* 1: assemble J once (linear problems)                              */
  int32_t krylov;       /* MRG_KRYLOV_*: AUTO = PCG for the symmetric thermal form, BiCGStab for 1+u^2 */
  int32_t gmg_full_setup; /* multigrid preconditioner and a re-assembled Jacobian: 1 rebuilds every level at
                             every Newton step; 0 (default) rebuilds the coarse Galerkin operators only at the
                             first step and when the previous Krylov solve needed more iterations than the one
                             right after the last full setup, level 0 always follows the new Jacobian */
} mrg_newton_opts;

/* Newton on F(u) = 0 with u on device (holding the initial guess; Dirichlet values are set first).
   Uses library-owned device workspace (allocated on first use, freed with the problem). */
int mrg_newton(mrg_problem* p, double* u_dev, const mrg_newton_opts* opts, mrg_solve_stats* stats,
               mrg_stream_t stream);

/* ---- batched multiscale-subgrid solves -------------------------------------------------------
   Replaces the per-macro-element loop of local solves (MultiscaleManager::evaluateMacroMicroMacroMap,
   src/managers/multiscale/multiscaleManager.cpp:866 -> SubGridDtN::subgridSolver, src/subgrid/subgridDtN.cpp:985
   -> SubGridDtN_Solver::solve, src/subgrid/subgridDtN_solver.cpp:136, assembly :681, Newton :903) for
   independent steady-thermal Q1 hexahedral local problems on the unit cube: Dirichlet data on every
   boundary node, kappa per cell, constant source.  One persistent launch (captured as a CUDA graph)
   assembles every problem's FP32 Jacobian and solves it by FP32 Jacobi-PCG with FP64 refinement. */
typedef struct mrg_batch mrg_batch;
typedef struct mrg_batch_desc {
  int32_t n_problems;
  const int32_t* sizes;     /* host [n_problems][3] cells per axis, each in [2, 16]          */
  const double* kappa;      /* host, concatenated per-cell kappa of all problems (cell order)  */
  const double* dirichlet;  /* host, concatenated per-node values; read at boundary nodes      */
  double source;            /* constant f                                                      */
} mrg_batch_desc;
typedef struct mrg_batch_info {
  int32_t n_problems;
  int32_t threads, ctas_per_sm; /* launch configuration (autotuned or set) */
  int32_t reserved;
  int64_t n_cells, n_nodes, nnz;
} mrg_batch_info;
typedef struct mrg_batch_opts {
  double tol;        /* ||r||_inf / ||r0||_inf per problem (FP64 residual) */
  double inner_tol;  /* FP32 PCG relative 2-norm tolerance                  */
  int32_t max_outer, max_inner;
} mrg_batch_opts;
typedef struct mrg_batch_stat {
  int32_t outer_iterations, inner_iterations;
  double rel_residual;
  int32_t status, reserved;
} mrg_batch_stat;
int mrg_batch_create(const mrg_batch_desc* desc, mrg_batch** out);
int mrg_batch_destroy(mrg_batch* b);
/* node_off / nnz_off: optional host [n_problems] offsets of each problem in u and J */
int mrg_batch_get_info(const mrg_batch* b, mrg_batch_info* info, int64_t* node_off, int64_t* nnz_off);
/* u_dev: double[n_nodes] (output: solutions); J_dev: float[nnz] (output: each problem's FP32 Jacobian on
   its canonical local graph).  stats: optional host [n_problems]; when given the call synchronises. */
int mrg_batch_solve(mrg_batch* b, double* u_dev, float* J_dev, const mrg_batch_opts* opts, mrg_batch_stat* stats,
                    mrg_stream_t stream);
/* Times the batch under each launch configuration and keeps the fastest (u_dev/J_dev used as scratch). */
int mrg_batch_autotune(mrg_batch* b, double* u_dev, float* J_dev, const mrg_batch_opts* opts, mrg_stream_t stream);
int mrg_batch_set_config(mrg_batch* b, int32_t threads, int32_t ctas_per_sm);

/* Jacobi PCG like mrg_solve_pcg (FP64 Jacobian only) that allocates nothing: no cudaMalloc, cudaFree,
   pinned-host or other allocating call.  No counterpart in the reference; it exists for callers that
   cannot allocate device memory themselves -- a runtime that owns all device memory and admits work
   against a fixed HBM budget, a framework whose pool allocator must be the only one, a latency-critical
   loop.  Its work vectors live in one fixed, file-scope device array of the library, sized for at most
   MRG_NOALLOC_MAX_DOFS unknowns (about 10.5 MB, held by every GPU that loads the library until the
   process exits); larger problems return MRG_EINVAL.  All calls share that array: calls whose GPU work
   overlaps race and must be serialised by the caller.  The first call on a device looks up the array's
   address with that device current; make it before any stream capture on that device. */
#define MRG_NOALLOC_MAX_DOFS (1 << 18)
int mrg_solve_pcg_noalloc(mrg_problem* p, const double* J_vals_dev, const double* b_dev, double* x_dev,
                          double rtol, int32_t maxiter, mrg_solve_stats* stats, mrg_stream_t stream);

/* Sustained FP64 and FP32 FMA issue rates of the current GPU (instructions per second), measured with
   an FMA-throughput kernel; the denominator of the FP64-pipe roofline.  No counterpart in the reference. */
int mrg_measure_fma_rates(double* fp64_fma_per_s, double* fp32_fma_per_s, mrg_stream_t stream);

/* ---- bounded device waits ---------------------------------------------------------------------
   Every device-side wait of the library's kernels has a time limit: the tensor-core Q2 Jacobian's
   mbarrier waits (default 2 s) and the staged SpMV's copy waits in mrg_spmv, the Krylov solvers and the
   multigrid levels (default 1 s).  When a wait runs out, the kernel stops waiting, lets its own copies and
   MMAs in flight land (bounded), frees the tensor memory it holds and exits, and the context stays usable.
   The solvers report MRG_ETIMEOUT; the Q2 assembly, which does not synchronise, reports it on the next Q2
   FP32 Jacobian call; mrg_spmv, which has no status word, leaves the rows of the timed-out tile unwritten.  No counterpart in the reference (its Kokkos kernels have no device waits).
     limit_ns       the limit for this problem's kernels; 0 restores the defaults
     withhold_copy  testing only: nonzero makes the first staged copy of those kernels never be issued, so
                    that its wait runs out (exercises the time-out path without a fault); 0 for normal use
   Waits for the handle's last stream and drops the problem's captured Krylov chunks and multigrid levels,
   which are rebuilt on their next use with the new policy. */
#define MRG_WAIT_LIMIT_MAX_NS 60000000000ull /* 60 s */
int mrg_set_wait_policy(mrg_problem* p, uint64_t limit_ns, int32_t withhold_copy);

/* ---- diagnostics ----------------------------------------------------------------------------- */
int mrg_last_error(char* buf, size_t len);   /* copies the calling thread's last error message */
const char* mrg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MRHYDE_GB300_H */
