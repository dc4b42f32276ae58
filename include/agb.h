/*
 * agb.h — C ABI of alamo_gb300, a GB300 (sm_103a) implementation of alamo's
 * nodal linear-elastic multigrid path: the Operator::Elastic stencil
 * (Fapply), its damped-Jacobi smoother (Fsmooth), the operator diagonal, the
 * residual, nodal restriction/prolongation, the per-level stiffness
 * coarsening, the Newton right-hand side and the multigrid V-cycle solve
 * behind Solver::Nonlocal::Linear, plus an FP32-cycle / FP64-refinement
 * mixed-precision solve.
 *
 * Every entry point replaces a reference interface (file:line inside the
 * reference project Gopal-B/alamo) cited beside it.  Conventions:
 *   - one handle = one single-level uniform node grid nx*ny*nz on one GPU
 *     (the current CUDA device when the handle is created);
 *   - node fields are float64, x fastest, no ghost nodes; vector fields are
 *     3 components stored one after another (SoA: comp*N + node);
 *   - stiffness per node in the reference's object layout (AoS):
 *     isotropic {lambda, mu}; major-minor the 21 entries data[0..20] of
 *     Set::Matrix4<3,MajorMinor> (src/Set/Matrix4_MajorMinor.H:327-375);
 *   - `where` says whether array arguments are host (AGB_MEM_HOST) or device
 *     (AGB_MEM_DEVICE) pointers; host arrays are copied in and out;
 *   - calls return when their work is complete; they never abort or trap:
 *     errors come back as agb_status, with detail in agb_last_error().
 *   - a handle is not re-entrant; use one handle per host thread.
 */
#ifndef AGB_H
#define AGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    AGB_OK = 0,
    AGB_NOT_CONVERGED = 1, /* iteration cap reached (MLMG's throw, Linear.H:137-146) */
    AGB_NAN = 2,           /* NaN in a residual or the solution (Elastic.cpp:262-286, Linear.H:122-126) */
    AGB_BAD_ARG = 3,       /* inconsistent sizes, null pointers, unknown enum values */
    AGB_CUDA_ERROR = 4,    /* a CUDA call failed; see agb_last_error() */
    AGB_NOT_READY = 5,     /* model or boundary condition not set (Elastic.H:127) */
    AGB_OUT_OF_MEMORY = 6,
    AGB_LIMIT = 7          /* request beyond a documented size limit */
} agb_status;

/* Set::Sym: Isotropic (2 values per node: lambda, mu), MajorMinor (21,
 * src/Set/Matrix4_MajorMinor.H:327-375), Major (45, the finite-deformation
 * tangent, src/Set/Matrix4_Major.H:274-320; per-node kernels only) */
typedef enum { AGB_SYM_ISOTROPIC = 0, AGB_SYM_MAJORMINOR = 1, AGB_SYM_MAJOR = 2 } agb_sym;
typedef enum { AGB_MEM_HOST = 0, AGB_MEM_DEVICE = 1 } agb_mem;
/* BC::Operator::Elastic::Elastic::Type (src/BC/Operator/Elastic/Elastic.H:26) */
typedef enum {
    AGB_BC_DISPLACEMENT = 0,
    AGB_BC_TRACTION = 1,
    AGB_BC_PERIODIC = 2,
    AGB_BC_NEUMANN = 3,
    AGB_BC_NONE = 4
} agb_bc_type;
typedef enum { AGB_PRECISION_FP64 = 0, AGB_PRECISION_MIXED = 1 } agb_precision;
/* AGB_SOLVER_VCYCLE: multigrid iterations on the correction equation as
 * amrex::MLMG runs them for the reference (F-cycles while the iteration count
 * is below opts.max_fmg_iter, V-cycles after; FP32 V-cycles in mixed
 * precision).  AGB_SOLVER_FGMRES: flexible GMRES whose
 * preconditioner is one V-cycle (AMReX's GMRES-with-MLMG-preconditioner
 * scheme); in mixed precision the FGMRES and its V-cycle run in FP32 inside
 * FP64 iterative refinement.  Both stop on the same FP64 residual test. */
typedef enum { AGB_SOLVER_VCYCLE = 0, AGB_SOLVER_FGMRES = 1 } agb_solver;
/* solver.bottom_solver of the reference (Linear.H:279-281): BiCGStab (the
 * reference's default), the smoother alone (final_smooth calls), or a dense
 * direct solve (explicit inverse of the coarsest operator, FP64; falls back
 * to BiCGStab when that operator is singular to working precision or has
 * more than 4000 unknowns). */
typedef enum { AGB_BOTTOM_BICGSTAB = 0, AGB_BOTTOM_DIRECT = 1, AGB_BOTTOM_SMOOTHER = 2 } agb_bottom_solver;
/* The smoother of every multigrid level.  AGB_SMOOTHER_JACOBI is the
 * reference's Operator<Grid::Node>::Fsmooth (src/Operator/Operator.cpp:88-154):
 * two damped-Jacobi sweeps per call, weight opts.omega.  AGB_SMOOTHER_GS has
 * no counterpart in the reference: a colour-ordered (multicolour)
 * Gauss-Seidel smoother, two sweeps per call, each sweep updating the eight
 * node colours (i & 1) + 2 (j & 1) + 4 (k & 1) in turn, in place; weight 1
 * on interior rows and opts.omega on boundary rows. */
typedef enum { AGB_SMOOTHER_JACOBI = 0, AGB_SMOOTHER_GS = 1 } agb_smoother;
/* The outer residual and solution update of the mixed-precision FGMRES
 * solve.  AGB_OUTER_FP64: FP64 arithmetic (the reference's
 * Operator<Grid::Node>::solutionResidual, src/Operator/Operator.cpp:635-657).
 * AGB_OUTER_DFLOAT: double-float arithmetic on the FP32 pipe (each value the
 * unevaluated sum of two floats, about 48 significant bits): the same
 * operator and update with relative rounding near 1e-14 instead of 1e-16, at
 * FP32 speed; the solution is returned in FP64.  Without psi only (psi runs
 * the FP64 form). */
typedef enum { AGB_OUTER_FP64 = 0, AGB_OUTER_DFLOAT = 1 } agb_outer_residual;

/* The FGMRES preconditioner (no counterpart in the reference, whose MLMG has
 * no Krylov outer iteration): one V-cycle on the correction equation, or one
 * F-cycle (the reference's mgFcycle form of its FP64 iteration: the residual
 * restricted to every level, the bottom solve, then on each finer level the
 * interpolated coarser correction as the start of a V-cycle).  Where the
 * F-cycle is unstable (a sharp stiffness jump: the reference's F-cycle
 * iteration stalls there too) FGMRES with it may not converge. */
typedef enum { AGB_PRECOND_V = 0, AGB_PRECOND_F = 1 } agb_precond_cycle;

/* Solver settings; field names follow the reference's `solver.*` keys
 * (Solver::Nonlocal::Linear::Parse, src/Solver/Nonlocal/Linear.H:296-382). */
typedef struct agb_solver_opts {
    int max_iter;             /* multigrid iterations before AGB_NOT_CONVERGED (200) */
    int pre_smooth;           /* Fsmooth calls before restriction (2) */
    int post_smooth;          /* Fsmooth calls after prolongation (2) */
    int final_smooth;         /* Fsmooth calls after a failed bottom solve (8) */
    int bottom_smooth;        /* Fsmooth calls after a good bottom solve (0) */
    int bottom_max_iter;      /* BiCGStab iterations on the coarsest level (200) */
    double bottom_tol_rel;    /* (1e-4) */
    double bottom_tol_abs;    /* (-1: off) */
    double omega;             /* Jacobi damping, Operator.H:123 (2/3) */
    int max_coarsening_level; /* -1: coarsen while every axis keeps >= 2 cells */
    int fixed_iter;           /* > 0: run exactly this many cycles */
    int verbose;
    int precision;            /* agb_precision (AGB_PRECISION_FP64) */
    int inner_cycles;         /* mixed V-cycle iteration: FP32 V-cycles per FP64 residual (1) */
    int solver;               /* agb_solver: V-cycle iteration (MLMG) or FGMRES(V-cycle) */
    int krylov_dim;           /* FGMRES: basis size per cycle, <= 39 (20) */
    double inner_tol;         /* mixed FGMRES: residual reduction of one FP32 inner solve (1e-4) */
    int bottom_solver;        /* agb_bottom_solver (AGB_BOTTOM_BICGSTAB) */
    int fine_kernel;          /* FP32 stencil kernels: 0 z-marching with TMA-staged stiffness on the
                                 levels that allow it (default), 1 one thread per node everywhere */
    int krylov_reorth;        /* FGMRES Gram-Schmidt: 1 re-orthogonalise once, 0 single pass (default) */
    int tma_min_nodes;        /* FP32 levels with at least this many nodes use the z-marching kernels
                                 (fine_kernel 0); smaller ones the per-node kernels (0: 30000) */
    int max_fmg_iter;         /* FP64 multigrid iteration (solver AGB_SOLVER_VCYCLE, precision FP64):
                                 iterations below this count run an F-cycle (MLMG::mgFcycle), later
                                 ones a V-cycle; Linear::PrepareMLMG sets 100000000, so every
                                 iteration is an F-cycle (src/Solver/Nonlocal/Linear.H:261) (100000000) */
    int smoother;             /* agb_smoother: the Fsmooth of every level (AGB_SMOOTHER_JACOBI) */
    int outer_residual;       /* agb_outer_residual of the mixed FGMRES solve (AGB_OUTER_FP64) */
    int precond_cycle;        /* agb_precond_cycle of FGMRES (AGB_PRECOND_V) */
} agb_solver_opts;

typedef struct agb_solve_report {
    int status;               /* agb_status of the solve */
    int iters;                /* multigrid iterations: F- or V-cycles in FP64, FP32 V-cycles in
                                 mixed precision (FGMRES: preconditioner V-cycles) */
    int nlevels;
    int bottom_iters;         /* BiCGStab iterations summed over cycles (last read) */
    int fp64_residuals;       /* FP64 fine-level residual evaluations */
    int reserved;
    double resnorm0;          /* ||rhs - A x0||_inf */
    double rhsnorm0;          /* ||rhs||_inf */
    double final_resnorm;     /* ||rhs - A x||_inf at exit (FP64) */
    double final_resnorm_l2;  /* ||rhs - A x||_2 at exit (FP64) */
    double rhsnorm_l2;        /* ||rhs||_2 */
    double seconds;           /* wall time of the call */
} agb_solve_report;

typedef struct agb_elastic agb_elastic;

/* ---------------------------------------------------------------- set-up */
agb_status agb_default_opts(agb_solver_opts* opts);

/* Operator::Elastic<SYM>::Elastic / define (src/Operator/Elastic.cpp:10-55)
 * with the multigrid hierarchy of Operator<Grid::Node>::define
 * (src/Operator/Operator.cpp:185-228) and Solver::Nonlocal::Linear::Define
 * (src/Solver/Nonlocal/Linear.H:36-43).  nx, ny, nz >= 3 nodes; dx = cell
 * size per axis; opts may be NULL for defaults. */
agb_status agb_elastic_create(agb_elastic** h, int nx, int ny, int nz, const double dx[3], int sym,
                              const agb_solver_opts* opts);
agb_status agb_elastic_destroy(agb_elastic* h);
/* Linear::set* / PrepareMLMG (src/Solver/Nonlocal/Linear.H:170-178, 255-290) */
agb_status agb_elastic_set_opts(agb_elastic* h, const agb_solver_opts* opts);
/* run on a caller's cudaStream_t (NULL: the handle's own stream) */
agb_status agb_elastic_set_stream(agb_elastic* h, void* cuda_stream);
/* Elastic::SetModel (src/Operator/Elastic.cpp:87-116): per-node stiffness,
 * 2 (isotropic) or 21 (major-minor) doubles per node, AoS. */
agb_status agb_elastic_set_model(agb_elastic* h, const double* C, int where);
/* read back the (coarsened) stiffness of a multigrid level, AoS */
agb_status agb_elastic_get_model(agb_elastic* h, int level, double* C, int where);
/* Elastic::SetBC (src/Operator/Elastic.H:61-65) with the tables of
 * BC::Operator::Elastic::Constant (src/BC/Operator/Elastic/Constant.H:
 * 435-436): type[26*3] (agb_bc_type) and val[26*3], region order of the
 * Face enum (src/BC/Operator/Elastic/Elastic.H:35-43). */
agb_status agb_elastic_set_bc(agb_elastic* h, const int* type, const double* val);
/* Operator<Grid::Node>::prepareForSolve (src/Operator/Operator.cpp:253-260):
 * stiffness on all levels (Elastic::averageDownCoeffsSameAmrLevel,
 * src/Operator/Elastic.cpp:746-836) and the diagonal of every level.  Called
 * implicitly by the solves after set_model / set_bc / set_opts. */
agb_status agb_elastic_prepare(agb_elastic* h);
/* Elastic::SetPsi (src/Operator/Elastic.cpp:118-137) and Newton::setPsi
 * (src/Solver/Nonlocal/Newton.H:46-49): the void indicator psi as a CELL
 * field, (nx-1)(ny-1)(nz-1) doubles, x fastest; small = m_psi_small
 * (reference default 1e-8).  Fapply, Diagonal and Fsmooth then scale the
 * stress by psi_avg = (1 - small) avg8(psi) + small and add
 * (C grad u) grad psi (1 - small) on interior rows (Elastic.cpp:191-260,
 * 341-363); coarse levels get the full-weighted psi of
 * averageDownCoeffsSameAmrLevel (Elastic.cpp:839-905); the Newton RHS uses
 * avg8(psi) div(dw) + dw grad psi (Newton.H:236-263).  Cells outside the
 * domain read 1.0.  psi NULL clears it.  With psi set the FP32 levels use
 * the per-node kernels (the z-marching ones carry no psi terms). */
agb_status agb_elastic_set_psi(agb_elastic* h, const double* psi, double small, int where);
agb_status agb_elastic_num_levels(agb_elastic* h, int* nlevels);
agb_status agb_elastic_level_dims(agb_elastic* h, int level, int dims[3]);

/* ------------------------------------------------------ operator hooks */
/* Elastic<SYM>::Fapply (src/Operator/Elastic.cpp:139-292): f = A u on a
 * multigrid level.  u, f: 3*N doubles of that level. */
agb_status agb_elastic_fapply(agb_elastic* h, int level, const double* u, double* f, int where);
/* the same operator evaluated in FP32 arithmetic (the mixed solve's cycle) */
agb_status agb_elastic_fapply_f32(agb_elastic* h, int level, const float* u, float* f, int where);
/* Elastic<SYM>::Diagonal (src/Operator/Elastic.cpp:296-379) */
agb_status agb_elastic_diagonal(agb_elastic* h, int level, double* diag, int where);
/* Operator<Grid::Node>::Fsmooth (src/Operator/Operator.cpp:88-154): each call
 * is two damped-Jacobi sweeps x <- (1-w) x + w (b - (Ax - Dx)) / D. */
agb_status agb_elastic_fsmooth(agb_elastic* h, int level, double* x, const double* b, int ncalls, int where);
/* Operator<Grid::Node>::solutionResidual / correctionResidual
 * (src/Operator/Operator.cpp:635-657): r = b - A x; norms (may be NULL)
 * receives {||r||_inf, ||r||_2}. */
agb_status agb_elastic_residual(agb_elastic* h, int level, const double* x, const double* b, double* r,
                                double norms[2], int where);
/* The FP32 forms of Fsmooth and the residual that the mixed-precision cycles
 * run (the z-marching TMA-staged kernels on the levels large enough for
 * them, the per-node kernels elsewhere), on the level's FP32 stiffness:
 * x <- ncalls x 2 damped-Jacobi sweeps (the same update as
 * agb_elastic_fsmooth, evaluated as x + w (b - Ax) / D); r = b - A x.
 * x, b, r: 3*N floats of that level. */
agb_status agb_elastic_fsmooth_f32(agb_elastic* h, int level, float* x, const float* b, int ncalls, int where);
agb_status agb_elastic_residual_f32(agb_elastic* h, int level, const float* x, const float* b, float* r, int where);
/* The fine-level residual r = b - A x of agb_elastic_residual evaluated in
 * double-float arithmetic (AGB_OUTER_DFLOAT: x, b and the stiffness as hi +
 * lo FP32 pairs, FP32 instructions only), returned in FP64; the norms are
 * those of r rounded to FP32.  No psi. */
agb_status agb_elastic_residual_dfloat(agb_elastic* h, const double* x, const double* b, double* r, double norms[2],
                                       int where);
/* Operator<Grid::Node>::restriction (src/Operator/Operator.cpp:262-363):
 * fine field of level crse_level-1 -> coarse field of level crse_level */
agb_status agb_elastic_restrict(agb_elastic* h, int crse_level, const double* fine, double* crse, int where);
/* Operator<Grid::Node>::interpolation (src/Operator/Operator.cpp:365-434):
 * fine (level fine_level) += P crse (level fine_level+1) */
agb_status agb_elastic_prolong_add(agb_elastic* h, int fine_level, const double* crse, double* fine, int where);

/* MLMG::mgVcycle on the fine level as the reference's hooks drive it: one
 * V-cycle on A cor = res from cor = 0 (pre-smoothing, correction residual,
 * restriction down to the bottom solve, prolongation and post-smoothing up).
 * precision AGB_PRECISION_MIXED runs the cycle in FP32 (res is rounded to
 * FP32, the bottom solve stays FP64); res and cor are FP64 arrays (3*N). */
agb_status agb_elastic_vcycle(agb_elastic* h, const double* res, double* cor, int precision, int where);

/* ------------------------------------------------------------- solves */
/* BC::Operator::Elastic::Constant::Init (src/BC/Operator/Elastic/
 * Constant.H:197-286): boundary values of the BC table into b (3*N). */
agb_status agb_elastic_bc_init(agb_elastic* h, double* b, int homogeneous, int where);
/* Newton::prepareForSolve right-hand side (src/Solver/Nonlocal/Newton.H:
 * 144-231): rhs = b - div(C (grad u - F0)) inside, b - BC(u, grad u,
 * C (grad u - F0)) on the boundary.  F0: NULL (f0_ncomp 0), one value per
 * node for F0 = s I (f0_ncomp 1) or 9 row-major values per node (9). */
agb_status agb_elastic_build_rhs(agb_elastic* h, const double* u, const double* b, const double* F0, int f0_ncomp,
                                 double* rhs, int where);
/* Solver::Nonlocal::Linear::solve (src/Solver/Nonlocal/Linear.H:131-147):
 * multigrid iterations (opts.max_fmg_iter: F-cycles, then V-cycles) or
 * FGMRES on A sol = rhs from the initial guess in sol until
 * ||rhs - A sol||_inf <= max(tol_abs, tol_rel * max(||rhs||_inf, ||r0||_inf)).
 * opts.precision selects the plain FP64 cycle or FP32 cycles inside FP64
 * iterative refinement.  rep may be NULL. */
agb_status agb_linear_solve(agb_elastic* h, double* sol, const double* rhs, double tol_rel, double tol_abs,
                            agb_solve_report* rep, int where);
/* Solver::Nonlocal::Newton::solve with nriters = 1 (src/Solver/Nonlocal/
 * Newton.H:279-358) for a linear model with eigenstrain F0: builds the RHS
 * at u, solves for the increment and adds it to u. */
agb_status agb_newton_solve(agb_elastic* h, double* u, const double* b, const double* F0, int f0_ncomp,
                            double tol_rel, double tol_abs, agb_solve_report* rep, int where);
/* Newton::solve with nriters iterations (Newton.H:279-358): each builds the
 * right-hand side at the current u, solves for the increment starting from
 * the previous increment (the reference keeps its correction field across
 * iterations), adds it to u and stops when max |increment| < nrtolerance
 * (the reference's absolute test).  *relnorm (may be NULL) = the last
 * max |increment|; rep describes the last linear solve. */
agb_status agb_newton_solve_n(agb_elastic* h, double* u, const double* b, const double* F0, int f0_ncomp,
                              double tol_rel, double tol_abs, int nriters, double nrtolerance, agb_solve_report* rep,
                              double* relnorm, int where);
/* Stress / strain / energy after a solve (src/Integrator/Base/Mechanics.H:
 * 210-248, src/Operator/Elastic.cpp:426-603): stress = C (grad u - F0),
 * strain = sym grad u, 9 row-major values per node; energy = sigma:eps / 2.
 * Outputs may be NULL. */
agb_status agb_elastic_stress_strain(agb_elastic* h, const double* u, const double* F0, int f0_ncomp,
                                     double* stress, double* strain, double* energy, int where);
/* Newton::solve (src/Solver/Nonlocal/Newton.H:144-196, 279-358) for
 * Model::Solid::Finite::NeoHookean (src/Model/Solid/Finite/NeoHookean.H:
 * 21-121) on a handle of AGB_SYM_MAJOR: up to nriters iterations of
 * F = I + grad u, dw = DW(F), DDW(F) as the operator's stiffness (every
 * multigrid level rebuilt), rhs = b - div dw / b - BC(u, grad u, dw), the
 * increment solved from zero with the handle's solver options, u += it;
 * stops when max |increment| < nrtolerance (relnorm: that norm).  model:
 * (mu, kappa) per node, AoS; u in/out. */
agb_status agb_newton_solve_neohookean(agb_elastic* h, const double* model, double* u, const double* b,
                                       double tol_rel, double tol_abs, int nriters, double nrtolerance,
                                       agb_solve_report* rep, double* relnorm, int where);
/* Elastic::Stress / Elastic::Strain (src/Operator/Elastic.cpp:426-549) on
 * the fine level: which 0 gives sigma = (C grad u) psi_avg (psi_avg = 1
 * without psi), which 1 gives eps = sym grad u; one-sided gradients on the
 * domain faces.  out is SoA per component (the MultiFab layout): voigt != 0
 * gives 6 components (00, 11, 22, 12, 20, 01), else 9 row-major. */
agb_status agb_elastic_tensor(agb_elastic* h, const double* u, int which, int voigt, double* out, int where);

/* ------------------------------------------------ AMR composite solve */
/* Solver::Nonlocal::Linear::solve on an AMR hierarchy (src/Solver/Nonlocal/
 * Linear.H:131-168 driving amrex::MLMG over AMR levels), with the operator's
 * hooks for it: reflux (src/Operator/Operator.cpp:526-633),
 * fixUpResidualMask (:230-251) and averageDownCoeffsDifferentAmrLevels
 * (src/Operator/Elastic.cpp:628-742).  Level 0: the domain, n0 nodes per
 * axis, spacing dx0, the boundary conditions of agb_composite_set_bc.
 * Level l >= 1 (refinement ratio 2): one box of nv[3 l + a] valid nodes
 * from level index lo[3 l + a] (entries of level 0 ignored); lo even, nv
 * odd, and the box with one ring of ghost nodes inside level l-1's valid
 * nodes.  A fine level's arrays (stiffness, F0, solution) cover the box and
 * its ghost ring: nv + 2 nodes per axis.  The solve runs the handle options'
 * V-cycles on each level (precision FP64 or mixed) inside the composite
 * iteration; it stops when the composite residual (every fine valid row and
 * every coarse row not under a finer box) is within max(tol_abs, tol_rel x
 * the composite right-hand side).  u: one array per level (output; ghost
 * rings hold the interpolated coarse values). */
typedef struct agb_composite agb_composite;
agb_status agb_composite_create(agb_composite** c, int nlev, const int n0[3], const double dx0[3], int sym,
                                const int* lo, const int* nv, const agb_solver_opts* opts);
agb_status agb_composite_destroy(agb_composite* c);
/* nodes per axis of a level's arrays */
agb_status agb_composite_level_dims(agb_composite* c, int level, int dims[3]);
/* the domain's boundary conditions (tables of agb_elastic_set_bc) */
agb_status agb_composite_set_bc(agb_composite* c, const int* type, const double* val);
/* the per-node stiffness of one level (AoS, as agb_elastic_set_model) */
agb_status agb_composite_set_model(agb_composite* c, int level, const double* C, int where);
/* F0: NULL or one eigenstrain array per level (NULL entries allowed),
 * f0_ncomp 1 or 9; iters: composite iterations; relnorm: the final relative
 * composite residual */
agb_status agb_composite_solve(agb_composite* c, double* const* u, const double* const* F0, int f0_ncomp,
                               double tol_rel, double tol_abs, int* iters, double* relnorm, int where);

/* ------------------------------------------------ allocation-free call */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * a host code whose memory arena took the whole device at start-up, a plugin
 * living inside such a code, or a time-stepping loop that must not call
 * cudaMalloc/cudaFree between steps because they can synchronise the device.
 * r = b - A x and its norms {||r||_inf, ||r||_2} with no allocation and no
 * handle.  Device memory: C_soa, the per-node stiffness split per component
 * (2 or 21 arrays of nx*ny*nz doubles one after another), and the vector
 * fields x, b, r (3*N doubles).  Host memory: dx, bc_type (the 26*3 table of
 * agb_elastic_set_bc, read on the host before the launch) and norms.  The
 * per-block partial norms live in a fixed 2 MiB device array inside the
 * library (AGB_NOALLOC_MAX_BLOCKS pairs of doubles, one per block of the
 * residual kernel, held by every GPU that loads the library until exit), so
 * grids of more than AGB_NOALLOC_MAX_BLOCKS blocks (about 33.5M nodes) return
 * AGB_LIMIT.  The first call on a device looks the array's address up and
 * caches it; a device reset after that call is not supported.  Calls share
 * the array: calls that overlap on the GPU race and give wrong norms.  Runs
 * on `stream` (NULL: the legacy default stream) and returns after it. */
#define AGB_NOALLOC_MAX_BLOCKS 131072
agb_status agb_residual_norms_noalloc(int nx, int ny, int nz, const double dx[3], int sym, const double* C_soa,
                                      const int* bc_type, const double* x, const double* b, double* r,
                                      double norms[2], void* stream);

/* ------------------------------------------------ learned initial guess */
/* No counterpart in the reference: a 3D U-Net (4 levels, 16/32/64/128
 * channels, 3x3x3 convolutions + ReLU, nodal full-weighting down- and
 * trilinear up-sampling, concatenated skips, 1x1x1 head) on the node grid of
 * one multigrid level, BF16 activations and weights with FP32 accumulation
 * on the tensor cores, FP32 master weights and Adam.  Inputs per node:
 * lambda, mu and the dilatational eigenstrain F0; output: the displacement.
 * n: nodes per axis of the network grid, 8 k + 1 >= 17 (65 for the trained
 * model).  features / target / u: 3 x n^3 doubles, component-major
 * (features: lambda, mu, F0).  Host or device pointers per `where`. */
typedef struct agb_unet agb_unet;
agb_status agb_unet_create(agb_unet** net, int n, uint64_t seed);
agb_status agb_unet_destroy(agb_unet* net);
agb_status agb_unet_num_params(const agb_unet* net, int64_t* count);
/* all parameters as one FP32 vector (host memory), for saving and loading */
agb_status agb_unet_get_params(agb_unet* net, float* out);
agb_status agb_unet_set_params(agb_unet* net, const float* in);
/* one Adam step (learning rate lr) on the mean squared error of one sample;
 * *loss = the loss before the step (in units of (1e-3)^2) */
agb_status agb_unet_train_step(agb_unet* net, const double* features, const double* target, float lr, double* loss,
                               int where);
agb_status agb_unet_predict(agb_unet* net, const double* features, double* u, int where);
/* Initial iterate for the linear solve of a Newton step from zero, on the
 * handle's grid: the model's (lambda, mu) -- the Voigt average for a
 * major-minor model -- and F0 (its trace / 3 for 9 components) are
 * restricted to the multigrid level whose grid is the network's, the
 * prediction is prolongated back to the fine level and written to u; rhs
 * (may be NULL) receives the Newton right-hand side at zero, so
 * agb_linear_solve(h, u, rhs, ...) then solves A u = rhs from the guess and
 * converges to the same displacement as agb_newton_solve from zero.
 * Fallback: when rhs - A u, restricted to the network's level (the smooth
 * part the multigrid cycles reduce slowly), has a larger 2-norm than rhs
 * itself, u is set to zero and *used = 0.  norms[0] = that norm at the
 * guess, norms[1] = at zero. */
agb_status agb_elastic_learned_guess(agb_elastic* h, agb_unet* net, const double* b, const double* F0, int f0_ncomp,
                                     double* u, double* rhs, double norms[2], int* used, int where);
/* Newton::solve (src/Solver/Nonlocal/Newton.H:279-358, nriters = 1, u = 0 on
 * entry) with the learned guess as the first iterate of the step's linear
 * solve, in one call: agb_elastic_learned_guess then agb_linear_solve on
 * device data, so host callers copy b (and F0) in and u out once.  u is
 * output only (the step starts from zero); used (may be NULL) reports
 * whether the guess was kept.  The solve stops at max(tol_abs, tol_rel
 * |rhs|_inf): the tolerance of the solve from zero, whatever the residual at
 * the guess (MLMG's max(|rhs|, |r0|) would loosen it after a guess whose
 * residual exceeds |rhs|). */
agb_status agb_newton_solve_guess(agb_elastic* h, agb_unet* net, double* u, const double* b, const double* F0,
                                  int f0_ncomp, double tol_rel, double tol_abs, agb_solve_report* rep, int* used,
                                  int where);
/* Test hook of the tensor-core convolution: X [V][Cin] BF16 channels-last
 * (device), W [Cout][Cin][27] FP32, bias [Cout] FP32 (may be NULL), output
 * Y (BF16) or Yf (FP32), exactly one non-NULL; stream may be NULL. */
agb_status agb_conv3_bf16(const void* X, int Cin, const float* W, const float* bias, int Cout, int nx, int ny, int nz,
                          int relu, void* Y, float* Yf, void* stream);
/* Test hook of the convolution's weight gradient: dW [Cout][CinW][27] (FP32)
 * += sum_v dY[v][o] X[v + tap][c] and db [Cout] += sum_v dY[v][o], X [V][Cin]
 * BF16 channels-last, dY [V][Cout] FP32 (device pointers); tensor_cores != 0
 * runs the tcgen05 kernel the training uses (dY rounded to BF16), 0 the FP32
 * CUDA-core kernel; stream may be NULL. */
agb_status agb_conv3_wgrad_bf16(const void* X, int Cin, int CinW, const float* dY, int Cout, int nx, int ny, int nz,
                                float* dW, float* db, int tensor_cores, void* stream);

/* --------------------------------------------------------- profiling */
/* Kernel families timed with CUDA events on the handle's stream when
 * profiling is on (fine level only). */
typedef enum {
    AGB_K_FAPPLY_F64 = 0,
    AGB_K_JACOBI_F64 = 1,
    AGB_K_RESIDUAL_F64 = 2,
    AGB_K_FAPPLY_F32 = 3,
    AGB_K_JACOBI_F32 = 4,
    AGB_K_RESIDUAL_F32 = 5,
    AGB_K_RESTRICT = 6,
    AGB_K_PROLONG = 7,
    AGB_K_BOTTOM = 8,
    AGB_K_KRYLOV = 9,  /* FGMRES Gram-Schmidt: dots, projections, normalisation, e = Z y */
    AGB_K_RESIDUAL_DF = 10, /* double-float outer residual of the mixed solve */
    AGB_K_NFAMILIES = 11
} agb_kernel_family;
agb_status agb_profile_enable(agb_elastic* h, int on);
agb_status agb_profile_reset(agb_elastic* h);
/* launches and summed device milliseconds of one family since the reset */
agb_status agb_profile_get(agb_elastic* h, int family, int64_t* launches, double* ms);
/* algorithmic bytes (each vector read or written once per launch) of the
 * timed launches of a family since the reset; kept for AGB_K_KRYLOV */
agb_status agb_profile_bytes(agb_elastic* h, int family, double* bytes);
/* kernels of this library launched since the handle was created */
agb_status agb_launch_count(agb_elastic* h, int64_t* launches);

/* ------------------------------------------------ synthetic inputs */
/* Set::Matrix4<3,MajorMinor>::Cubic(C11, C12, C44, R)
 * (src/Set/Matrix4_MajorMinor.H:518-547), R row-major. */
agb_status agb_cubic_stiffness(double C11, double C12, double C44, const double R[9], double out21[21]);
/* Uniform doubles in [lo, hi) from std::mt19937_64(seed) (53-bit mantissa). */
agb_status agb_synth_uniform(uint64_t seed, int64_t n, double lo, double hi, double* out);
/* One spherical inclusion: nodes x = (i,j,k) dx with |x - center| < radius
 * get (lam_in, mu_in) and F0 = eps_in I, others (lam_out, mu_out), F0 = 0.
 * C: 2 doubles per node; F0s: 1 double per node (may be NULL). */
agb_status agb_synth_inclusion_iso(int nx, int ny, int nz, const double dx[3], const double center[3], double radius,
                                   double lam_in, double mu_in, double lam_out, double mu_out, double eps_in,
                                   double* C, double* F0s);
/* Voronoi polycrystal: nseeds seeds uniform in the box, each node belongs to
 * its nearest seed; every grain gets the cubic stiffness rotated by a
 * Haar-uniform rotation (unit quaternion from 4 normals).  C: 21 doubles per
 * node (AoS); grain (may be NULL): grain id per node. */
agb_status agb_synth_voronoi_cubic(int nx, int ny, int nz, const double dx[3], int nseeds, uint64_t seed, double C11,
                                   double C12, double C44, double* C, int32_t* grain);
/* Non-overlapping spheres (rejection sampling): radius uniform in
 * [rmin, rmax], centres uniform in the box, inclusion (lam_in, mu_in) with
 * dilatational eigenstrain s uniform in [smin, smax]; matrix
 * (lam_out, mu_out).  placed receives the number of spheres placed. */
agb_status agb_synth_spheres_iso(int nx, int ny, int nz, const double dx[3], int nspheres, uint64_t seed, double rmin,
                                 double rmax, double lam_in, double mu_in, double lam_out, double mu_out, double smin,
                                 double smax, double* C, double* F0s, int* placed);
/* The same spheres with the diffuse interface of the reference's ellipse
 * initial condition (src/IC/Ellipse.H:56-75 with A = I / r^2): each sphere
 * contributes eta = 0.5 - 0.5 erf((d^2 - r^2) / (eps d)) at distance d from
 * its centre; the sum, clipped to [0, 1], mixes the two phases linearly
 * (C = (1 - eta) C_out + eta C_in) and F0s = sum of eta_m s_m. */
agb_status agb_synth_spheres_diffuse(int nx, int ny, int nz, const double dx[3], int nspheres, uint64_t seed,
                                     double rmin, double rmax, double eps, double lam_in, double mu_in, double lam_out,
                                     double mu_out, double smin, double smax, double* C, double* F0s, int* placed);

const char* agb_status_string(int status);
const char* agb_last_error(void);
const char* agb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* AGB_H */
