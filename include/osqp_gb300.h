/*
 * osqp_gb300.h -- public C API of the GB300 OSQP solver.
 *
 * The types, constants and functions below keep the layout, values and
 * meaning of OSQP 1.0's public API so that a program written against OSQP
 * links against libosqp_gb300.so unchanged:
 *   types      include/public/osqp_api_types.h:37-187
 *   constants  include/public/osqp_api_constants.h:28-222
 *   functions  include/public/osqp_api_functions.h:36-454
 * Struct field order and enum values are part of the ABI and therefore match
 * the reference exactly.  Defaults follow the reference's CUDA build
 * (OSQP_ALGEBRA_CUDA): rho_is_vec 0, adaptive_rho_tolerance 2,
 * check_termination 5, and OSQP_INFTY 1e17 in single precision.
 *
 * Precision: the library is built twice from the same sources.
 *   libosqp_gb300.so      OSQPFloat = float  (reference CUDA default, OSQP_USE_FLOAT)
 *   libosqp_gb300_f64.so  OSQPFloat = double
 * OSQPInt is 32-bit in both, as in the reference CUDA backend
 * (CMakeLists.txt:178-183).  Every norm, dot product and termination
 * quantity is reduced in FP64 on the device in both builds.
 */
#ifndef OSQP_GB300_H
#define OSQP_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#ifdef OSQP_USE_LONG
typedef long long OSQPInt;
#else
typedef int OSQPInt;
#endif

#ifdef OSQP_USE_FLOAT
typedef float OSQPFloat;
#else
typedef double OSQPFloat;
#endif

/* ---- capabilities, statuses, solver kinds (osqp_api_constants.h:28-88) ---- */
enum osqp_capabilities_type {
  OSQP_CAPABILITY_DIRECT_SOLVER   = 0x01,
  OSQP_CAPABILITY_INDIRECT_SOLVER = 0x02,
  OSQP_CAPABILITY_CODEGEN         = 0x04,
  OSQP_CAPABILITY_UPDATE_MATRICES = 0x08,
  OSQP_CAPABILITY_DERIVATIVES     = 0x10
};

enum osqp_status_type {
  OSQP_SOLVED = 1,
  OSQP_SOLVED_INACCURATE,
  OSQP_PRIMAL_INFEASIBLE,
  OSQP_PRIMAL_INFEASIBLE_INACCURATE,
  OSQP_DUAL_INFEASIBLE,
  OSQP_DUAL_INFEASIBLE_INACCURATE,
  OSQP_MAX_ITER_REACHED,
  OSQP_TIME_LIMIT_REACHED,
  OSQP_NON_CVX,
  OSQP_SIGINT,
  OSQP_UNSOLVED
};

enum osqp_polish_status_type {
  OSQP_POLISH_LINSYS_ERROR        = -2,
  OSQP_POLISH_FAILED              = -1,
  OSQP_POLISH_NOT_PERFORMED       = 0,
  OSQP_POLISH_SUCCESS             = 1,
  OSQP_POLISH_NO_ACTIVE_SET_FOUND = 2
};

enum osqp_linsys_solver_type {
  OSQP_UNKNOWN_SOLVER = 0,
  OSQP_DIRECT_SOLVER,
  OSQP_INDIRECT_SOLVER
};

typedef enum {
  OSQP_NO_PRECONDITIONER = 0,
  OSQP_DIAGONAL_PRECONDITIONER
} osqp_precond_type;

enum osqp_error_type {
  OSQP_NO_ERROR = 0,
  OSQP_DATA_VALIDATION_ERROR = 1,
  OSQP_SETTINGS_VALIDATION_ERROR,
  OSQP_LINSYS_SOLVER_INIT_ERROR,
  OSQP_NONCVX_ERROR,
  OSQP_MEM_ALLOC_ERROR,
  OSQP_WORKSPACE_NOT_INIT_ERROR,
  OSQP_ALGEBRA_LOAD_ERROR,
  OSQP_FOPEN_ERROR,
  OSQP_CODEGEN_DEFINES_ERROR,
  OSQP_DATA_NOT_INITIALIZED,
  OSQP_FUNC_NOT_IMPLEMENTED,
  OSQP_LAST_ERROR_PLACE
};

/* ---- default settings and hard limits (osqp_api_constants.h:106-222) ---- */
#define OSQP_VERBOSE               (1)
#define OSQP_WARM_STARTING         (1)
#define OSQP_SCALING               (10)
#define OSQP_POLISHING             (0)
#define OSQP_RHO                   (0.1)
#define OSQP_SIGMA                 (1E-06)
#define OSQP_ALPHA                 (1.6)
#define OSQP_RHO_MIN               (1e-06)
#define OSQP_RHO_MAX               (1e06)
#define OSQP_RHO_TOL               (1e-04)
#define OSQP_RHO_EQ_OVER_RHO_INEQ  (1e03)
#define OSQP_RHO_IS_VEC            (0)
#define OSQP_CG_MAX_ITER           (20)
#define OSQP_CG_TOL_REDUCTION      (10)
#define OSQP_CG_TOL_FRACTION       (0.15)
#define OSQP_ADAPTIVE_RHO_UPDATE_DISABLED   (0)
#define OSQP_ADAPTIVE_RHO_UPDATE_ITERATIONS (1)
#define OSQP_ADAPTIVE_RHO_UPDATE_TIME       (2)
#define OSQP_ADAPTIVE_RHO_UPDATE_KKT_ERROR  (3)
#define _OSQP_ADAPTIVE_RHO_UPDATE_LAST_VALUE (4)
#define OSQP_ADAPTIVE_RHO_UPDATE_DEFAULT    (OSQP_ADAPTIVE_RHO_UPDATE_ITERATIONS)
#define OSQP_ADAPTIVE_RHO_INTERVAL  (50)
#define OSQP_ADAPTIVE_RHO_TOLERANCE (2.0)
#define OSQP_ADAPTIVE_RHO_FRACTION  (0.4)
#define OSQP_ADAPTIVE_RHO_MULTIPLE_TERMINATION (4)
#define OSQP_ADAPTIVE_RHO_FIXED     (100)
#define OSQP_MAX_ITER              (4000)
#define OSQP_EPS_ABS               (1E-3)
#define OSQP_EPS_REL               (1E-3)
#define OSQP_EPS_PRIM_INF          (1E-4)
#define OSQP_EPS_DUAL_INF          (1E-4)
#define OSQP_SCALED_TERMINATION    (0)
#define OSQP_TIME_LIMIT            (1e10)
#ifdef OSQP_USE_FLOAT
#define OSQP_CHECK_DUALGAP         (0)
#else
#define OSQP_CHECK_DUALGAP         (1)
#endif
#define OSQP_CHECK_TERMINATION     (5)
#define OSQP_DELTA                 (1E-6)
#define OSQP_POLISH_REFINE_ITER    (3)

#ifndef OSQP_NULL
#define OSQP_NULL 0
#endif
#ifndef OSQP_NAN
#define OSQP_NAN ((OSQPFloat)0x7fc00000UL)
#endif
#ifdef OSQP_USE_FLOAT
#define OSQP_INFTY ((OSQPFloat)1e17)
#else
#define OSQP_INFTY ((OSQPFloat)1e30)
#endif
#define OSQP_DIVISION_TOL   (1.0 / OSQP_INFTY)
#define OSQP_PRINT_INTERVAL 200
#define OSQP_MIN_SCALING    (1e-04)
#define OSQP_MAX_SCALING    (1e+04)
#define OSQP_CG_TOL_MIN     (1E-7)
#define OSQP_CG_POLISH_TOL  (1e-5)
#ifdef OSQP_USE_FLOAT
#define OSQP_ZERO_DEADZONE  (1e-10)
#else
#define OSQP_ZERO_DEADZONE  (1e-15)
#endif

/* ---- data types (osqp_api_types.h:37-187; field order is ABI) ---- */
typedef struct {
  OSQPInt    m;
  OSQPInt    n;
  OSQPInt*   p;
  OSQPInt*   i;
  OSQPFloat* x;
  OSQPInt    nzmax;
  OSQPInt    nz;
  OSQPInt    owned;
} OSQPCscMatrix;

typedef struct {
  OSQPInt device;
  enum osqp_linsys_solver_type linsys_solver;
  OSQPInt allocate_solution;
  OSQPInt verbose;
  OSQPInt profiler_level;
  OSQPInt warm_starting;
  OSQPInt scaling;
  OSQPInt polishing;
  OSQPFloat rho;
  OSQPInt   rho_is_vec;
  OSQPFloat sigma;
  OSQPFloat alpha;
  OSQPInt           cg_max_iter;
  OSQPInt           cg_tol_reduction;
  OSQPFloat         cg_tol_fraction;
  osqp_precond_type cg_precond;
  OSQPInt   adaptive_rho;
  OSQPInt   adaptive_rho_interval;
  OSQPFloat adaptive_rho_fraction;
  OSQPFloat adaptive_rho_tolerance;
  OSQPInt   max_iter;
  OSQPFloat eps_abs;
  OSQPFloat eps_rel;
  OSQPFloat eps_prim_inf;
  OSQPFloat eps_dual_inf;
  OSQPInt   scaled_termination;
  OSQPInt   check_termination;
  OSQPInt   check_dualgap;
  OSQPFloat time_limit;
  OSQPFloat delta;
  OSQPInt   polish_refine_iter;
} OSQPSettings;

typedef struct {
  char      status[32];
  OSQPInt   status_val;
  OSQPInt   status_polish;
  OSQPFloat obj_val;
  OSQPFloat dual_obj_val;
  OSQPFloat prim_res;
  OSQPFloat dual_res;
  OSQPFloat duality_gap;
  OSQPInt   iter;
  OSQPInt   rho_updates;
  OSQPFloat rho_estimate;
  OSQPFloat setup_time;
  OSQPFloat solve_time;
  OSQPFloat update_time;
  OSQPFloat polish_time;
  OSQPFloat run_time;
  OSQPFloat primdual_int;
  OSQPFloat rel_kkt_error;
} OSQPInfo;

typedef struct {
  OSQPFloat* x;
  OSQPFloat* y;
  OSQPFloat* prim_inf_cert;
  OSQPFloat* dual_inf_cert;
} OSQPSolution;

typedef struct OSQPWorkspace_ OSQPWorkspace;

typedef struct {
  OSQPSettings*  settings;
  OSQPSolution*  solution;
  OSQPInfo*      info;
  OSQPWorkspace* work;
} OSQPSolver;

typedef struct {
  OSQPInt embedded_mode;
  OSQPInt float_type;
  OSQPInt printing_enable;
  OSQPInt profiling_enable;
  OSQPInt interrupt_enable;
  OSQPInt derivatives_enable;
} OSQPCodegenDefines;

extern const char* OSQP_STATUS_MESSAGE[];
extern const char* OSQP_ERROR_MESSAGE[];

/* ---- functions (osqp_api_functions.h) ---------------------------------- */
/* CSC helpers: osqp_api_functions.h:36-120 */
OSQPCscMatrix* OSQPCscMatrix_new(OSQPInt m, OSQPInt n, OSQPInt nzmax,
                                 OSQPFloat* x, OSQPInt* i, OSQPInt* p);
void           OSQPCscMatrix_free(OSQPCscMatrix* mat);
OSQPCscMatrix* OSQPCscMatrix_zeros(OSQPInt m, OSQPInt n);
OSQPCscMatrix* OSQPCscMatrix_identity(OSQPInt m);
OSQPCscMatrix* OSQPCscMatrix_diag_scalar(OSQPInt m, OSQPInt n, OSQPFloat scalar);
OSQPCscMatrix* OSQPCscMatrix_diag_vec(OSQPInt m, OSQPInt n, OSQPFloat* vals);
void           OSQPCscMatrix_set_data(OSQPCscMatrix* M, OSQPInt m, OSQPInt n, OSQPInt nzmax,
                                      OSQPFloat* x, OSQPInt* i, OSQPInt* p);
/* settings / codegen-define objects: osqp_api_functions.h:138-170 */
OSQPSettings*       OSQPSettings_new(void);
void                OSQPSettings_free(OSQPSettings* settings);
OSQPCodegenDefines* OSQPCodegenDefines_new(void);
void                OSQPCodegenDefines_free(OSQPCodegenDefines* defs);
/* library information: osqp_api_functions.h:180-215 */
OSQPInt     osqp_capabilities(void);
const char* osqp_version(void);
const char* osqp_error_message(OSQPInt error_flag);
void        osqp_get_dimensions(OSQPSolver* solver, OSQPInt* m, OSQPInt* n);
/* solver life cycle: osqp_api_functions.h:237-300 (osqp_api.c:332-1133) */
OSQPInt osqp_setup(OSQPSolver** solverp, const OSQPCscMatrix* P, const OSQPFloat* q,
                   const OSQPCscMatrix* A, const OSQPFloat* l, const OSQPFloat* u,
                   OSQPInt m, OSQPInt n, const OSQPSettings* settings);
OSQPInt osqp_solve(OSQPSolver* solver);
OSQPInt osqp_get_solution(OSQPSolver* solver, OSQPSolution* solution);
OSQPInt osqp_cleanup(OSQPSolver* solver);
/* warm start and updates: osqp_api_functions.h:315-430 (osqp_api.c:1184-1464) */
OSQPInt osqp_warm_start(OSQPSolver* solver, const OSQPFloat* x, const OSQPFloat* y);
void    osqp_cold_start(OSQPSolver* solver);
OSQPInt osqp_update_data_vec(OSQPSolver* solver, const OSQPFloat* q_new,
                             const OSQPFloat* l_new, const OSQPFloat* u_new);
OSQPInt osqp_update_data_mat(OSQPSolver* solver,
                             const OSQPFloat* Px_new, const OSQPInt* Px_new_idx, OSQPInt P_new_n,
                             const OSQPFloat* Ax_new, const OSQPInt* Ax_new_idx, OSQPInt A_new_n);
void    osqp_set_default_settings(OSQPSettings* settings);
OSQPInt osqp_update_settings(OSQPSolver* solver, const OSQPSettings* new_settings);
OSQPInt osqp_update_rho(OSQPSolver* solver, OSQPFloat rho_new);
/* Derivatives and code generation exist only with the reference's builtin
 * algebra (CMakeLists.txt:208-216).  These return OSQP_FUNC_NOT_IMPLEMENTED,
 * exactly as the reference's CUDA build does (osqp_api.c:1540-1634). */
OSQPInt osqp_adjoint_derivative_compute(OSQPSolver* solver, OSQPFloat* dx, OSQPFloat* dy);
OSQPInt osqp_adjoint_derivative_get_mat(OSQPSolver* solver, OSQPCscMatrix* dP, OSQPCscMatrix* dA);
OSQPInt osqp_adjoint_derivative_get_vec(OSQPSolver* solver, OSQPFloat* dq, OSQPFloat* dl, OSQPFloat* du);
void    osqp_set_default_codegen_defines(OSQPCodegenDefines* defines);
OSQPInt osqp_codegen(OSQPSolver* solver, const char* output_dir, const char* prefix,
                     OSQPCodegenDefines* defines);

#ifdef __cplusplus
}
#endif

#endif /* OSQP_GB300_H */
