/*
 * cm_fe.h — C ABI of the GB300 finite-elasticity assembly library
 * (libcm_fe.so).
 *
 * The library replaces the per-element hot loop of OpenCMISS-Iron's static
 * nonlinear finite-element assembly for incompressible Mooney-Rivlin and
 * transversely-isotropic Guccione elasticity: the element residual and
 * Jacobian with Gauss-point constitutive stress, and their addition into the
 * compressed-row (CSR) Jacobian and the residual vector.  The assembled
 * system is handed unchanged to the caller's Newton/linear solver.
 *
 * Conventions (mirroring the reference's generated C bindings,
 * bindings/generate_bindings/c.py:31-40 and :165-225):
 *   - every entry point returns an int status: FE_NO_ERROR (0) on success,
 *     a negative FE_ERR_* code otherwise; fe_last_error() returns the text;
 *   - objects are opaque handles; arrays are (pointer, size) pairs of plain
 *     C types; no entry point aborts the process;
 *   - degrees of freedom are numbered like the reference's dependent field
 *     on one rank (field_routines.f90:10354-10540, "separated component" dof
 *     order): u_x of all u nodes, u_y, u_z, then the hydrostatic pressure
 *     (one per element for element-based pressure, else one per pressure
 *     node).  The dependent field holds the deformed position z (the
 *     reference initialises it from the geometric field), not a displacement.
 *   - dof, residual and matrix-value arrays may live in host memory or in
 *     device memory of the current CUDA device; the library detects which.
 *     Calls given host memory copy through pinned staging buffers and return
 *     after the result is back in host memory; calls given device memory are
 *     asynchronous on the given stream (NULL = legacy default stream).
 */
#ifndef CM_FE_H
#define CM_FE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define FE_NO_ERROR 0
#define FE_ERR_INVALID_ARGUMENT (-1)
#define FE_ERR_CUDA (-2)
#define FE_ERR_OUT_OF_MEMORY (-3)
#define FE_ERR_NOT_SUPPORTED (-4)
#define FE_ERR_NUMERICAL (-5) /* a Gauss point had det F <= 0 or a non-finite value */
#define FE_ERR_PATTERN (-6)   /* an element entry has no slot in the CSR pattern */

/* Constitutive laws: the reference's equations-set subtypes
 * (equations_set_constants.f90:121, :135). */
#define FE_LAW_MOONEY_RIVLIN 1
#define FE_LAW_GUCCIONE 15

/* Interpolation of the hydrostatic-pressure component. */
#define FE_PRESSURE_ELEMENT_BASED 0 /* one constant per element */
#define FE_PRESSURE_NODE_BASED 1    /* trilinear Lagrange on its own nodes */

/* Mesh and equations-set description.  The geometric field, the fibre field
 * and the three displacement components share mesh component 1 (tensor-product
 * Lagrange, 2 or 3 nodes per xi direction); a node-based pressure uses a
 * trilinear mesh component.  Element node order is xi1 fastest, then xi2,
 * then xi3 (BASIS_LHTP node numbering, basis_routines.f90:2251-2374). */
typedef struct fe_mesh_desc {
  int32_t num_elements;
  int32_t num_nodes_u;         /* nodes of mesh component 1 */
  int32_t num_nodes_p;         /* pressure nodes; 0 for element-based pressure */
  int32_t nodes_per_xi_u;      /* 2 trilinear, 3 triquadratic */
  int32_t pressure_interpolation; /* FE_PRESSURE_* */
  int32_t law;                 /* FE_LAW_* */
  int32_t num_material_components; /* 2 (c1, c2) for MR; 4 (C, bf, bt, bfs) for Guccione */
  int32_t materials_per_element;   /* 0: one set for all elements; 1: one set per element */
  const int32_t* element_nodes_u;  /* [num_elements][nodes_per_xi_u^3], 0-based */
  const int32_t* element_nodes_p;  /* [num_elements][8], 0-based; NULL if element-based */
  const double* geometry;          /* [3][num_nodes_u], component-major */
  const double* materials;         /* [num_material_components] or [num_elements][..] */
  const double* fibre_angles;      /* NULL, or [3][num_nodes_u] fibre/imbrication/sheet (radians) */
} fe_mesh_desc;

typedef struct fe_equations_set* fe_handle;

/* Equations-set set-up: validates the mesh, numbers the dofs, builds the
 * Jacobian's CSR sparsity pattern (JacobianMatrix_StructureCalculate,
 * equations_matrices_routines.f90:5048-5340), the element colouring used for
 * the deterministic scatter, and the device-resident geometric Gauss-point
 * data.  Replaces EQUATIONS_MATRICES_CREATE_FINISH (:403) for this path. */
int fe_create(const fe_mesh_desc* desc, fe_handle* out);
int fe_destroy(fe_handle h);

/* The same structure calculation on the GPU (current device): counting,
 * sorting and de-duplicating the neighbourhood of every row node in device
 * kernels.  Same arguments and results as fe_structure_calculate (desc
 * arrays in host memory); row_ptr and col may be host or device memory.
 * Synchronises `stream` before returning. */
int fe_structure_calculate_device(const fe_mesh_desc* desc, int32_t base, int64_t* num_dofs, int64_t* nnz,
                                  int32_t* row_ptr, int32_t* col, void* stream);

/* Host-only structure calculation (no device needed): the CSR pattern the
 * set-up of fe_create builds for this mesh (JacobianMatrix_StructureCalculate,
 * equations_matrices_routines.f90:5048-5340).  num_dofs and nnz are always
 * returned; row_ptr (num_dofs+1) and col (nnz) are filled when not NULL, with
 * 1-based (base = 1, as ROW_INDICES/COLUMN_INDICES) or 0-based indices. */
int fe_structure_calculate(const fe_mesh_desc* desc, int32_t base, int64_t* num_dofs, int64_t* nnz,
                           int32_t* row_ptr, int32_t* col);

/* Sizes: number of dofs (= rows = columns) and number of CSR nonzeros. */
int fe_sizes(fe_handle h, int64_t* num_dofs, int64_t* nnz);

/* Copy the CSR pattern out (host arrays).  base = 1 gives the reference's
 * 1-based ROW_INDICES / COLUMN_INDICES (matrix_vector.f90, MATRIX_TYPE
 * types.f90:858-877); base = 0 gives 0-based indices.  row_ptr has
 * num_dofs+1 entries, col has nnz entries. */
int fe_csr_pattern(fe_handle h, int32_t base, int32_t* row_ptr, int32_t* col);

/* Residual evaluation: r = assembled element residuals at dof vector x
 * (EQUATIONS_SET_RESIDUAL_EVALUATE_STATIC_FEM, equations_set_routines.f90:
 * 5483-5640, with FiniteElasticity_FiniteElementResidualEvaluate,
 * finite_elasticity_routines.f90:1260-1639, and EQUATIONS_MATRICES_ELEMENT_ADD,
 * equations_matrices_routines.f90:1259-1395).  FP64.  r is overwritten. */
int fe_residual_evaluate(fe_handle h, const double* x, double* r, void* stream);

/* Jacobian evaluation in FP64: CSR values (nnz, in pattern order) of the
 * assembled Jacobian at x (EQUATIONS_SET_JACOBIAN_EVALUATE_STATIC_FEM,
 * equations_set_routines.f90:4878-5024, with
 * FiniteElasticity_FiniteElementJacobianEvaluate,
 * finite_elasticity_routines.f90:842-1175, and
 * EQUATIONS_MATRICES_JACOBIAN_ELEMENT_ADD, equations_matrices_routines.f90:
 * 3174-3225).  values is overwritten.  If r is not NULL the residual at x is
 * produced by the same pass. */
int fe_jacobian_evaluate(fe_handle h, const double* x, double* values, double* r, void* stream);

/* Mixed-precision Jacobian: the displacement-displacement block in FP32, the
 * displacement-pressure coupling blocks (and the structurally zero
 * pressure-pressure block) in FP64.  The two value arrays follow the split
 * pattern returned by fe_mixed_layout().  If r is not NULL the FP64 residual
 * at x is produced by the same pass.  No counterpart in the reference (which
 * assembles in FP64 only); its FP64 parts match fe_jacobian_evaluate.
 * Outputs in host memory are delivered as fe_set_host_output selects; the
 * call returns after they are written. */
int fe_jacobian_evaluate_mixed(fe_handle h, const double* x, float* values_uu, double* values_coupling,
                               double* r, void* stream);

/* Split layout of the mixed Jacobian.  Rows of displacement dofs keep their
 * displacement columns in values_uu (uu_row_ptr over the 3*num_nodes_u u rows)
 * and their pressure columns in values_coupling; rows of pressure dofs keep
 * all their columns in values_coupling.  cp_row_ptr has num_dofs+1 entries.
 * Both arrays are 0-based host arrays; either may be NULL. */
int fe_mixed_layout(fe_handle h, int64_t* nnz_uu, int64_t* nnz_coupling, int32_t* uu_row_ptr,
                    int32_t* cp_row_ptr);

/* Surface-pressure follower load (FiniteElasticity_SurfacePressure{Residual,
 * Jacobian}Evaluate, finite_elasticity_routines.f90:3215-3361, :3049-3208):
 * values holds [3][num_nodes_u] nodal pressures, component n loading the
 * boundary faces normal to xi_n (the reference's pressure-values parameter set
 * of the DELUDELN variable).  Faces whose nodal values are all zero carry no
 * load.  Host or device memory; copied.  NULL removes the load.  Applies to
 * every later residual and Jacobian evaluation. */
int fe_set_surface_pressure(fe_handle h, const double* values);

/* A second equations set on the same mesh (no counterpart in the reference,
 * where each equations set builds its own structures): the clone shares the
 * source's mesh-only device arrays -- pattern, rank tables, colouring,
 * geometry cache, quadrature tables -- and the host pattern, and starts with
 * copies of the source's materials, surface-pressure load and precision and
 * assembly settings, which it then changes independently
 * (fe_set_materials, fe_set_surface_pressure).  Shared arrays are freed with
 * the last handle that uses them; handles may be destroyed in any order.
 * Meant for many load / material variants of one geometry, e.g. the members
 * of one fe_batch. */
int fe_clone(fe_handle src, fe_handle* out);

/* Replaces the material parameters given to fe_create (same layout: one set
 * of num_material_components values, or one per element when
 * materials_per_element was set), as an update of the reference's materials
 * field parameter set does for every later evaluation
 * (finite_elasticity_routines.f90:652 reads them per Gauss point).  Host or
 * device memory; copied. */
int fe_set_materials(fe_handle h, const double* materials);

/* Arithmetic of the high-precision parts of fe_residual_evaluate and
 * fe_jacobian_evaluate_mixed (the residual and the displacement-pressure
 * coupling blocks).  FE_HIGH_PRECISION_FP64 (the default) uses IEEE binary64.
 * FE_HIGH_PRECISION_DOUBLE_FLOAT uses unevaluated pairs of FP32 numbers
 * (about 48 significant bits) on the FP32 pipes, which GB300 runs far faster
 * than its FP64 pipe; results stay within about 1e-13 relative of FP64.
 * No counterpart in the reference (which runs FP64 only). */
#define FE_HIGH_PRECISION_FP64 0
#define FE_HIGH_PRECISION_DOUBLE_FLOAT 1
int fe_set_high_precision(fe_handle h, int32_t mode);

/* How fe_jacobian_evaluate_mixed adds the element contributions into the
 * CSR values and the residual (both deterministic; no counterpart in the
 * reference, which adds element by element, MATRIX_VALUES_ADD_DP2,
 * matrix_vector.f90:2756-2880).
 * FE_ASSEMBLY_STAGED (the default): every element stores its entries in a
 * per-element record on the device, and each CSR row is formed once from the
 * records of the elements around the row's node, in increasing element
 * number: in the same launch, by the block that assembles the node's last
 * element (where one row node's rows fit that kernel's shared memory), else
 * by a second kernel.  Every matrix sector is written once and never read.  The records take, per element, 4 (3 n_p)^2 +
 * 8 n_q 3 n_p + 8 (3 n_p + n_q) bytes (32 kB for a triquadratic element with
 * nodal pressure), allocated on the first staged evaluation and kept with
 * the handle.
 * FE_ASSEMBLY_COLOURED: one launch per element colour, each element adding
 * its entries straight into the CSR arrays (the first contributor in colour
 * order stores, later ones add).  No extra memory.
 * The two orders sum in different orders, so they agree to rounding, not
 * bit for bit; each is bit-reproducible. */
#define FE_ASSEMBLY_STAGED 0
#define FE_ASSEMBLY_COLOURED 1
int fe_set_assembly_order(fe_handle h, int32_t order);

/* How fe_jacobian_evaluate_mixed delivers outputs that are in host memory
 * (no counterpart in the reference, whose matrices live in host memory).
 * FE_HOST_OUTPUT_STREAMED (the default; staged order): the assembly runs in
 * up to 16 launches over consecutive ranges of elements; after each, the rows
 * whose elements are all assembled (for a mesh numbered like the elements,
 * the leading rows of each row block) are copied to the host on a second
 * stream while the next launches run; the residual follows in one copy.
 * Device staging for the outputs.  By default at most 12 launches of equal
 * runs of whole waves of the kernel's resident blocks.
 * FE_HOST_OUTPUT_IN_PLACE (staged order): outputs in page-locked host memory
 * (cudaHostAlloc / cudaHostRegister) are written in place by the row gather
 * over the host link, without a device copy of the result.
 * FE_HOST_OUTPUT_AFTER: assembled into device staging, copied afterwards.
 * The values are the same bit for bit in every mode.  Where the streamed or
 * in-place mode does not apply (the coloured order; for streaming, a mesh
 * whose row neighbourhoods exceed the fused kernel's scratch; for in place,
 * pageable memory) the call copies after the assembly.  chunks: the launches of a
 * streamed assembly, 1..16 of equal element counts, or 0 for the wave plan
 * above. */
#define FE_HOST_OUTPUT_STREAMED 0
#define FE_HOST_OUTPUT_IN_PLACE 1
#define FE_HOST_OUTPUT_AFTER 2
int fe_set_host_output(fe_handle h, int32_t mode, int32_t chunks);

/* Element-level evaluation for a contiguous range of elements (0-based), the
 * direct counterparts of FiniteElasticity_FiniteElementResidualEvaluate /
 * ..JacobianEvaluate(EQUATIONS_SET, ELEMENT_NUMBER).  Element matrices are
 * written column-major (ELEMENT_JACOBIAN%MATRIX(row, col)), n x n each with
 * n = fe_element_size(); element vectors n each. */
int fe_element_size(fe_handle h, int32_t* n);
int fe_element_residuals(fe_handle h, const double* x, int32_t first, int32_t count, double* out, void* stream);
int fe_element_jacobians(fe_handle h, const double* x, int32_t first, int32_t count, double* out, void* stream);

/* ---- Batched assembly (no counterpart in the reference, which evaluates one
 * equations set per call).  A batch groups independent equations sets of the
 * current device (any mix of trilinear / triquadratic elements and pressure
 * interpolations) and assembles all of them with the mixed-precision kernel in
 * ONE persistent cooperative launch that walks the element colours in order,
 * with a grid barrier between colours.  Repeated launches are bit-identical;
 * the result agrees with one fe_jacobian_evaluate_mixed call per member to
 * FP32 rounding in the displacement block and FP64 rounding elsewhere.  The
 * member handles must outlive the batch; members with a surface-pressure
 * load get their boundary faces after each colour's volume work (a second
 * grid barrier per colour); the residual and coupling blocks are computed in
 * FP64.  A batch holds at most 256 members (FE_ERR_NOT_SUPPORTED beyond):
 * their parameters live in one constant-memory table per device, so batched
 * launches and replays of all batches on a device run one after another,
 * whatever streams they are issued on. */
typedef struct fe_batch_s* fe_batch;

int fe_batch_create(const fe_handle* handles, int32_t count, fe_batch* out);
int fe_batch_destroy(fe_batch b);

/* x[i], values_uu[i], values_coupling[i] (and r[i] when r is not NULL) are
 * DEVICE pointers of member i, in the layouts of fe_jacobian_evaluate_mixed;
 * the arrays of pointers are host arrays of length count.  Asynchronous on
 * stream; fe_batch_check() reports numerical and launch failures. */
int fe_batch_jacobian_evaluate_mixed(fe_batch b, const double* const* x, float* const* values_uu,
                                     double* const* values_coupling, double* const* r, void* stream);
int fe_batch_check(fe_batch b, void* stream);

/* Launch configuration: variant (elements per group for triquadratic /
 * trilinear members: 0 = 4/8, 1 = 4/4, 2 = 2/4, 3 = 2/2, 4 = 3/2 compiled for
 * three CTAs per SM; 5 = no persistent launch but the single-set kernels, one
 * launch per member and colour, which the autotuner picks when the members
 * are large enough to fill the GPU on their own), CTAs per SM, and
 * consecutive element groups per work unit (both ignored by variant 5). */
int fe_batch_set_config(fe_batch b, int32_t variant, int32_t ctas_per_sm, int32_t block_groups);
int fe_batch_get_config(fe_batch b, int32_t* variant, int32_t* ctas_per_sm, int32_t* block_groups,
                        double* tuned_ms);

/* Autotuner: times every launch configuration (repeats launches each, CUDA
 * events on stream) on the given buffers and keeps the fastest.  Synchronous. */
int fe_batch_autotune(fe_batch b, const double* const* x, float* const* values_uu,
                      double* const* values_coupling, double* const* r, int32_t repeats, void* stream);

/* Captures one batched assembly with the given buffers into a CUDA graph;
 * fe_batch_replay() launches it on stream (same buffers, current inputs; the
 * members' surface-pressure loads as they were at capture). */
int fe_batch_capture(fe_batch b, const double* const* x, float* const* values_uu,
                     double* const* values_coupling, double* const* r, void* stream);
int fe_batch_replay(fe_batch b, void* stream);
/* Diagnostic for the failure detection of the persistent launch (no
 * counterpart in the reference).  The grid barrier between colours polls at
 * most `polls` times (0: the default limit, a few seconds) and then gives up,
 * sets the batch status word and lets the kernel run on and return;
 * fe_batch_check then reports "a grid barrier gave up waiting".  With
 * extra_arrivals = 1 every barrier waits for one CTA more than the grid has,
 * so every barrier gives up: this exercises that path without a GPU fault
 * (polls must then be 1..4096, so the launch still ends within milliseconds;
 * its results are not valid).  (0, 0) restores the default. */
int fe_batch_set_barrier_limits(fe_batch b, uint32_t polls, uint32_t extra_arrivals);
/* Kernels the batch has run (a replay counts the kernels of its graph). */
int fe_batch_launch_count(fe_batch b, int64_t* count);

/* ---- Residual evaluation that allocates nothing (no counterpart in the
 * reference; same arithmetic as fe_residual_evaluate).
 *
 * fe_residual_evaluate given host memory stages x and r through device
 * buffers that it allocates on its first such call; a caller that must not
 * cause a device allocation at that point (one whose device memory is
 * already committed, so that a cudaMalloc inside a Newton iteration could
 * fail, or one that cannot accept the device-wide synchronisation a
 * cudaMalloc can imply) uses this variant instead.  It stages x and r in one
 * fixed array of 2 * FE_NOALLOC_MAX_DOFS doubles (16 MiB) that is part of the
 * library's device image, and calls no allocating function.
 *
 *  - problems with more than FE_NOALLOC_MAX_DOFS dofs are rejected with
 *    FE_ERR_INVALID_ARGUMENT;
 *  - x and r may be host or device memory; the call returns after r is
 *    written (it synchronises `stream`);
 *  - nothing in the array needs to start at zero: x is copied in whole and
 *    every residual entry is first stored, then added to, by the kernels;
 *  - the array is shared by every handle of a device, so overlapping calls
 *    would race on it: the library serialises them with a process-wide lock,
 *    and every return from the call (error returns included) first waits for
 *    the work it queued on `stream`;
 *  - fe_create looks up the array's device address (cudaGetSymbolAddress)
 *    for its device and caches it; that lookup loads the library module that
 *    holds the array, so the 16 MiB are committed on the device when the
 *    first handle is created there, not inside a later call of this
 *    function. */
#define FE_NOALLOC_MAX_DOFS 1048576
int fe_residual_evaluate_noalloc(fe_handle h, const double* x, double* r, void* stream);

/* ---- Newton load step (replaces the SNES solve the reference runs around the
 * assembly: SOLVER_NEWTON_LINESEARCH defaults, solver_routines.f90:17803-17812,
 * line search :18772-18775, tolerances :18674; Dirichlet rows and columns
 * dropped from the linear system as the solver mapping does,
 * solver_mapping_routines.f90:1420,1592).
 *
 * One load increment: the fixed dofs take fixed_values (the caller applies
 * the increment rule NEW = CUR + (FULL - CUR)/(N - i + 1) of
 * equations_set_routines.f90:6568-6590 to form them); x, in: the initial
 * guess (the reference's: the current field), out: the converged state.
 * Newton with the FP64 Jacobian (fe_jacobian_evaluate), stopping when
 * ||r_free||_2 <= atol or after max_iterations; each step solves the Newton
 * system by right-preconditioned restarted GMRES (classical Gram-Schmidt
 * with one re-orthogonalisation) with a block-diagonal preconditioner
 * (Jacobi on displacement rows, the inverse of diag(B diag(A)^-1 B^T) on
 * pressure rows), then takes a cubic backtracking line search on
 * 1/2 ||r_free||^2 (sufficient decrease alpha, step cap max_step); a trial
 * state with det F <= 0 counts as a failed trial step.  Everything runs on
 * the device; x may be host or device memory.  When a line search finds no
 * trial step with sufficient decrease (down to min_lambda), the step is
 * rejected: x keeps the state from before it, the report says
 * line_search_failed, and Newton stops unconverged.  Returns FE_ERR_NUMERICAL when
 * the initial state already has an inverted element, FE_NO_ERROR otherwise
 * (convergence is in the report). */
typedef struct fe_newton_options {
  int32_t max_iterations;     /* 50 */
  double atol;                /* 1e-10 on ||r_free||_2 */
  double alpha;               /* 1e-4, line-search sufficient decrease */
  double max_step;            /* 1e8, cap on ||dx||_2 */
  double min_lambda;          /* 1e-10, smallest line-search step */
  double ksp_rtol;            /* 1e-5, GMRES relative tolerance (reference KSP default) */
  int32_t ksp_restart;        /* 30 */
  int32_t ksp_max_iterations; /* 600 per Newton step */
  int32_t forcing;            /* 0: fixed ksp_rtol; 1: Eisenstat-Walker choice 2 */
} fe_newton_options;

typedef struct fe_newton_report {
  int32_t iterations;         /* Newton iterations taken */
  int32_t converged;          /* 1 when ||r_free||_2 <= atol */
  int64_t linear_iterations;  /* GMRES iterations over all Newton steps */
  double residual_norm_initial;
  double residual_norm;       /* final ||r_free||_2 */
  double last_lambda;         /* step length of the last line search */
  int32_t line_search_failed; /* 1 when the last line search found no step with sufficient
                                 decrease; x is then the state from before that step */
} fe_newton_report;

void fe_newton_options_default(fe_newton_options* options);
int fe_newton_load_step(fe_handle h, const int32_t* fixed_dofs, const double* fixed_values, int64_t num_fixed,
                        double* x, const fe_newton_options* options, fe_newton_report* report, void* stream);

/* Waits for the handle's work on `stream` and reports numerical problems
 * seen by the kernels since the last call (FE_ERR_NUMERICAL) — the device
 * counterpart of the reference's error flags, set instead of trapping. */
int fe_check(fe_handle h, void* stream);

/* Number of kernels launched by the library since the handle was created. */
int fe_launch_count(fe_handle h, int64_t* count);

/* Copies the text of the last error of the calling thread into buf
 * (cmfe_ExtractErrorMessage, bindings/python/opencmiss/_iron_utils.py:77). */
int fe_last_error(char* buf, int32_t size);

#ifdef __cplusplus
}
#endif

#endif /* CM_FE_H */
