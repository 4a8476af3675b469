/*
 * elpaso_gb300.h -- C ABI of the GB300 frequency-response path.
 *
 * Drop-in for the PETSc Mat-assembly + KSP section of elpasoC's
 * `frequency-basic` analysis:
 *
 *   reference seam (paths inside elpasoCore/source/)
 *   ------------------------------------------------------------------
 *   analysis/frequency/analysisfrequencybasic.cpp:74-279  FullRun
 *     :75  activateDofsAtNodes          -> numbering in elp_model_create
 *     :76  optimizeMatrixPattern        -> pattern in elp_model_create
 *     :81  initializeSolverObjects      -> symbolic phase, elp_model_analyse
 *     :128 assembleGlobalTensors        -> elp_model_assemble (once, not per w)
 *     :137 interface contributions      -> elp_model_assemble
 *     :143 applyNodalLoads              -> right-hand side in elp_model_create
 *     :156 getGlobalBCs/insertBoundaryConditions -> per-w combine in elp_solve
 *     :181 solveEquationSystem (MUMPS)  -> elp_solve
 *
 * Conventions (mirroring PetscErrorCode / INFAMCHKERRQ in
 * math/mathlibrary.h:101-109, but never aborting the process):
 *   - every call returns int status, 0 = success; elp_last_error() gives text;
 *   - caller-owned inputs are copied; outputs go to caller buffers;
 *   - complex numbers are interleaved (re, im) doubles, like the HDF5 compound
 *     {real, imag} the reference writes (misc/hdf5/outputh5.h:231);
 *   - row/column indices are 0-based (the reference's HDF5 export is 1-based,
 *     math/mathlibrary.cpp:62).
 *   - a model handle may be used by one host thread at a time; distinct
 *     handles are independent. The server API is thread-safe.
 */
#ifndef ELPASO_GB300_H
#define ELPASO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define ELP_OK 0
#define ELP_ERR_ARG 1          /* invalid argument / malformed model        */
#define ELP_ERR_CUDA 2         /* CUDA runtime error                        */
#define ELP_ERR_NOMEM 3        /* allocation failed / HBM budget exceeded   */
#define ELP_ERR_GEOMETRY 4     /* non-positive Jacobian (elementfem.cpp:97) */
#define ELP_ERR_SINGULAR 5     /* zero pivot that static pivoting can't fix */
#define ELP_ERR_NOCONV 6       /* refinement did not reach the tolerance    */
#define ELP_ERR_STATE 7        /* call out of order (e.g. solve before assemble) */
#define ELP_ERR_TIMEOUT 8      /* server wait ran out                        */

/* ---- element and material vocabulary (reference names) ----------------- */
/* element/elementfactory.cpp:34-109 string tags */
#define ELP_BRICK8 1   /* "Brick8": 8-node linear solid hexahedron, x1 x2 x3      */
#define ELP_DSG4 2     /* "DSG4":   4-node Reissner-Mindlin plate, x3 w1 w2       */
#define ELP_FLUID8 3   /* "Fluid8": 8-node acoustic hexahedron, fluid pressure    */

/* material/materialfactory.cpp:34-113 tags */
#define ELP_STR_LIN_ELA_ISO_DIR 1 /* isotropic elastic, real E               */
#define ELP_STR_LIN_VIS_ISO_DIR 2 /* isotropic visco, E(1+i eta) / E(1+i w eta) */
#define ELP_AF_LIN_UAF_ISO_DIR 3  /* ideal acoustic fluid: c, rho            */

/* degrees of freedom: fedata/basics_dof.h:24-60 (subset used on this path) */
#define ELP_DOF_X1 0
#define ELP_DOF_X2 1
#define ELP_DOF_X3 2
#define ELP_DOF_W1 3
#define ELP_DOF_W2 4
#define ELP_DOF_W3 5
#define ELP_DOF_FLUID 16
#define ELP_NUM_KNOWN_DOFS 21

typedef struct {
  int kind;        /* ELP_STR_LIN_ELA_ISO_DIR / ELP_STR_LIN_VIS_ISO_DIR / ELP_AF_LIN_UAF_ISO_DIR */
  double E;        /* Young's modulus (structure)                             */
  double nu;       /* Poisson's ratio                                         */
  double rho;      /* density (structure or fluid)                            */
  double t;        /* plate thickness (DSG4)                                  */
  double eta;      /* loss factor (visco)                                     */
  int visco_type;  /* 1: E(1+i eta), 2: E(1+i w eta) (materialstructurevisco.cpp:284-285) */
  double c;        /* speed of sound (fluid)                                  */
  /* Frequency-dependent E and eta of a visco material, as the reference reads
   * them from a file or dataset of rows (frequency [Hz], value)
   * (materialstructurevisco.cpp:75-170) and interpolates linearly in w, held
   * constant outside the table (updateMaterial, :229-287). n = 0: the scalar
   * E / eta above. With an E table, E above is the modulus the stiffness is
   * assembled with (0: the table's first value); the per-w coefficient is
   * E(w) / E. Rows in ascending frequency; the tables are copied. */
  int n_E_table;
  const double* E_table;   /* n_E_table x 2, row-major                        */
  int n_eta_table;
  const double* eta_table; /* n_eta_table x 2, row-major                      */
} elp_material;

typedef struct {
  int type;               /* ELP_BRICK8 / ELP_DSG4 / ELP_FLUID8                 */
  int material;           /* index into elp_model_desc.materials                */
  int64_t n_elements;
  const int32_t* connectivity; /* n_elements x nodes-per-element node INDICES    */
} elp_element_block;

typedef struct {
  double ori;             /* orientation (+1/-1); C and C^T scaled by -ori       */
  int32_t structure_nodes[4]; /* node indices (DSG4 plate nodes)                 */
  int32_t fluid_nodes[4];     /* node indices (Fluid8 nodes; geometry taken here) */
  int fluid_material;     /* index into materials (kept for the interface)       */
} elp_interface_quad;      /* InterfaceMindlin: elementinterfacefactory.cpp:62-98 */

typedef struct {
  int32_t node;           /* node index                                          */
  int32_t dof;            /* ELP_DOF_*                                           */
  double value_re, value_im; /* prescribed value (F[row] = value)                */
} elp_fixed_dof;

typedef struct {
  int32_t node;           /* node index                                          */
  double f[3];            /* Fx Fy Fz on x1 x2 x3 (nodalforcestructure.cpp:46-73) */
} elp_nodal_force;

typedef struct {
  int32_t node;           /* node index                                          */
  double m[3];            /* Mx My Mz on the active rows of w1 w2 w3
                             (applyNodalMoments, analysis.cpp:281-364)           */
} elp_nodal_moment;

typedef struct {
  int32_t node;           /* node index                                          */
  double p;               /* fluid point source: F[fluid row] += 4 pi p
                             (applyNodalForces, analysis.cpp:243-265)            */
} elp_fluid_source;

/* Normal-velocity load on a face of a Fluid8 element (cElementLoadVn,
 * elementfluid3d.cpp:241-309): F += -(i vn / w) int_face N dA at the face's
 * four nodes. face 1..6 selects cShapeHex8's surfaces[face - 1]
 * (shapehex8.cpp:119-150), as the input's Face attribute does. */
typedef struct {
  int32_t block;          /* index into blocks (an ELP_FLUID8 block)            */
  int32_t face;           /* 1..6                                               */
  int64_t element;        /* element index within the block                     */
  double vn;              /* normal velocity                                    */
} elp_vn_load;

/* Constant traction on a face of a Brick8 element (cElementLoadStructureConst,
 * elementloadstructureconst.cpp; cElementStructureBrick::assembleLoadVector and
 * evaluateSurfaceIntegral, elementstructurebrick.cpp:556-662): the u1 u2 u3
 * rows of the face's four nodes get sum_s C(z, s) t_d with
 * C(z, s) = int_face N_z N_s dA, the same traction t at every face node.
 * The reference reads three amplitudes and one phase: t_d = amp_d e^(i phase).
 * face 1..6 as for elp_vn_load. The load does not depend on w. */
typedef struct {
  int32_t block;          /* index into blocks (an ELP_BRICK8 block)            */
  int32_t face;           /* 1..6                                               */
  int64_t element;        /* element index within the block                     */
  double t[6];            /* (re, im) of t1, t2, t3                             */
} elp_face_traction;

typedef struct {
  int64_t n_nodes;
  const int64_t* node_ids;  /* reference node ids; numbering follows ascending id */
  const double* coords;     /* 3 x n_nodes                                        */
  int n_materials;
  const elp_material* materials;
  int n_blocks;
  const elp_element_block* blocks;
  int64_t n_interfaces;
  const elp_interface_quad* interfaces;
  int64_t n_fixed;
  const elp_fixed_dof* fixed;
  int64_t n_forces;
  const elp_nodal_force* forces;
  int64_t n_moments;
  const elp_nodal_moment* moments;
  int64_t n_fluid_sources;
  const elp_fluid_source* fluid_sources;
  int64_t n_vn_loads;
  const elp_vn_load* vn_loads;
  int64_t n_face_tractions;
  const elp_face_traction* face_tractions;
} elp_model_desc;

typedef struct elp_model elp_model;

typedef struct {
  int64_t n_dofs;
  int64_t nnz;
  int64_t n_elements;
  int64_t n_fronts;
  int64_t factor_entries;   /* sum over fronts of m^2                         */
  double factor_flops;      /* real flops of one complex numeric factorisation */
  int n_levels;
  int max_front;
  int n_struct_groups;      /* distinct loss-factor groups of structure K     */
  double gemm_flops;        /* real flops of the Schur (trailing) updates of one factorisation */
  double factor_bytes;      /* bytes of the factors read by one forward+backward sweep, FP32 fronts */
  int64_t n_nonpositive_jacobians; /* Brick8 / Fluid8 Gauss points with det J <= 0 in the last
                               assembly: the reference prints a message for each and goes on
                               (cElementFEM::setupJacobian3D, element/elementfem.cpp:183-188),
                               so they are counted, not an error; a DSG4 element with
                               det J <= 0 fails the assembly with ELP_ERR_GEOMETRY as the
                               reference throws (setupJacobian2D, elementfem.cpp:97-100) */
  int64_t factor_stored;    /* complex entries of the factors kept per frequency (L and U:
                               p^2 + 2 p b per front)                                        */
  int64_t front_pool_peak;  /* most complex entries of full m x m fronts alive at once when the
                               tree levels are factorised in order                           */
  int64_t front_pool;       /* complex entries of the front pool per frequency (first-fit
                               regions, >= front_pool_peak); the workspace per frequency is the
                               pool plus the factors (factor_stored), not the sum of all m^2  */
  /* Device memory, for capacity planning (and what the serving loop charges
   * against its budget): the model's resident arrays (value arrays, pattern,
   * right-hand side, element lists, symbolic maps), and the workspace of ONE
   * frequency slot per precision [ELP_FP64_PLAIN, ELP_MIXED] and front store
   * [whole fronts, compact factor store]; a batch of S frequencies takes S
   * times that. Workspace figures are 0 before the symbolic phase.          */
  int64_t device_array_bytes;
  int64_t workspace_bytes_per_frequency[2][2];
} elp_model_info;

/* precision of the numeric factorisation */
#define ELP_FP64_PLAIN 0   /* FP64 fronts, FP64 refinement (the drop-in)       */
#define ELP_MIXED 1        /* FP32 fronts (tensor-core Schur updates) + FP64 refinement */

typedef struct {
  double rel_residual;     /* ||f - A u||_2 / ||f||_2, computed in FP64          */
  double growth;           /* max |U| / max |A| over fronts (pivot growth)       */
  int iterations;          /* refinement iterations taken                        */
  int static_pivots;       /* pivots replaced by the static-pivot floor          */
  int converged;           /* rel_residual <= tolerance                          */
  double ms_combine, ms_factor, ms_solve, ms_refine; /* device time per phase    */
} elp_solve_info;

/* ---- model lifetime ---------------------------------------------------- */

/* Copies the description, numbers DOFs (analysis.cpp:475-520), builds the
 * CSR pattern (analysis.cpp:806-867 + 1238-1246, interface blocks
 * elementinterfacestructural.cpp:152-179; negative rows dropped, explicit
 * zeros kept, diagonal always present), BC rows (analysis.cpp:366-454) and
 * the nodal-force right-hand side (analysis.cpp:171-279). Host only. */
int elp_model_create(const elp_model_desc* desc, elp_model** out);

/* Integrates every element once on the GPU (one persistent launch over all
 * element types) and scatters K, M, fluid K/M and the coupling C into
 * w-independent CSR value arrays resident in HBM. Replaces the per-w
 * element loop analysisfrequencybasic.cpp:281-304. */
int elp_model_assemble(elp_model* m);

/* Arithmetic of the Brick8 / Fluid8 element contractions (no counterpart in
 * the reference, whose element code is FP64):
 *   ELP_ASSEMBLY_FP64 (default): FP64 throughout, the drop-in;
 *   ELP_ASSEMBLY_DOUBLE_FLOAT: the shape gradients and the Gauss-point sums
 *     in FP32 pairs (error-free products and sums, ~48 significant bits);
 *     J, det J and J^-1 in FP64. Entries differ from the FP64 ones by
 *     ~1e-14 of the sum of the magnitudes of their terms (well inside the
 *     1e-12 parity bar), but a residual measured against an FP64-assembled
 *     matrix then carries ~1e-14 || |A| |x| || / ||f||: keep FP64 for
 *     models whose || |A| |x| || is far above ||f|| (clamped stiff plates).
 * DSG4 plates and interface quads are FP64 in both. Setting it on an
 * assembled model re-runs the assembly. */
#define ELP_ASSEMBLY_FP64 0
#define ELP_ASSEMBLY_DOUBLE_FLOAT 1
int elp_model_set_assembly(elp_model* m, int arithmetic);

/* Symbolic phase: nested-dissection ordering, assembly tree, front index
 * maps (once per model; the reference leaves this to MUMPS's analysis). */
int elp_model_analyse(elp_model* m);

int elp_model_get_info(const elp_model* m, elp_model_info* info);

/* CSR pattern, 0-based. row_ptr has n+1 entries, col_idx nnz. */
int elp_model_pattern(const elp_model* m, int32_t* row_ptr, int32_t* col_idx, int64_t* nnz);

/* Global row of (node index, dof) or -1 if inactive (cDegreesOfFreedom::getGlobalRow). */
int elp_model_global_rows(const elp_model* m, int32_t* rows_out /* n_nodes x 21 */);

/* Values of A(w) on the pattern after BC rows (what the reference holds in
 * m_K right before KSPSolve), complex interleaved, nnz entries. Device
 * combine, copied to the host. */
int elp_model_system_values(elp_model* m, double omega, double* values_out);

/* Right-hand side F after nodal loads and BC values, complex interleaved:
 * the w-independent part (normal-velocity loads excluded). */
int elp_model_rhs(const elp_model* m, double* f_out);

/* Right-hand side at angular frequency omega: F + (1/omega) G, G the
 * normal-velocity loads (zero on Dirichlet rows), complex interleaved. */
int elp_model_rhs_omega(const elp_model* m, double omega, double* f_out);

/* Solve A(w_k) u_k = f for n_omega angular frequencies. f == NULL uses the
 * model's own right-hand side at each w_k (elp_model_rhs_omega). x_out: n_omega x n complex interleaved.
 * info: n_omega entries (may be NULL). tol: target relative residual
 * (<= 0 selects 1e-10). */
int elp_solve(elp_model* m, const double* omegas, int n_omega, int precision,
              const double* f_or_null, double* x_out, elp_solve_info* info, double tol);

/* Cell stresses of a solution x (n complex interleaved host buffer, e.g. one
 * frequency of elp_solve's output) at angular frequency omega, computed on the
 * device (ELP_ERR_CUDA without one) as the reference computes them after a
 * solve (cAnalysis::computeStressesCells, analysis.cpp:869-905):
 * 9 complex slots per element, elements in descriptor order (blocks, then
 * elements; the reference orders them by ascending element id, Id0n).
 * Brick8: sigma at the element centre, slots 0..5
 * (elementstructurebrick.cpp:48-159); DSG4: the Mindlin plate stresses of the
 * upper surface in sigma, of the lower surface in sigma_lower, slots 0, 1, 3
 * (elementstructuremindlin.cpp:51-175); other slots and Fluid8 elements 0.
 * sigma_lower may be NULL. */
int elp_cell_stresses(const elp_model* m, double omega, const double* x, double* sigma, double* sigma_lower);

/* Nodal stresses of a solution x at omega, on the device, one thread per
 * node summing its elements in a fixed order (cAnalysis::computeStressesNodes,
 * analysis.cpp:907-935): 9 complex slots per node, nodes in ascending id
 * (GlobalSeqId). Brick8 adds its centre stress divided by the number of
 * elements at the node to slots 0..5 (elementstructurebrick.cpp:161-270);
 * Fluid8 adds grad p at each corner to slots 6..8, unaveraged
 * (elementfluid3d.cpp:380-557); DSG4 adds nothing (not implemented there). */
int elp_node_stresses(const elp_model* m, double omega, const double* x, double* sigma_nodes);

int elp_model_destroy(elp_model* m);

/* Text of the last error on the calling thread. */
const char* elp_last_error(void);

/* ---- device-resident variants (inputs/outputs already in HBM) ----------- */

/* Same as elp_solve but f_dev / x_dev are device pointers (complex
 * interleaved doubles, n_omega x n for x). stream may be 0. */
int elp_solve_device(elp_model* m, const double* omegas, int n_omega, int precision,
                     const double* f_dev, double* x_dev, elp_solve_info* info, double tol,
                     void* stream);

/* Re-runs the element integration on the device without host work, for
 * timing: returns the device time of the assembly kernel(s) in ms. */
int elp_model_time_assembly(elp_model* m, int repeats, double* ms_per_assembly,
                            double* ms_kernel_only);

/* ---- allocation-free residual check ------------------------------------ */

/* No counterpart in the reference: it exists for callers that cannot
 * allocate device memory while they run (device memory owned by another
 * framework's pool or a fixed budget that cannot grow, an embedding that
 * forbids allocation after start-up, a loop that must not pay the implicit
 * synchronisation of cudaMalloc / cudaFree). Computes r = f - A(w_k) x_k and
 * ||r||_2 / ||f||_2 for n_omega <= ELP_NOALLOC_MAX_OMEGA frequencies of an
 * assembled model; f_dev, x_dev, r_dev are the caller's device buffers
 * (n_omega x n complex interleaved), rel_residual_out is host memory
 * (n_omega doubles). It calls no allocating routine: its scratch is one
 * fixed device array of about 0.5 MB that every GPU loading the library
 * keeps until the process exits. Larger n_omega is rejected with
 * ELP_ERR_ARG. All calls share that array: calls that overlap on the GPU
 * race on it. The first call on a device looks up the array's device
 * address; make it before any stream capture. The model must be assembled;
 * the symbolic phase is not needed. Its launches are not counted or timed
 * by elp_profile, so it allocates nothing with profiling on either. */
#define ELP_NOALLOC_MAX_OMEGA 64
int elp_residual_noalloc(elp_model* m, const double* omegas, int n_omega, const double* f_dev,
                         const double* x_dev, double* r_dev, double* rel_residual_out, void* stream);

/* ---- tuning and the autotuner ------------------------------------------ */

/* No reference counterpart (MUMPS and PETSc take their own parameters).
 * How a model is factorised, never what is computed; 0 or a negative value
 * takes the default (the ELP_* environment variable if set, else the value
 * measured best on the coupled plate-cavity sweep), except pack_count, where 0
 * means never and a negative value the default:
 *   leaf            nested-dissection leaf size in DOFs (128)
 *   schur_tile      columns of a converter-kernel Schur tile: 32 or 64 (64)
 *   pack_count      packed tensor-core Schur kernel on levels of at most this
 *                   many fronts (300; 0: never) ...
 *   pack_min_border ... whose largest border has at least this many rows (300)
 *   lanes           workspace lanes a batch of 16+ frequencies is split over (4)
 * A new leaf size redoes the symbolic phase at the next solve; the other
 * knobs rebuild the workspaces. */
typedef struct {
  int leaf;
  int schur_tile;
  int pack_count;
  int pack_min_border;
  int lanes;
} elp_tuning;
int elp_model_set_tuning(elp_model* m, const elp_tuning* t);
/* The tuning in effect, defaults resolved. */
int elp_model_get_tuning(const elp_model* m, elp_tuning* t);
/* Project-written autotuner: times solves of the caller's frequencies (at
 * most 64) while it tries each knob in turn (leaf 64/128/256, tile 32/64,
 * packed levels on/off, lanes 1/2/4 for 16+ frequencies), keeps whatever
 * was fastest, leaves the model tuned so and reports the choice, the
 * seconds of its timed solve and the number of trials. */
int elp_model_autotune(elp_model* m, const double* omegas, int n_omega, int precision, elp_tuning* chosen,
                       double* seconds, int* trials);

/* ---- groups of models: frontal updates grouped across models ----------- */

/* No reference counterpart (elpasoC solves one model per process). A group
 * solves several models together as ONE system, their disjoint union, so
 * that each tree level of the multifrontal factorisation is one launch over
 * the fronts of every member, and every member's elements are integrated in
 * one pass: many small models keep the GPU busy instead of leaving it idle
 * between their own small launches. Each member keeps its own frequencies,
 * its own right-hand side (its F(w), as elp_solve with f == NULL) and its own
 * numbering; results and infos are reported per member. The members are
 * copied at creation (the group does not refer to them later); their
 * loss-factor groups are merged by value, at most 8 distinct in a group.
 * Convergence is per member: the mixed path runs one Krylov process per
 * (member, frequency) with its own stopping test; the plain path's
 * refinement freezes each member once it reaches tol. A hard member fails
 * only itself. Each member's residual is measured on its own rows and
 * reported in its info. */
typedef struct elp_group elp_group;
int elp_group_create(elp_model* const* models, int n_models, elp_group** out);
/* Sizes of the combined system (n_dofs, nnz, fronts, ... of all members). */
int elp_group_info(const elp_group* g, elp_model_info* info);
/* omegas: n_models x n_omega angular frequencies, member-major (member k's
 * at omegas[k * n_omega + j]); x_out: member k's n_omega x n_k solutions
 * (complex interleaved) after the earlier members' blocks; info (may be
 * NULL): n_models x n_omega, member-major. Status as elp_solve. */
int elp_group_solve(elp_group* g, const double* omegas, int n_omega, int precision, double* x_out,
                    elp_solve_info* info, double tol);
int elp_group_destroy(elp_group* g);
/* Tuning of a group's combined system, and its autotuner (as for a model;
 * omegas as for elp_group_solve). */
int elp_group_set_tuning(elp_group* g, const elp_tuning* t);
int elp_group_autotune(elp_group* g, const double* omegas, int n_omega, int precision, elp_tuning* chosen,
                       double* seconds, int* trials);

/* ---- fault injection for failure-path tests ---------------------------- */

/* No counterpart in the reference. Arms one host-side fault, made on the host
 * so that no test has to fault the GPU: it fires on the `countdown`-th
 * matching event after the call (1: the next one), once.
 *   ELP_FAULT_DEVICE_ALLOC: a device allocation of the library reports an
 *     allocation failure without calling the allocator (the call in progress
 *     returns ELP_ERR_NOMEM and leaves the model usable);
 *   ELP_FAULT_HOST_ALLOC: a host allocation point of model creation or of
 *     the host symbolic phase throws std::bad_alloc (ELP_ERR_NOMEM);
 *   ELP_FAULT_TC_WAIT: a packed tensor-core Schur launch runs with its
 *     producer issuing no copy and every wait bounded at 2^14 polls, so its
 *     MMA and epilogue waits run out with no copy or MMA in flight; the
 *     kernel sets its error flag and returns, and the solve returns
 *     ELP_ERR_CUDA;
 *   ELP_FAULT_NONE disarms all. */
#define ELP_FAULT_NONE 0
#define ELP_FAULT_DEVICE_ALLOC 1
#define ELP_FAULT_HOST_ALLOC 2
#define ELP_FAULT_TC_WAIT 3
int elp_fault_inject(int kind, int countdown);

/* ---- kernel test hook --------------------------------------------------- */

/* No counterpart in the reference. Runs ONE front update of the mixed path's
 * factorisation on caller-given FP32 complex fronts, so that its tensor-core
 * arithmetic can be checked against a plain FP64 product. fronts: `slots`
 * fronts one after another, each m x m column-major (m = p + b), complex
 * interleaved floats, updated in place; k0 = 32 step:
 *   ELP_KERNEL_GEMM_COL:   F[k0:m, k0:k0+32] -= F[k0:m, 0:k0] F[0:k0, k0:k0+32]
 *   ELP_KERNEL_GEMM_ROW:   F[k0:k0+32, k0+32:m] -= F[k0:k0+32, 0:k0] F[0:k0, k0+32:m]
 *   ELP_KERNEL_GEMM_SCHUR: S = F[p:m, p:m] - F[p:m, 0:p] F[0:p, p:m]; written
 *     into F, or with `parents` (slots x parent_m^2 complex, same layout) added
 *     into parent[pmap[i], pmap[j]] instead (the extend-add fused into the
 *     update), F left as it was;
 *   ELP_KERNEL_PACKED_SCHUR: S added into the parents through the packed
 *     operands (split once into TF32 planes, bulk-copied by the MMA kernel);
 *   ELP_KERNEL_GEMM_SCHUR_32: as ELP_KERNEL_GEMM_SCHUR with 128 x 32 tiles
 *     (the narrow tile the tuning may select).
 * pmap: b distinct parent positions. Returns ELP_ERR_ARG for inconsistent
 * sizes. */
#define ELP_KERNEL_GEMM_COL 0
#define ELP_KERNEL_GEMM_ROW 1
#define ELP_KERNEL_GEMM_SCHUR 2
#define ELP_KERNEL_PACKED_SCHUR 3
#define ELP_KERNEL_GEMM_SCHUR_32 4
int elp_front_update_test(int kernel, int p, int b, int step, int slots, float* fronts, int parent_m,
                          const int32_t* pmap, float* parents);

/* ---- launch counting and per-kernel device timing ---------------------- */

/* Kernel classes, in the order of the arrays below:
 *  0 assemble, 1 dscale, 2 scatter, 3 panel, 4 border, 5 urow, 6 gemm,
 *  7 extend_add, 8 forward, 9 backward, 10 residual, 11 norms, 12 rhs,
 *  13 update, 14 values, 15 gemm_tc (tensor-core Crout and Schur updates
 *  from the fronts), 16 spmv, 17 fwd_border, 18 bwd_u12, 19 krylov (GMRES
 *  vector kernels), 20 schur_tc (tensor-core Schur update from packed
 *  operands), 21 pack (TF32 split of the packed operands).
 * No reference counterpart (the reference times whole phases with
 * cStopwatch, basics/watch/stopwatch.cpp:35-64). elp_profile(1) resets the
 * counters and records a CUDA event pair around every launch on its stream;
 * elp_profile(0) resets and counts launches only. */
int elp_profile(int enable);
#define ELP_PROFILE_CLASSES 22
int elp_profile_read(double* ms /* [ELP_PROFILE_CLASSES] */, int64_t* launches, int64_t* timed,
                     int* n_classes);

/* Measured FP64 FMA throughput of the current device in TFLOP/s (a chain of
 * independent FMAs on every SM, timed with CUDA events; no reference
 * counterpart): the roofline of the FP64 kernels (plain path, assembly). */
int elp_peak_fp64(double* tflops);

/* ---- serving loop (continuous batching over resident models) ------------ */

typedef struct elp_server elp_server;

typedef struct {
  int64_t hbm_budget_bytes;  /* admission limit for resident models + work:
                                every model's resident arrays and each
                                workspace lane, charged before allocation    */
  int max_inflight;          /* worker threads: batches on the device at once */
  int precision;             /* ELP_FP64_PLAIN / ELP_MIXED                    */
  double tol;                /* relative residual target                      */
  int omega_batch;           /* most frequencies factorised together; a batch
                                takes fewer when the budget has less room     */
} elp_server_config;

typedef struct {
  int64_t request_id;
  int status;                /* ELP_OK or error code                          */
  int n_omega;
  double latency_ms;         /* arrival -> last frequency done                */
  double max_rel_residual;
} elp_request_result;

int elp_server_create(const elp_server_config* cfg, elp_server** out);
/* Registers a model; returns its slot id. The first worker that picks up
 * one of its requests charges the model's resident arrays against the budget
 * (sized on the host, before any device allocation), then assembles and
 * analyses it if needed; a model whose arrays plus a one-frequency workspace
 * exceed the budget fails its requests with ELP_ERR_NOMEM. Models may be
 * added while batches run. Once registered, the model belongs to the server
 * until the server is destroyed: the caller must not use the handle, and
 * the server releases workspaces the model made before. */
int elp_server_add_model(elp_server* s, elp_model* m, int* model_id);
/* Queues a sweep request. x_out (n_omega x n complex) must stay valid until
 * the result is returned by elp_server_wait. */
int elp_server_submit(elp_server* s, int model_id, const double* omegas, int n_omega,
                      double* x_out, int64_t* request_id);
/* Waits for the next completed request (timeout_ms < 0: wait forever). */
int elp_server_wait(elp_server* s, elp_request_result* result, double timeout_ms);
int elp_server_destroy(elp_server* s);

#ifdef __cplusplus
}
#endif
#endif /* ELPASO_GB300_H */
