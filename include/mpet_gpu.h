/*
 * mpet_gpu.h - C ABI of libmpetgpu, the GB300 (sm_103a) assemble + solve
 * engine for the backward-Euler / theta-scheme MPET block system of
 * waterscapes' mpet.MPETSolver.
 *
 * The reference is pure Python on top of DOLFIN/PETSc; there is no native
 * FFI in it.  Each entry point below replaces one native call that
 * MPETSolver makes through DOLFIN or PETSc (file:line in the reference's
 * src/mpet/mpet/ tree), so that a Python MPETSolver can keep its API and
 * call this library through ctypes instead.
 *
 * Conventions
 *  - Every function returns an int status: MPET_OK (0) or a negative
 *    MPET_ERR_* code.  Nothing aborts or traps; the text of the last error
 *    is available from mpet_last_error().
 *  - Arrays named *_host are host memory.  All other array arguments are
 *    device pointers (CUDA global memory on the context's device), e.g.
 *    torch.Tensor.data_ptr() of a CUDA tensor.
 *  - Work is ordered on the context's stream (mpet_set_stream; default:
 *    a stream the context creates).  One context per host thread.
 *  - Global DOF order ("block natural"): P2 nodes are the vertices
 *    followed by the edges sorted by (low, high) vertex id; displacement
 *    DOF (node i, component k) = 3*i + k; pressure DOF of network a at
 *    vertex v = Nu + a*nv + v with Nu = 3*(nv + ne).
 */
#ifndef MPET_GPU_H
#define MPET_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPET_OK 0
#define MPET_ERR_INVALID (-1)   /* bad argument or size */
#define MPET_ERR_NOMEM (-2)     /* device or host allocation failed */
#define MPET_ERR_CUDA (-3)      /* CUDA runtime error */
#define MPET_ERR_MAXIT (-4)     /* Krylov iteration limit reached */
#define MPET_ERR_BREAKDOWN (-5) /* Krylov breakdown (indefinite preconditioner, NaN) */
#define MPET_ERR_TIMEOUT (-6)   /* a bounded device wait gave up */
#define MPET_ERR_STATE (-7)     /* call order violated (e.g. solve before setup) */

#define MPET_MAX_NETWORKS 8

#define MPET_PRECISION_FP64 0  /* FP64 matrix, FP64 MINRES, FP64 AMG */
#define MPET_PRECISION_MIXED 1 /* FP32 inner MINRES + AMG inside FP64 refinement */

/* Block systems.  MPET_FORM_MPET: u and the J network pressures (MPETSolver,
 * src/mpet/mpet/mpetsolver.py:196-261).  MPET_FORM_TOTAL_PRESSURE: u, the
 * total pressure p0 = lmbda div u - sum_i alpha_i p_i and the networks
 * (MPETTotalPressureSolver, src/mpet/mpet/mpettotalpressuresolver.py:262-305);
 * pressure field 0 is p0 and fields 1..J-1 the networks, so num_networks,
 * alpha, c, K, S and the continuity markers count p0 as field 0 (alpha[0] = 1
 * weights p0 in the rank-one term, c[0] = K[0] = S[0][*] = S[*][0] = 0, and
 * field 0 carries no boundary condition). */
/* Krylov methods.  AUTO: MINRES when the transfer matrix S is symmetric (the
 * system is then symmetric), restarted GMRES with the same block-diagonal
 * preconditioner (right-preconditioned) otherwise; the reference's direct
 * solve has no such restriction (S = ((0, 2), (1, 0)) in
 * src/mpet/test/test_convergence_mpetsolver.py:112-118). */
#define MPET_KRYLOV_AUTO 0
#define MPET_KRYLOV_MINRES 1
#define MPET_KRYLOV_GMRES 2

#define MPET_FORM_MPET 0
#define MPET_FORM_TOTAL_PRESSURE 1

typedef struct mpet_ctx mpet_ctx;

/* Problem and solver parameters.  Material keys follow MPETProblem.params
 * (src/mpet/mpet/mpetproblem.py:169-180, J/alpha/K/S/c with E,nu converted
 * to mu,lmbda by convert_to_mu_lmbda, mpetproblem.py:13-16); theta follows
 * MPETSolver.default_params (mpetsolver.py:86-98). */
typedef struct mpet_params {
    int32_t num_networks;              /* J (A in the configs), 1..8 */
    int32_t precision;                 /* MPET_PRECISION_* */
    double mu, lmbda;                  /* Lame parameters */
    double alpha[MPET_MAX_NETWORKS];   /* Biot-Willis coefficients */
    double c[MPET_MAX_NETWORKS];       /* storage coefficients */
    double K[MPET_MAX_NETWORKS];       /* permeabilities */
    double S[MPET_MAX_NETWORKS * MPET_MAX_NETWORKS]; /* transfer, row-major J x J (stride 8) */
    double theta;                      /* theta-scheme weight */
    double rtol;                       /* relative preconditioned residual, e.g. 1e-10 */
    double inner_rtol;                 /* mixed: reduction per inner FP32 MINRES solve (<= 0: 3e-4) */
    int32_t maxit;                     /* Krylov iterations per solve (all inner solves) */
    int32_t max_outer;                 /* refinement sweeps per solve */
    double amg_theta;                  /* strength threshold, e.g. 0.1 */
    int32_t amg_cheb_degree;           /* Chebyshev smoother degree, e.g. 4 */
    int32_t amg_coarse_size;           /* dense solve below this size, e.g. 500 */
    int32_t check_every;               /* host convergence check period (iterations) */
    int32_t amg_p2_to_p1;              /* 1: displacement hierarchy starts with the P1-in-P2
                                          embedding (p-multigrid), then aggregation */
    int32_t prec_network_modes;        /* 1: the pressure blocks of the preconditioner act on the
                                          eigenmodes of the network coupling (see below), 0: on
                                          the networks (the reference form, mpetsolver.py:270) */
    double prec_u_weight;              /* w in the displacement block w (grad u, grad v) of the
                                          preconditioner; the reference form uses mu
                                          (mpetsolver.py:269), mu + lmbda balances the blocks;
                                          <= 0 means mu */
    double prec_u_shift;               /* g in + g (u, v) added to that block (keeps it definite
                                          when the displacement has no Dirichlet condition, e.g.
                                          with rigid-motion modes); 0 for none */
    int32_t formulation;               /* MPET_FORM_*: the block system assembled */
    int32_t prec_u_form;               /* displacement block of the preconditioner: 0 = the
                                          vector Laplacian w (grad u, grad v) (the reference's
                                          form family, mpetsolver.py:269); 1 = the displacement
                                          block of the system itself, smoothed-aggregation AMG
                                          with rigid-body modes (3D with node blocks, Dirichlet
                                          displacement, no batch; otherwise form 0 is used) */
    double prec_p0_weight;             /* total-pressure form: w0 in the p0 block w0 (p0, w0) of
                                          the preconditioner (the reference form uses 1,
                                          mpettotalpressuresolver.py:281); <= 0 means 1 */
    int32_t krylov;                    /* MPET_KRYLOV_*: the Krylov method of the solves */
    int32_t gmres_restart;             /* GMRES restart length (<= 0: 30, at most 64) */
    int32_t amg_cheb_degree_fine;      /* Chebyshev degree on the finest level of every
                                          hierarchy (<= 0: amg_cheb_degree) */
    int32_t inner_loop;                /* 0: each inner Krylov solve is one graph launch with a
                                          device-side loop (default); 1: three-iteration graph
                                          replays with a host check after each (test hook) */
    int32_t amg_cheb_degree_coarse;    /* Chebyshev degree on the levels from
                                          amg_cheb_coarse_level on, in every hierarchy
                                          (<= 0: amg_cheb_degree; the Python solver's
                                          default is 3) */
    int32_t amg_cheb_coarse_level;     /* first level that takes amg_cheb_degree_coarse
                                          (<= 0: 2) */
    int32_t prec_u_order;              /* rows of the first displacement level (device set-up):
                                          0 (default) the P2 node order, 1 a spatial (Morton)
                                          order of the nodes, each 256-row window sorted by row
                                          length (slower at 64^3: 2.04 ms for the level against
                                          1.33; kept as an option) */
} mpet_params;

typedef struct mpet_stats {
    int32_t iterations;     /* total Krylov iterations */
    int32_t outer;          /* refinement sweeps (1 for FP64) */
    int32_t status;         /* MPET_OK, MPET_ERR_MAXIT or MPET_ERR_BREAKDOWN */
    int32_t pad;
    double relres;          /* final preconditioned residual / initial */
    double relres_true;     /* final ||D^-1 r||_2 / ||D^-1 b||_2 in FP64 */
} mpet_stats;

/* Context ---------------------------------------------------------------- */
int mpet_ctx_create(int device, mpet_ctx** out);
int mpet_ctx_destroy(mpet_ctx* ctx);
const char* mpet_last_error(const mpet_ctx* ctx);
int mpet_set_stream(mpet_ctx* ctx, void* cuda_stream);
int mpet_synchronize(mpet_ctx* ctx);

/* Mesh and markers (host arrays).  Replaces the DOLFIN Mesh / MeshFunction
 * inputs of MPETProblem (mpetproblem.py:103-166).  tets: nc x 4 vertex ids;
 * bfacets: nf x 3 boundary facets; markers: (1 + J) x nf, row 0 the
 * momentum markers, row 1 + a those of network a (0 Dirichlet, 1 Neumann,
 * 2 Robin, anything else unmarked). */
int mpet_mesh_upload(mpet_ctx* ctx, int64_t nv, const double* xyz_host, int64_t nc,
                     const int32_t* tets_host, int64_t nf, const int32_t* bfacets_host,
                     const int32_t* markers_host, int32_t num_networks);

/* The same for dim = 2 (triangles: cells nc x 3, boundary facets nf x 2
 * segments; coordinates still nv x 3 with z ignored) or dim = 3.  In 2D the
 * displacement has 2 components per P2 node (DOF 2*i + k) and every
 * assembly, boundary-term and solve entry point works as in 3D, as in the
 * reference's 2D tests (test_convergence_mpetsolver.py); batches and the
 * adjoint are built for tetrahedra only (MPET_ERR_INVALID in 2D). */
int mpet_mesh_upload_dim(mpet_ctx* ctx, int32_t dim, int64_t nv, const double* xyz_host, int64_t nc,
                         const int32_t* cells_host, int64_t nf, const int32_t* bfacets_host,
                         const int32_t* markers_host, int32_t num_networks);

/* Dofmap, CSR sparsity pattern and Dirichlet DOF lists, built on the GPU.
 * Replaces create_function_spaces (mpetsolver.py:100-132), DOLFIN's
 * SparsityPatternBuilder used by assemble(self.a) (mpetsolver.py:335) and
 * the topological DOF search of DirichletBC (mpetsolver.py:63-84). */
int mpet_setup(mpet_ctx* ctx, const mpet_params* params);
int mpet_update_params(mpet_ctx* ctx, const mpet_params* params);
int mpet_get_sizes(mpet_ctx* ctx, int64_t* N, int64_t* nnz, int64_t* nnodes, int64_t* nedges);
/* Copies of the pattern (row_ptr N+1, col nnz) and the edge list (2 x ne). */
int mpet_get_pattern(mpet_ctx* ctx, int64_t* row_ptr_host, int32_t* col_host);
int mpet_get_edges(mpet_ctx* ctx, int64_t* edges_host);

/* Matrix assembly: assemble(self.a) + Robin axpy + bc.apply(A)
 * (mpetsolver.py:335-344 / 412-419).  apply_bc != 0 replaces Dirichlet
 * rows by unit rows (DirichletBC.apply).  In mixed precision an FP32 copy
 * of the values is written in the same pass. */
int mpet_assemble(mpet_ctx* ctx, double dt, int32_t apply_bc);
int mpet_get_values(mpet_ctx* ctx, double* values_host);

/* Dirichlet data.  field 0 = displacement (DirichletBC(VP.sub(0)),
 * mpetsolver.py:74), field 1 + a = network a (mpetsolver.py:81).
 * mpet_get_bc copies the DOF ids and their coordinates (count x 3) into
 * device arrays; mpet_set_bc_values takes the values at those DOFs
 * (device array, same order; displacement values node-major). */
int mpet_get_bc_count(mpet_ctx* ctx, int32_t field, int64_t* count);
int mpet_get_bc(mpet_ctx* ctx, int32_t field, int32_t* dofs, double* coords);
int mpet_set_bc_values(mpet_ctx* ctx, int32_t field, const double* values);

/* Sources as Lagrange interpolants at the current step (device arrays or
 * NULL for zero): f at P2 nodes (nnodes x 3, node-major), g of network a at
 * vertices (J x nv).  They enter b exactly as the reference's L0 / L1 dx
 * terms (mpetsolver.py:233, 249). */
int mpet_set_sources(mpet_ctx* ctx, const double* f_nodes, const double* g_vertices);

/* Per-cell permeabilities (device array J x nc, cell order of the upload;
 * NULL = the constants params.K).  K_a as a DG0 field in the form
 * -dt (K_a grad pm_a, grad q_a) (mpetsolver.py:200) and in the preconditioner
 * (:270); the matrix and preconditioner must be rebuilt afterwards. */
int mpet_set_cell_permeability(mpet_ctx* ctx, const double* K_cells);

/* Rigid-motion nullspace of the displacement (MPETProblem.u_has_nullspace,
 * mpetsolver.py:115-124, 204-207, basis of rm_basis_L2.py:10-74): Z is a
 * device array nz x Nu (nz = 3 in 2D, 6 in 3D) of the modes' nodal values in
 * the displacement DOF layout, L2-orthonormal.  The reference adds one
 * multiplier r_i per mode, r_i (Z_i, u) + z_i (Z_i, v); rigid motions are
 * divergence-free, so they span the kernel of the coupled operator and each
 * solve takes r_i = Z_i^T b_u, removes sum_i r_i M Z_i from the right-hand
 * side, solves the consistent singular system and projects the displacement
 * to (Z_i, u) = 0.  The displacement may have no Dirichlet DOFs (else
 * MPET_ERR_INVALID).  mpet_get_rigid_multipliers returns the r_i of the last
 * solve. */
int mpet_set_rigid_modes(mpet_ctx* ctx, int32_t nz, const double* Z);
int mpet_get_rigid_multipliers(mpet_ctx* ctx, double* r_host);

/* Constant-pressure constraints (the reference's p_has_nullspace,
 * src/mpet/mpet/mpetsolver.py:120-124, 209-215): for each listed network
 * (without Dirichlet DOFs) the constraint int p_a = 0 with a Lagrange
 * multiplier p_null (an R-space unknown in the reference), solved by the
 * Schur complement of the multipliers (nq extra solves after each assembly).
 * The preconditioner block of such a network gets + dt theta K_a / diam^2 (p, w).
 * mpet_get_pressure_multipliers writes the nq multipliers of the last solve. */
int mpet_set_pressure_constraints(mpet_ctx* ctx, int32_t nq, const int32_t* networks);
int mpet_get_pressure_multipliers(mpet_ctx* ctx, double* lambda_host);

/* Per-cell storage coefficients c_a (device array J x nc) and transfer
 * coefficients S_ab (J x J x nc, S_cells[(a J + b) nc + cell], symmetric in
 * a, b per cell for MINRES); either may be NULL (= the constants of
 * params).  The DG0 forms of c_a and S_ab in mpetsolver.py:200-201 and the
 * preconditioner (:270); used for batches of independent instances with
 * their own parameters in one mesh.  The matrix and preconditioner must be
 * rebuilt afterwards. */
int mpet_set_cell_coefficients(mpet_ctx* ctx, const double* c_cells, const double* S_cells);

/* Declare the uploaded mesh a batch of ninst independent instances (disjoint
 * instance meshes in one upload; vertex_instance: host array, the instance
 * of every vertex).  The system and the preconditioner stay one block-
 * diagonal operator run by the same kernels; the solves then converge every
 * instance to params.rtol on its own (per-instance residual scaling and
 * stopping; the stats report the worst instance).  No reference counterpart:
 * the reference runs one problem per MPETSolver.  MPET_ERR_INVALID if an
 * edge joins two instances. */
int mpet_set_batch(mpet_ctx* ctx, int32_t ninst, const int32_t* vertex_instance);

/* Per-instance relative preconditioned residual of the last batch solve
 * (host array of ninst). */
int mpet_get_batch_relres(mpet_ctx* ctx, double* relres_host);

/* Boundary facets (the nf facets of mpet_mesh_upload, same order): their P2
 * nodes (nf x 6: the three vertices ascending, then the edges (1,2), (0,2),
 * (0,1)) and area + outward unit normal (nf x 4), copied into device arrays
 * so that facet data can be evaluated at those nodes. */
int mpet_get_facet_data(mpet_ctx* ctx, int32_t* facet_nodes, double* area_normal);

/* Facet data as Lagrange interpolants (device arrays, NULL = none):
 *  MPET_FACET_TRACTION           s at the 6 facet P2 nodes, nf x 6 x 3 (used on
 *                                momentum marker 1: (s, v) ds_m(1) in L0, mpetsolver.py:233)
 *  MPET_FACET_FLUX               I_a at the 3 facet vertices, J x nf x 3 (marker 1:
 *                                dt (I_a, q_a) ds(1) in L1, :249)
 *  MPET_FACET_ROBIN_BETA         beta_a at t0 + theta dt, J x nf x 3 (marker 2, rhs(F2a), :252-254)
 *  MPET_FACET_ROBIN_PRESSURE     p_robin_a at t0 + theta dt, J x nf x 3
 *  MPET_FACET_ROBIN_BETA_MATRIX  beta_a for the Robin matrix lhs(F2a) added by
 *                                mpet_assemble (A.axpy, :336-338), J x nf x 3 */
#define MPET_FACET_TRACTION 0
#define MPET_FACET_FLUX 1
#define MPET_FACET_ROBIN_BETA 2
#define MPET_FACET_ROBIN_PRESSURE 3
#define MPET_FACET_ROBIN_BETA_MATRIX 4
int mpet_set_facet_data(mpet_ctx* ctx, int32_t kind, const double* values);

/* Right-hand side: assemble(L) + sum assemble(L1) + assemble(L0) and
 * bc.apply(b) (mpetsolver.py:356-376).  up_prev and b are device arrays
 * of length N. */
int mpet_rhs(mpet_ctx* ctx, double dt, const double* up_prev, double* b);

/* Which displacement block the preconditioner runs: 1 = elasticity AMG
 * (prec_u_form 1 and applicable), 0 = the vector Laplacian. */
int mpet_get_prec_info(mpet_ctx* ctx, int32_t* u_elasticity);

/* Where the last mpet_setup_preconditioner went (ms, wall clock): ms4_host[0]
 * the preconditioner blocks assembled on the GPU, [1] their downloads, [2]
 * the host set-up of every hierarchy (run concurrently), [3] uploads and
 * SpMV autotuning.  No reference counterpart
 * (measurement of what hypre's set-up does inside PETSc, mpetsolver.py:507). */
int mpet_get_setup_timing(mpet_ctx* ctx, double* ms4_host);

/* Where mpet_setup_preconditioner builds the smoothed-aggregation
 * hierarchies of the Laplacian-form blocks: 1 (default) on the GPU, from the
 * blocks where they are assembled (strength, prolongator smoothing, Galerkin
 * products and transposes in device kernels; the greedy aggregation pass and
 * the coarsest dense inverse on the host); 0 on the host (blocks downloaded,
 * hierarchies built by CPU threads, uploaded).  Both follow the same recipe
 * and give the same hierarchies up to the rounding of their spectral-radius
 * estimates.  Replaces the set-up half of the reference's hypre BoomerAMG
 * (PETScKrylovSolver("minres", "hypre_amg"), src/mpet/mpet/mpetsolver.py:507;
 * mpettotalpressuresolver.py:448).  The next set-up rebuilds everything. */
int mpet_set_amg_setup(mpet_ctx* ctx, int32_t where);

/* The SpMV variant the set-up autotuner chose for each level of hierarchy
 * `block` (bits as for the system matrix; 8: the system's displacement block,
 * 16: matrix-free first level): its operator, prolongation and restriction
 * (-1 on the coarsest level).  Arrays of mpet_get_amg_info's level count; any
 * may be NULL.  No reference counterpart (tuning report). */
int mpet_get_amg_variants(mpet_ctx* ctx, int32_t block, int32_t* a_variant, int32_t* p_variant, int32_t* r_variant);

/* Where the last device set-up (mpet_set_amg_setup(ctx, 1)) spent its time,
 * summed over its hierarchies (ms): ms8[0] block copies, [1] diagonals and
 * spectral radii, [2] strength graphs and aggregation, [3] tentative and
 * smoothed prolongators, [4] transposes, [5] Galerkin products, [6] coarsest
 * inverses, [7] FP32 copies, SpMV layouts and autotuning.  No reference
 * counterpart (set-up report). */
int mpet_get_amg_setup_phases(mpet_ctx* ctx, double* ms8);

/* Copies out level `level` of hierarchy `block` (0 displacement, 1..J the
 * networks): which = 0 its operator, 1 its prolongation (FP64 CSR, int64 row
 * pointers).  Each output may be NULL; call once with rp, ci, v NULL for the
 * sizes (n rows, m columns, nnz entries), then with arrays of n + 1, nnz and
 * nnz elements.  No reference counterpart (inspection and test hook). */
int mpet_get_amg_matrix(mpet_ctx* ctx, int32_t block, int32_t level, int32_t which, int64_t* n, int64_t* m,
                        int64_t* nnz, int64_t* rp, int32_t* ci, double* v);

/* Block-diagonal preconditioner (mpetsolver.py:264-271): one smoothed-
 * aggregation AMG hierarchy per diagonal block, built for this dt. */
int mpet_setup_preconditioner(mpet_ctx* ctx, double dt);
int mpet_get_amg_info(mpet_ctx* ctx, int32_t block, int32_t* levels, int64_t* sizes_host,
                      int64_t* nnz_host);

/* Per-level cost of one hierarchy (block 0: displacement, a >= 1: pressure
 * block a), in the context's precision: ms_host[k] = median time (ms) of a
 * V-cycle started at level k over `reps` launches, each from a flushed L2;
 * bytes_host[k] = the algorithmic bytes of level k's own work (every matrix
 * entry and row pointer once per product, every vector once per read or
 * write).  Level k's own time is ms_host[k] - ms_host[k+1].  Arrays hold 16
 * entries.  No reference counterpart (measurement of the preconditioner
 * that hypre applies inside PETSc, mpetsolver.py:507-556). */
int mpet_profile_vcycle(mpet_ctx* ctx, int32_t block, int32_t reps, int32_t* nlev, double* ms_host,
                        double* bytes_host);

/* Solve A x = b with the assembled (BC-applied) matrix; x holds the
 * initial guess on entry (its Dirichlet entries are replaced by the BC
 * values).  Replaces LUSolver(A, "mumps").solve / PETScKrylovSolver
 * ("minres", "hypre_amg").solve (mpetsolver.py:379, 456, 556). */
int mpet_solve(mpet_ctx* ctx, const double* b, double* x, mpet_stats* stats);

/* One time step from up_prev: rhs (with the BC values and sources last
 * set) and solve into up (initial guess up_prev).  MPETSolver.step without
 * the matrix assembly, i.e. one pass of the solve_direct time loop
 * (mpetsolver.py:424-462). */
int mpet_step(mpet_ctx* ctx, double dt, const double* up_prev, double* up, mpet_stats* stats);

/* z = M^-1 r with the block-diagonal AMG preconditioner (one V-cycle per
 * block); r, z device arrays of length N in the hierarchy's precision (FP32
 * for MPET_PRECISION_MIXED, FP64 otherwise).  The preconditioner the
 * reference's iterative path hands to PETSc (solver.set_operators(A, P),
 * mpetsolver.py:553). */
int mpet_apply_preconditioner(mpet_ctx* ctx, int32_t precision, const void* r, void* z);

/* FP64 residual r = b - A x of the assembled (Dirichlet-row) system and its
 * Jacobi-scaled norms: norms_host[0] = ||D^-1 r||_2, norms_host[1] =
 * ||D^-1 b||_2 (D = |diag A|).  The relative residual the reference's Krylov
 * path monitors (PETScKrylovSolver.solve, mpetsolver.py:556) in the
 * diagonally scaled norm; the reduction uses the context's scratch. */
int mpet_residual(mpet_ctx* ctx, const double* b, const double* x, double* r, double* norms_host);

/* Same result as mpet_residual for callers that cannot allocate device
 * memory (their allocator already holds the device's free memory, or they
 * may not allocate after start-up).  No counterpart in the reference: it
 * exists only for such callers.  It allocates nothing: the reduction scratch
 * is a 256 KiB static device array that every GPU on which a context was
 * created keeps until exit, so the system may have at most 33,554,432 rows
 * (larger systems get MPET_ERR_INVALID).  mpet_ctx_create looks up the
 * array's device address (and so loads it onto the device); if that failed,
 * the first call on the device retries and should come before any stream
 * capture.  The call synchronises the context's stream, since it returns the
 * norms to the host.  Calls that overlap on the GPU share the array and
 * race. */
int mpet_residual_noalloc(mpet_ctx* ctx, const double* b, const double* x, double* r, double* norms_host);

/* y = A x with the assembled values; precision selects FP64 (x, y double)
 * or the FP32 copy (x, y float).  Used by tests and the bandwidth bench. */
int mpet_spmv(mpet_ctx* ctx, int32_t precision, const void* x, void* y);

/* apply_symmetric / MatZeroRowsColumns (src/mpet/mpet/bc_symmetric.py:11-22):
 * zero the Dirichlet columns of the assembled matrix in place (rows were
 * replaced by mpet_assemble).  b, if not NULL, is lifted with x_bc. */
int mpet_apply_symmetric(mpet_ctx* ctx, double* b, const double* x_bc);

/* Set-up autotuning of the system-matrix SpMV: ms per launch (from a
 * flushed L2) of the variants 0..5, indexed by the variant bits (bit 0: 8
 * instead of 4 entries per lane per batch; bit 1: CSR rows staged in shared
 * memory by bulk copies; bit 2: SELL-32 copy, one thread per row), and in
 * ms7_host[6] of variant 8 (node-block copy: one column id per 3x3, 3xJ, Jx3
 * or JxJ block of a P2 node's or vertex's rows), 0 where not applicable; and
 * the chosen variant.  No reference counterpart (engine introspection for
 * benchmarks). */
int mpet_get_spmv_tuning(mpet_ctx* ctx, double* ms7_host, int32_t* chosen);

/* The same for the FP64 products of the system matrix (the refinement
 * residual).  In mixed precision they are tuned apart from the FP32 copy,
 * with the residual epilogue they run with; otherwise this repeats
 * mpet_get_spmv_tuning.  No reference counterpart (tuning report). */
int mpet_get_spmv_tuning_fp64(mpet_ctx* ctx, double* ms7_host, int32_t* chosen);

/* Size of the node-block copy: blocks of the matrix (one column id each) and
 * stored values including padding.  No reference counterpart. */
int mpet_get_node_block_info(mpet_ctx* ctx, int64_t* blocks, int64_t* stored_values);

/* Override the autotuned system-matrix SpMV variant (bits as above) for the
 * products of both precisions;
 * MPET_ERR_INVALID if the variant cannot run on this matrix.  Every variant
 * computes the same product (summation order differs).  No reference
 * counterpart (tuning and test hook). */
int mpet_set_spmv_variant(mpet_ctx* ctx, int32_t variant);

/* First level of the displacement preconditioner hierarchy (the block
 * w (grad u, grad v) of mpetsolver.py:269 on P2 nodes): its products formed
 * matrix-free from per-cell data (mode 1), from its CSR copy (0), or chosen
 * per set-up by timing both (-1, default).  Takes effect at the next
 * mpet_setup_preconditioner.  mpet_get_prec_matrix_free reports the choice
 * and the two timed medians (ms; 0 when not timed).  No reference
 * counterpart (engine option, tuning report and test hook). */
int mpet_set_prec_matrix_free(mpet_ctx* ctx, int32_t mode);
int mpet_get_prec_matrix_free(mpet_ctx* ctx, int32_t* used, float* ms2_host);

/* Which kernel computes the displacement element blocks of tetrahedra (the
 * 30 x 30 part of the element matrix, mpetsolver.py:196-201): 1 (default) the
 * tensor cores (tcgen05 MMAs on exact 11-bit slices of the FP64 element
 * features, combined in 64-bit integers), 0 the FP64 CUDA-core kernel.  Both
 * give FP64 values; the next mpet_assemble uses the choice.  No reference
 * counterpart (engine option and test hook). */
int mpet_set_element_kernel(mpet_ctx* ctx, int32_t kind);

/* Bound (in polls) of the bounded waits of the staged SpMV's tile copies
 * (default 4,194,304).  A wait that gives up sets the context's device error
 * flag; the call that launched it then returns MPET_ERR_TIMEOUT and the
 * context stays usable.  0 makes every tile wait give up at once (the copies
 * still land: the kernel then waits for them under the default bound before
 * it exits), which is how the timeout path is tested without a fault.  No
 * reference counterpart (test hook). */
int mpet_set_wait_limit(mpet_ctx* ctx, int32_t polls);

/* Batches: whether the system and preconditioner products of the batched
 * inner iterations skip the rows of instances that have converged (1, the
 * default) or run over every instance (0).  The results of the instances
 * still iterating are the same either way; skipping makes an iteration cost
 * what the unconverged instances need.  Takes effect at the next solve;
 * set before mpet_setup_preconditioner, it also lets the set-up autotuner
 * offer the staged CSR kernel again (which cannot skip).  No reference
 * counterpart (engine option and test hook). */
int mpet_set_batch_skip(mpet_ctx* ctx, int32_t on);

/* The same override for every matrix of the AMG hierarchies (operators,
 * prolongations, restrictions): each takes the variant where it can run and
 * the CSR register kernel (0) elsewhere, until the next
 * mpet_setup_preconditioner.  No reference counterpart (test hook). */
int mpet_set_hierarchy_spmv_variant(mpet_ctx* ctx, int32_t variant);

/* Timing counters (CUDA events on the context's stream), cumulative since
 * the context was created: ms spent replaying the MINRES iteration graph
 * and the iterations it ran, ms of whole solves (refinement sweeps
 * included), and the kernels launched.  No reference counterpart. */
int mpet_get_timing(mpet_ctx* ctx, double* inner_ms, int64_t* inner_iterations,
                    double* solve_ms, int64_t* kernel_launches);

/* ---- a posteriori error indicators (AdaptiveMPETSolver) --------------------
 * DG0 indicators of src/mpet/mpet/adaptivempetsolver.py:82-155 for the step
 * up_prev -> up (device vectors of length N) with time step dt:
 * eta_p[K] (zeta_p_K), eta_u[K] (zeta_u_K), eta_u_dt[K] (zeta_u_dt_K), one
 * device double per cell each, and the scalar R4p (:148-155) into *r4p_host.
 * f_nodes / f_prev_nodes: body force at the current and previous time at the
 * P2 nodes (nnodes x dim, NULL = 0); g_vert: sources at the vertices (J x nv,
 * NULL = 0).  Interior facets, built once by the caller: ifacets (n_ifacets x 4
 * int32: cell+, local vertex of cell+ opposite the facet, cell-, its local
 * opposite vertex; local numbering of the ascending-sorted cell) and
 * cell_facets (nc x (dim+1) int32: the interior facet opposite each local
 * vertex, -1 on the boundary); both are range-checked on the device first.
 * MPET form, scalar K, c, S and no batch only (MPET_ERR_INVALID otherwise). */
int mpet_error_indicators(mpet_ctx* ctx, double dt, const double* up, const double* up_prev,
                          const double* f_nodes, const double* f_prev_nodes, const double* g_vert,
                          int64_t n_ifacets, const int32_t* ifacets, const int32_t* cell_facets,
                          double* eta_p, double* eta_u, double* eta_u_dt, double* r4p_host);

/* ---- discrete adjoint with respect to per-cell permeability ----------------
 * The reference has no adjoint; these entry points differentiate the
 * solve_direct time loop (mpetsolver.py:382-462) as this library discretises
 * it, with respect to the per-cell K_a fields of mpet_set_cell_permeability.
 * All vectors are device arrays of length N unless stated otherwise. */

/* Final-pressure misfit 1/2 sum_a (p_a - p*_a)^T M (p_a - p*_a), M the P1
 * mass matrix, of the state up against p_target (J x nv, network-major).
 * Writes the value to *loss_host and, when dloss is not NULL, its gradient
 * with respect to up (zero on the displacement rows). */
int mpet_pressure_misfit(mpet_ctx* ctx, const double* up, const double* p_target, double* loss_host,
                         double* dloss);

/* out = B^T lam with its Dirichlet rows zeroed, B the old-state operator of
 * the right-hand side (the rows -alpha_a (div u, q) - c_a (p_a, q)
 * + dt (1-theta) [K_a (grad p_a, grad q) + sum_b S_ab (p_a - p_b, q)]): the
 * seed of the adjoint step one step earlier.  MPET_ERR_INVALID for theta < 1
 * with Robin terms set (their (1-theta) part is not differentiated). */
int mpet_adjoint_rhs(mpet_ctx* ctx, double dt, const double* lam, double* out);

/* One adjoint step: solve A^T lam = seed with lam zero on the Dirichlet DOFs
 * (the seed's Dirichlet rows are ignored; A^T = A needs a symmetric S, else
 * MPET_ERR_INVALID), then, when grad_K (J x nc) is not NULL, add
 *   dt |e| grad lam_a . grad(theta p_a + (1 - theta) p_prev_a)
 * per cell e, the step's contribution to dL/dK_a(e) (dA/dK_a(e) =
 * -dt theta L_e and dB/dK_a(e) = dt (1-theta) L_e on the p_a block). */
int mpet_adjoint_step(mpet_ctx* ctx, double dt, const double* seed, const double* up_prev, const double* up,
                      double* lam, double* grad_K, mpet_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* MPET_GPU_H */
