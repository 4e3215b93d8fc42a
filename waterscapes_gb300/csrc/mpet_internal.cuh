// Internal declarations of libmpetgpu (not part of the C ABI).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mpet_gpu.h"

namespace mpet {

struct Error {
    int code;
    std::string msg;
};

[[noreturn]] inline void fail(int code, const std::string& msg) { throw Error{code, msg}; }

#define MPET_CUDA(call)                                                                  \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            ::mpet::fail(MPET_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define MPET_CHECK_LAUNCH() MPET_CUDA(cudaGetLastError())

// Device allocation tracked by the context so destroy() frees everything.
// Every allocation carries kTail spare bytes, so bulk copies whose size is
// rounded up to 16 bytes may read past the last element without leaving it.
// Simplex constants of the P2/P1 pair on triangles (D = 2) and tetrahedra
// (D = 3): vertices, edges, P2 nodes per cell; vertices and P2 nodes per
// boundary facet.  Local P2 nodes: the vertices, then the edges in UFC
// order (tet (2,3),(1,3),(1,2),(0,3),(0,2),(0,1); triangle (1,2),(0,2),(0,1)).
template <int D>
struct Simplex;
template <>
struct Simplex<3> {
    static constexpr int NV = 4, NE = 6, NN = 10, FV = 3, FN = 6;
    static constexpr int EA = 0x000112, EB = 0x123233;  // edge e = (EA >> 4e & 15, EB >> 4e & 15)
};
template <>
struct Simplex<2> {
    static constexpr int NV = 3, NE = 3, NN = 6, FV = 2, FN = 3;
    static constexpr int EA = 0x001, EB = 0x122;
};
template <int D>
__host__ __device__ __forceinline__ int edge_end(int e, int k) {
    return ((k == 0 ? Simplex<D>::EA : Simplex<D>::EB) >> (4 * e)) & 15;
}

// Scoped temporary device buffer (freed on scope exit).
struct TmpBuf {
    void* p = nullptr;
    explicit TmpBuf(size_t bytes) {
        if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
            cudaGetLastError();
            fail(MPET_ERR_NOMEM, "temporary cudaMalloc of " + std::to_string(bytes) + " bytes failed");
        }
    }
    ~TmpBuf() {
        if (p) cudaFree(p);
    }
    template <typename T>
    T* as() { return (T*)p; }
};

struct DevPool {
    static constexpr size_t kTail = 64;
    std::vector<void*> ptrs;
    template <typename T>
    T* alloc(int64_t n) {
        if (n <= 0) n = 1;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, (size_t)n * sizeof(T) + kTail);
        if (e != cudaSuccess) {
            cudaGetLastError();
            fail(MPET_ERR_NOMEM, "cudaMalloc of " + std::to_string((size_t)n * sizeof(T)) + " bytes failed");
        }
        ptrs.push_back(p);
        return (T*)p;
    }
    void release(void* p) {
        if (!p) return;
        for (auto& q : ptrs)
            if (q == p) {
                cudaFree(q);
                q = nullptr;
            }
    }
    void free_all() {
        for (auto p : ptrs)
            if (p) cudaFree(p);
        ptrs.clear();
    }
};

// CSR with int64 row pointers and int32 column ids; values in FP64 and
// (optionally) an FP32 copy sharing the same pattern.
// Node-block copy of the system matrix.  The rows of a P2 node (3
// displacement rows) and of a vertex (J pressure rows) share their columns,
// which come in blocks: 3x3 (node-node), 3xJ (node-vertex), Jx3, JxJ.  One
// column id per block; slices of 32 nodes / vertices store their blocks
// lane-interleaved (value q of block k of lane l at voff + (k*B + q)*32 + l),
// padded to the slice's widest row with zero blocks.  Within windows of 2048
// consecutive nodes (vertices) the lanes take them in order of decreasing
// row length, so the padding stays small.
struct NbSlice {
    int64_t coff, voff;  // first column id / value of the slice
    int32_t w2, w1;      // blocks per lane with node columns / vertex columns
};
struct NodeBlocks {
    int64_t nsu = 0, nsp = 0;  // node slices (displacement rows), vertex slices (pressure rows)
    NbSlice* sl = nullptr;     // nsu + nsp
    int32_t* perm = nullptr;   // (nsu + nsp) * 32: node / vertex of each slice lane, -1 past the end
    int32_t* cols = nullptr;
    float* v32 = nullptr;
    double* v64 = nullptr;
    int64_t ncols = 0, nvals = 0;  // stored (with padding)
    int64_t nblocks = 0;           // blocks of the matrix (without padding)
    int32_t* skl = nullptr;        // batches: lowest and highest instance of each slice's lanes
};

struct Csr {
    int64_t n = 0, m = 0, nnz = 0;
    int64_t* rp = nullptr;
    int32_t* ci = nullptr;
    double* v64 = nullptr;
    float* v32 = nullptr;
    int lpr = 32;  // lanes per row used by the SpMV kernels
    // Row tiles for the shared-memory staged SpMV: tiles[t]..tiles[t+1] are
    // whole rows holding at most SPMV_TILE entries (ntiles = 0: not staged).
    int32_t* tiles = nullptr;
    int ntiles = 0;
    int max_row = 0;  // longest row (entries)
    // SpMV variant: bit 0 = 8 entries per lane per batch (else 4, only with
    // 32 lanes per row, or with the SELL copy), bit 1 = shared-memory staged
    // (needs tiles; with bit 2: the SELL kernel with its epilogue loads after
    // the accumulation, 6 and 7), bit 2 = SELL-32 copy (needs s_off);
    // 8 = node-block copy (9: its FP32 kernel held to 64 registers, 4 blocks per
    // SM); 32 = SELL-32 with FP16 off-diagonals (needs s_v16)
    int variant = 0;
    // mixed precision: variant and lanes per row of the FP64 products when they
    // were tuned apart from the FP32 copy's (-1: none, use variant / lpr)
    int variant64 = -1;
    int lpr64 = 32;
    // SELL-32 copy: slices of 32 rows, column-major within a slice, padded
    // to the slice's longest row with zero values at the row's last column
    // (column 0 for empty rows); s_off[s] is the first entry of slice s
    // (nslices + 1 offsets)
    int64_t nslices = 0;
    int64_t* s_off = nullptr;
    int32_t* s_ci = nullptr;
    float* s_v32 = nullptr;
    double* s_v64 = nullptr;
    // half-precision SELL values (variant 32, FP32 products of a first AMG
    // level): off-diagonal entries as FP16 times s_h_scale (a power of two),
    // diagonal slots 0; the diagonal in FP32 (s_d32) is the exact row sum minus
    // the rounded off-diagonals, so the rounded operator keeps the row sums
    // (and the symmetry) of the original one
    __half* s_v16 = nullptr;
    float* s_d32 = nullptr;
    float s_h_scale = 1.f;
    // node-block copy (system matrix only; variant 8)
    NodeBlocks* nb = nullptr;
    // batches: per 32-row slice the lowest and highest instance of its rows
    // (lo > hi for a slice without rows); the products of the batched
    // iterations skip a slice whose instances have all converged
    int32_t* skl = nullptr;
};

struct AmgLevel {
    Csr A, P, R;       // P: n x nc (prolongation), R = P^T
    bool mf = false;   // products with A formed matrix-free from per-cell data (first displacement level)
    double* dinv64 = nullptr;
    float* dinv32 = nullptr;
    double rho = 1.0;  // spectral radius estimate of D^-1 A
    bool nb_uu = false;  // operator = displacement block of the system's node-block copy
    // work buffers, each n * nvec elements of double (reused for float)
    void* x = nullptr;
    void* b = nullptr;
    void* r = nullptr;
    void* d = nullptr;
    void* t0 = nullptr;
    void* t1 = nullptr;
    int32_t* inst = nullptr;  // batches: instance of each row
};

struct AmgHier {
    int nvec = 1;
    int cheb_degree = 3;
    int cheb_degree0 = 3;  // on the finest level
    int cheb_degree_c = 3;  // on levels cheb_level_c, ...
    int cheb_level_c = 2;
    std::vector<AmgLevel> lev;
    int64_t ncoarse = 0;
    double* cinv = nullptr;  // dense inverse of the coarsest operator, FP64
    void* pack_in = nullptr;  // padded (nvec = 4) input/output of the first level
    void* pack_out = nullptr;
    // first-level row of each P2 node and its inverse when the first level is in
    // a spatial order (owned by the context; null: node order)
    const int32_t* perm = nullptr;
    const int32_t* iperm = nullptr;
};

// Device-resident MINRES scalars (all FP64).
struct MinresScalars {
    double beta1, beta, oldb, alfa, dbar, epsln, oldeps, phibar, phi, cs, sn, gamma, delta, gbar;
    double c_r1;     // beta/oldb (0 on the first iteration)
    double c_r2;     // alfa/beta
    double inv_beta; // 1/beta
    double inv_gamma;
    double rel;      // phibar / beta1
    double flag;     // 1 = breakdown
    double nr2, nb2; // outer residual sums
    double nr, inv_nr, inv_nb;  // sqrt(nr2), 1/sqrt(nr2), 1/sqrt(nb2) (0 for 0)
    // FP32 copies of the scalars the FP32 vector kernels read, written with the
    // FP64 values: those kernels then convert nothing per element on the
    // narrow FP64 pipe
    float f_inv_beta, f_c_r1, f_c_r2, f_oldeps, f_delta, f_inv_gamma, f_phi, f_pad;
};

// Host-side setup of one SA hierarchy from an FP64 CSR (amg_setup.cpp).
struct HostCsr {
    int64_t n = 0, m = 0;
    std::vector<int64_t> rp;
    std::vector<int32_t> ci;
    std::vector<double> v;
};
struct HostAmgLevel {
    HostCsr A, P, R;
    std::vector<double> dinv;
    double rho = 1.0;
};
struct HostAmg {
    std::vector<HostAmgLevel> lev;
    int64_t ncoarse = 0;
    std::vector<double> cinv;
};
// P0, if given, is the prolongator of the first level (otherwise smoothed aggregation).
// (nthreads: OpenMP threads of this set-up, <= 0: every host thread; rho0_device: with
// P0 given, leave the first level's spectral radius to the GPU, marked rho < 0)
void amg_setup_host(HostCsr A, const HostCsr* P0, double theta, int coarse_size, int max_levels, HostAmg& out,
                    int nthreads = 0, bool rho0_device = false);
// threads for host set-ups: the affinity set, capped by a cgroup CPU quota
int host_threads();
void sym_eig(int n, const double* A, double* Q, double* lam);
// block smoothed aggregation from a first level A1 with near-nullspace B1 (A1.n x nb_cols,
// row-major) and bs unknowns per node
void amg_setup_block_host(const HostCsr& A1, const std::vector<double>& B1, int nb_cols, int bs, double theta,
                          int coarse_size, int max_levels, HostAmg& out);
double tridiag_max_eig_host(const std::vector<double>& a, const std::vector<double>& b);
bool setup_u_elasticity(mpet_ctx* c, bool fp32);
void p1_elasticity_host(int64_t nv, const std::vector<int64_t>& vptr, const std::vector<int32_t>& vadj,
                        const std::vector<int64_t>& inc_ptr, const std::vector<int32_t>& inc,
                        const std::vector<double>& geo, const std::vector<int32_t>& cells,
                        const std::vector<int64_t>& cidx, double mu, double lmbda, HostCsr& A);
// worst condition number of P(t)^-1 (C + t g diag(K)) over t = 10^(0.1 s), s = first_step..60
double network_kappa(int J, const double* C, const double* K, double g, const double* Q, const double* lam,
                     int first_step = 0);

}  // namespace mpet

struct mpet_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    mpet::DevPool pool;

    // mesh
    int dim = 3;                  // 2: triangles, 3: tetrahedra
    int64_t nv = 0, nc = 0, nf = 0, ne = 0, nnodes = 0;
    int J = 0;
    double* x = nullptr;          // nv * 3
    int32_t* cells = nullptr;     // nc * 4 (ascending vertex ids)
    int32_t* bfacets = nullptr;   // nf * 3
    int32_t* markers = nullptr;   // (1 + J) * nf
    int64_t* edge_key = nullptr;  // ne, lo * nv + hi, ascending
    int32_t* cell_nodes = nullptr;// nc * 10
    double* geo = nullptr;        // nc * 16: grad lambda_0..3 (12), |T|
    int64_t* n2_ptr = nullptr;    // P2 node adjacency
    int32_t* n2_col = nullptr;
    int64_t n2_nnz = 0;
    int64_t* n1_ptr = nullptr;    // vertices adjacent to each P2 node
    int32_t* n1_col = nullptr;
    int64_t n1_nnz = 0;
    int64_t* inc_ptr = nullptr;   // node -> (cell * 16 + local) incidence
    int32_t* inc = nullptr;
    uint16_t* rank2 = nullptr;    // nc * 100
    uint16_t* rank1 = nullptr;    // nc * 40

    // global system
    int64_t N = 0, Nu = 0, nnz = 0;
    mpet::Csr A;                  // rp/ci/v64/v32
    mpet::NodeBlocks A_nb;        // node-block copy of A
    double* dinv = nullptr;       // |diag|^-1 (1 where 0), FP64

    // Dirichlet data
    int64_t nbc_nodes[1 + MPET_MAX_NETWORKS] = {0};
    int32_t* bc_nodes[1 + MPET_MAX_NETWORKS] = {nullptr};
    int64_t nbc_dofs = 0;
    int64_t bc_off[2 + MPET_MAX_NETWORKS] = {0};  // dof offsets per field in bc_dofs
    int32_t* bc_dofs = nullptr;
    double* bc_vals = nullptr;
    uint8_t* node_bc = nullptr;   // nnodes flags (displacement)
    uint8_t* vert_bc = nullptr;   // J * nv flags
    uint8_t* dof_bc = nullptr;    // N flags

    // sources (borrowed device pointers)
    const double* f_nodes = nullptr;
    const double* g_vert = nullptr;
    const double* K_cells = nullptr;  // per-cell permeability (J x nc) or null
    const double* c_cells = nullptr;  // per-cell storage coefficient (J x nc) or null
    const double* S_cells = nullptr;  // per-cell transfer coefficients (J x J x nc) or null

    // boundary facets: P2 nodes (nf x 6), area + outward normal (nf x 4) and
    // the boundary-node -> (facet * 8 + local) incidence
    int32_t* fnodes = nullptr;
    double* fgeo = nullptr;
    int64_t* bn_ptr = nullptr;
    int32_t* bn_list = nullptr;
    // facet data (borrowed device pointers, MPET_FACET_*)
    const double* f_traction = nullptr;
    const double* f_flux = nullptr;
    const double* f_beta = nullptr;
    const double* f_probin = nullptr;
    const double* f_beta_matrix = nullptr;

    mpet_params prm{};
    bool mesh_ready = false, setup_done = false, assembled = false, precond_ready = false;
    bool values_mixed = false;
    double asm_dt = 0.0, prec_dt = -1.0;

    // preconditioner blocks
    mpet::Csr Lu;                 // mu-Laplacian on P2 nodes (pattern n2)
    mpet::Csr Pp[MPET_MAX_NETWORKS]; // P1 blocks (pattern n1 restricted to vertices)
    mpet::AmgHier amg_u;
    mpet::AmgHier amg_p[MPET_MAX_NETWORKS];

    // Krylov work
    void* kv = nullptr;           // v
    void* kr[3] = {nullptr, nullptr, nullptr};
    void* kw[3] = {nullptr, nullptr, nullptr};
    void* kd = nullptr;           // correction
    double* ox = nullptr;         // outer FP64 vectors
    double* orr = nullptr;
    double* ob = nullptr;
    unsigned char* l2_flush = nullptr;  // 256 MiB written between autotuner launches
    double* adj_b = nullptr;      // adjoint right-hand side (Dirichlet rows zeroed)
    double* adj_loss = nullptr;   // misfit value (1 double)
    double* elem_buf = nullptr;   // staged per-cell element data of the assembly, or null
    bool u_elast = false;         // displacement preconditioner block: elasticity AMG (else Laplacian)
    bool u_hier_valid = false;    // the Laplacian displacement hierarchy can be kept by the next set-up
    // matrix-free first level of the displacement hierarchy: per-cell data (nc x 8
    // floats or doubles), the float tables of its element operator, and the choice
    void* mf_cell = nullptr;
    float* mf_tab = nullptr;
    int mf_mode = -1;             // -1 autotuned, 0 CSR, 1 matrix-free (test hook)
    float mf_ms[2] = {0.f, 0.f};  // autotuner: Chebyshev product with the CSR level / matrix-free
    bool gmres = false;           // solves by restarted GMRES (non-symmetric system)
    // constant-pressure constraints (int p_k = 0, multiplier p_null_k): networks, the P1
    // load vector (int phi_v), W_k = A^-1 B_k^T (nq x N), the inverse of B W, multipliers
    int nq = 0;
    int q_net[MPET_MAX_NETWORKS] = {0};
    double* q_load = nullptr;
    double* q_W = nullptr;
    double q_Sinv[4 * MPET_MAX_NETWORKS * MPET_MAX_NETWORKS] = {0};  // inverse of the (nq + nk)^2 system
    double* q_N = nullptr;        // nk Euclidean-orthonormal kernel vectors of A among the
    int q_nk = 0;                 //   constant pressures of the constrained networks (N each)
    double q_lambda[MPET_MAX_NETWORKS] = {0};
    bool q_dirty = true;
    double prec_p_shift[MPET_MAX_NETWORKS] = {0};  // + shift (p_a, w_a) in pressure block a
    void* gm_V = nullptr;         // GMRES basis, (restart + 1) x N doubles
    void* gm_z = nullptr;         // N doubles each
    void* gm_w = nullptr;
    void* gm_r = nullptr;
    double* gm_part = nullptr;    // (restart + 1) * NB_RED reduction partials
    double* gm_h = nullptr;       // restart + 1 device scalars
    double* gm_h_host = nullptr;  // pinned
    int gm_m = 0;                 // restart length the buffers hold
    bool elem_tried = false;
    int elem_kernel = 1;          // element blocks of tetrahedra: 1 tensor cores, 0 FP64 CUDA cores
    bool amg_device = true;       // Laplacian-form hierarchies built on the GPU (false: host set-up)
    bool bc_cols_zeroed = false;  // mpet_apply_symmetric zeroed the Dirichlet columns of A (until the next assembly)
    bool rhs_div_matrix = true;   // pressure rows' divergence term from the node-block product (test hook: false)
    int32_t* u_perm = nullptr;    // P2 node -> row of the spatially ordered first displacement level
    int32_t* u_iperm = nullptr;   // and back (built once per mesh)
    // last device set-up, summed over its hierarchies (ms): block copy, diagonal +
    // spectral radius, strength + aggregation, tentative + smoothed prolongator,
    // transposes, Galerkin products, coarsest inverse, layouts + autotuning
    double amg_phase_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    // error-indicator scratch: per-facet terms, per-cell R4p density, its sum, bad-index flag
    double* est_fval = nullptr;
    int64_t est_fval_cap = 0;
    double* est_r4 = nullptr;
    double* est_sum = nullptr;
    int32_t* est_bad = nullptr;
    double* partials = nullptr;   // reduction partials
    mpet::MinresScalars* sc = nullptr;
    mpet::MinresScalars* sc_host = nullptr;  // pinned

    // side streams: the pressure-block V-cycles run concurrently with the
    // displacement V-cycle (fork/join with events; parallel graph branches)
    cudaStream_t side[MPET_MAX_NETWORKS] = {nullptr};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[MPET_MAX_NETWORKS] = {nullptr};

    // MINRES iterations replayed from a CUDA graph (3 iterations per launch)
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t mr_graph = nullptr;  // whole inner solve: WHILE node over 3 iterations
    void* loop_ctl = nullptr;            // device loop control (target, budget, iterations)
    void* loop_ctl_host = nullptr;       // pinned copy
    cudaGraphExec_t mr_graph3 = nullptr; // 3 iterations, host-checked replays (inner_loop = 1)
    int64_t mr_graph3_launches = 0;
    int64_t mr_graph_launches = 0;  // kernels per graph launch

    // batch of independent instances in one mesh (ninst = 0: one instance):
    // DOF chunks of one instance each, the chunks of every instance in row
    // order, per-chunk partial sums and per-instance scalars
    int ninst = 0;
    int64_t nchunks = 0;
    int64_t* ch_lo = nullptr;
    int32_t* ch_len = nullptr;
    int32_t* ch_inst = nullptr;
    int32_t* inst_cptr = nullptr;
    int32_t* inst_chunks = nullptr;
    double* ch_part = nullptr;
    double* inst_v = nullptr;
    double* inst_host = nullptr;  // pinned
    // batched MINRES: scalars, done flags and inner targets per instance
    mpet::MinresScalars* bsc = nullptr;
    mpet::MinresScalars* bsc_host = nullptr;  // pinned
    double* bdone = nullptr;
    double* bdone_host = nullptr;             // pinned
    double* btarget = nullptr;
    double* bval = nullptr;                   // per-instance reduced sums
    cudaGraphExec_t bmr_graph = nullptr;
    int64_t bmr_graph_launches = 0;
    // instance of each P2 node (vertices first), the skip maps of the matrices
    // (Csr::skl) once built, and the done flags the products test (set only
    // while the batched iterations are captured; null: no product skips)
    int32_t* node_inst = nullptr;
    bool skip_maps = false;
    bool batch_skip = true;  // skip converged instances' slices (test hook: false)
    const double* skip_done = nullptr;

    // rigid-motion modes of the displacement (nz x Nu, L2-orthonormal), their
    // mass-weighted duals M Z, the multipliers of the last solve and a
    // right-hand-side scratch vector
    int nrigid = 0;
    double* rigid_Z = nullptr;
    double* rigid_MZ = nullptr;
    double rigid_r[6] = {0, 0, 0, 0, 0, 0};
    double* rigid_b = nullptr;

    // network eigenmodes of the pressure preconditioner (prec_network_modes):
    // per instance Q (J x J, column i = mode i) and lambda (J); vertex and
    // cell instance ids (batches); transformed residual / correction (J x nv)
    bool net_modes = false;
    double* mode_Q = nullptr;
    double* mode_lam = nullptr;
    int32_t* vert_inst = nullptr;
    int32_t* cell_inst = nullptr;
    double* mode_r = nullptr;
    double* mode_z = nullptr;

    // set by a kernel whose bounded wait gave up (read after each solve)
    int* dev_err = nullptr;
    int mbar_spin_limit = 1 << 22;  // polls of a staged-SpMV tile wait (test hook lowers it)
    double spmv_variant_ms[7] = {0, 0, 0, 0, 0, 0, 0};  // variants 0..5 and 8 (node blocks)
    double spmv_variant_ms64[7] = {0, 0, 0, 0, 0, 0, 0};  // FP64 residual products of the mixed path

    // timing
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double t_inner_ms = 0.0, t_solve_ms = 0.0;  // MINRES graph replays / whole solves
    // last preconditioner set-up (ms): block assembly (GPU), block downloads, host
    // hierarchies (built concurrently), uploads + autotuning
    double setup_ms[4] = {0, 0, 0, 0};
    int64_t n_inner_its = 0;
    cudaEvent_t ev_in0 = nullptr, ev_in1 = nullptr, ev_sv0 = nullptr, ev_sv1 = nullptr;
    int64_t n_spmv = 0, n_launch = 0;
    bool timing = false;
};

namespace mpet {

constexpr int NB_RED = 1216;  // fixed block count of every reduction kernel (152 SMs x 8)
constexpr int RED_THREADS = 256;
constexpr int BATCH_CHUNK = 4096;  // rows per chunk of the per-instance reductions

#ifdef __CUDACC__
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over a 256-thread block in a fixed order; result valid in thread 0.
__device__ __forceinline__ double block_sum256(double v, double* sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        t = warp_sum(t);
    }
    __syncthreads();
    return t;
}

// Sum of NB_RED partials by one 256-thread block (fixed order).
__device__ __forceinline__ double sum_partials(const double* p, double* sh) {
    double v = 0.0;
    for (int i = threadIdx.x; i < NB_RED; i += 256) v += p[i];
    return block_sum256(v, sh);
}
#endif

// setup.cu
void build_topology(mpet_ctx* c);
void build_pattern(mpet_ctx* c);
void build_bc(mpet_ctx* c);

// facets.cu
void build_facets(mpet_ctx* c);
void launch_facet_rhs(mpet_ctx* c, double dt, const double* up_prev, double* b);
void launch_robin_matrix(mpet_ctx* c, double dt);

// assemble.cu
void launch_assemble_matrix(mpet_ctx* c, double dt, bool apply_bc, bool write32);
void launch_assemble_prec_blocks(mpet_ctx* c, double dt);
// per-cell data of the matrix-free first displacement level (c->mf_cell, c->mf_tab);
// leaves c->mf_cell null when HBM is short
void launch_mf_cells(mpet_ctx* c, double dt);
void setup_network_modes(mpet_ctx* c, double dt);
void set_instances(mpet_ctx* c, int ninst, const int32_t* vertex_inst_host);
void launch_rhs(mpet_ctx* c, double dt, const double* up_prev, double* b);
// b_p += (pressure rows, displacement columns of the assembled system) u: the
// -alpha_a (div u^n, q_a) term of the right-hand side from the FP64 node-block
// copy; false when that copy cannot serve (none, or its columns were changed)
bool rhs_div_from_matrix(mpet_ctx* c, const double* up_prev, double* b);
void launch_bc_vector(mpet_ctx* c, double* b);
void launch_set_bc_in_x(mpet_ctx* c, double* x);
void launch_zero_bc_columns(mpet_ctx* c, double* b, const double* xbc);
void launch_zero_bc_rows(mpet_ctx* c, double* b);
void launch_adjoint_rhs(mpet_ctx* c, double dt, const double* lam, double* out);
void launch_mass_u(mpet_ctx* c, const double* f_nodes, double* out);
void launch_adjoint_grad(mpet_ctx* c, double dt, const double* lam, const double* up_prev, const double* up,
                         double* grad);
void launch_misfit(mpet_ctx* c, const double* up, const double* target, double* dloss, double* loss_dev);
// returns nonzero when the facet tables are inconsistent with the mesh
int launch_error_indicators(mpet_ctx* c, double dt, const double* up, const double* up_prev, const double* f,
                            const double* fp, const double* g, int64_t nfi, const int32_t* ifacets,
                            const int32_t* cell_facets, double* eta_p, double* eta_u, double* eta_udt,
                            double* r4_host);

// noalloc.cu: device address of the static residual scratch, looked up at
// context creation
void noalloc_prepare(int device);

// elem_tc.cu: the displacement element blocks of tetrahedra on the tensor cores
// (same record as k_elem_uu<3>)
void launch_elem_uu_tc(mpet_ctx* c, double mu, double lmbda, double* out);

// solve.cu
template <typename T>
void spmv(mpet_ctx* c, const Csr& A, int nvec, const T* x, T* y);
void upload_amg(mpet_ctx* c, AmgHier& h, const HostAmg& ha, int nvec, bool fp32);
// frees the device arrays of a hierarchy (before it is rebuilt)
void release_hier(mpet_ctx* c, AmgHier& h);
// Smoothed-aggregation hierarchy built on the GPU from a device block (FP64
// CSR) with the same recipe as amg_setup_host; with_p0: the first
// prolongator is the P1-in-P2 embedding of the free vertices (the block is
// the P2 displacement Laplacian).  ms[0] = hierarchy, ms[1] = layouts and
// autotuning (amg_device.cu).
void amg_setup_device(mpet_ctx* c, AmgHier& h, const Csr& A0, bool with_p0, double theta, int coarse_size,
                      int max_levels, int nvec, bool fp32, double ms[2]);
// FP32 copies, SpMV layouts, work buffers and autotuning of a hierarchy whose
// FP64 levels (A, P, R, dinv64, rho) and coarsest inverse are on the device
void finish_device_hier(mpet_ctx* c, AmgHier& h, int nvec, bool fp32);
double device_rho(mpet_ctx* c, const Csr& A, const double* dinv);
// greedy aggregation and dense SPD inverse of the host set-up (amg_setup.cpp)
int64_t aggregate(const HostCsr& S, std::vector<int64_t>& agg);
bool cholesky_inverse(std::vector<double>& a, int64_t n, std::vector<double>& inv);
// homogeneous: the Dirichlet entries of x are zero (adjoint solves) instead
// of the values set by mpet_set_bc_values
int solve_system(mpet_ctx* c, const double* b, double* x, mpet_stats* st, bool homogeneous = false);
void alloc_krylov(mpet_ctx* c);
void autotune_system(mpet_ctx* c);
void residual_norms(mpet_ctx* c, const double* b, const double* x, double* r, double* norms);
void apply_preconditioner(mpet_ctx* c, int precision, const void* r, void* z);
void profile_vcycle(mpet_ctx* c, int block, int reps, int* nlev, double* ms, double* bytes);
void setup_batch(mpet_ctx* c, int ninst, const int32_t* vertex_inst);
// batches: per-slice instance ranges of the system matrix and of every level
// of the Laplacian-form hierarchies (after each preconditioner set-up)
void build_skip_maps(mpet_ctx* c);
void batch_relres(mpet_ctx* c, double* out);
int choose_lpr(int64_t n, int64_t nnz);
void build_tiles(mpet_ctx* c, Csr& A, const int64_t* rp_host);
void build_sell(mpet_ctx* c, Csr& A, bool fp32, bool with64);
// the FP16 SELL values of A (after build_sell; needs A.v64)
void build_sell_half(mpet_ctx* c, Csr& A);
void fill_sell(mpet_ctx* c, Csr& A);
void build_node_blocks(mpet_ctx* c);
bool device_fits(mpet_ctx* c, size_t bytes);
void refresh_system_copies(mpet_ctx* c);
bool spmv_variant_available(const Csr& A, int variant);
constexpr int SPMV_TILE = 2048;  // entries per staged tile
void destroy_minres_graph(mpet_ctx* c);
void convert_values_to_f32(mpet_ctx* c);

}  // namespace mpet
