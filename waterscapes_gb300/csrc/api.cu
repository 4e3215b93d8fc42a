// extern "C" entry points of libmpetgpu (declared in include/mpet_gpu.h).
// Every entry point converts internal errors into status codes; nothing
// aborts, traps or exits.
#include <string.h>

#include <algorithm>
#include <chrono>
#include <exception>
#include <thread>

#include "mpet_internal.cuh"

using namespace mpet;

#define API_BEGIN(ctx)                  \
    if (!(ctx)) return MPET_ERR_INVALID; \
    try {                               \
        MPET_CUDA(cudaSetDevice((ctx)->device));
#define API_END(ctx)                                   \
    }                                                  \
    catch (const Error& e) {                           \
        (ctx)->err = e.msg;                            \
        return e.code;                                 \
    }                                                  \
    catch (const std::exception& e) {                  \
        (ctx)->err = e.what();                         \
        return MPET_ERR_NOMEM;                         \
    }                                                  \
    return MPET_OK;

static void require(bool cond, int code, const char* msg) {
    if (!cond) fail(code, msg);
}

extern "C" {

static const char* solve_status_message(int s) {
    switch (s) {
        case MPET_ERR_MAXIT: return "Krylov iteration limit reached";
        case MPET_ERR_TIMEOUT: return "a staged SpMV copy did not complete within its wait limit";
        case MPET_ERR_BREAKDOWN: return "Krylov breakdown (non-finite or indefinite preconditioned residual)";
        default: return "solve failed";
    }
}

int mpet_ctx_create(int device, mpet_ctx** out) {
    if (!out) return MPET_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return MPET_ERR_CUDA;
    }
    mpet_ctx* c = new (std::nothrow) mpet_ctx();
    if (!c) return MPET_ERR_NOMEM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return MPET_ERR_CUDA;
    }
    c->own_stream = true;
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    cudaEventCreate(&c->ev_in0);
    cudaEventCreate(&c->ev_in1);
    cudaEventCreate(&c->ev_sv0);
    cudaEventCreate(&c->ev_sv1);
    mpet::noalloc_prepare(device);
    *out = c;
    return MPET_OK;
}

int mpet_ctx_destroy(mpet_ctx* c) {
    if (!c) return MPET_ERR_INVALID;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    destroy_minres_graph(c);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    for (int a = 0; a < MPET_MAX_NETWORKS; ++a) {
        if (c->side[a]) cudaStreamDestroy(c->side[a]);
        if (c->ev_join[a]) cudaEventDestroy(c->ev_join[a]);
    }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    c->pool.free_all();
    if (c->sc_host) cudaFreeHost(c->sc_host);
    if (c->loop_ctl_host) cudaFreeHost(c->loop_ctl_host);
    if (c->inst_host) cudaFreeHost(c->inst_host);
    if (c->bsc_host) cudaFreeHost(c->bsc_host);
    if (c->bdone_host) cudaFreeHost(c->bdone_host);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (cudaEvent_t e : {c->ev_in0, c->ev_in1, c->ev_sv0, c->ev_sv1})
        if (e) cudaEventDestroy(e);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return MPET_OK;
}

const char* mpet_last_error(const mpet_ctx* c) { return c ? c->err.c_str() : "null context"; }

int mpet_set_stream(mpet_ctx* c, void* stream) {
    API_BEGIN(c)
    if (c->own_stream && c->stream) {
        MPET_CUDA(cudaStreamSynchronize(c->stream));
        MPET_CUDA(cudaStreamDestroy(c->stream));
    }
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
    API_END(c)
}

int mpet_synchronize(mpet_ctx* c) {
    API_BEGIN(c)
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    API_END(c)
}

int mpet_mesh_upload_dim(mpet_ctx* c, int32_t dim, int64_t nv, const double* xyz, int64_t nc, const int32_t* cells,
                         int64_t nf, const int32_t* bfacets, const int32_t* markers, int32_t J) {
    API_BEGIN(c)
    require(!c->mesh_ready, MPET_ERR_STATE, "mesh already uploaded to this context");
    require(dim == 2 || dim == 3, MPET_ERR_INVALID, "dim must be 2 (triangles) or 3 (tetrahedra)");
    require(nv > 0 && nc > 0 && nf >= 0 && xyz && cells, MPET_ERR_INVALID, "empty mesh");
    require(J >= 1 && J <= MPET_MAX_NETWORKS, MPET_ERR_INVALID, "num_networks must be in 1..8");
    require(nf == 0 || (bfacets && markers), MPET_ERR_INVALID, "facets without markers");
    require(nv < 2147483647LL / 4, MPET_ERR_INVALID, "too many vertices");
    const int cv = dim + 1;
    for (int64_t i = 0; i < cv * nc; ++i)
        require(cells[i] >= 0 && cells[i] < nv, MPET_ERR_INVALID, "cell vertex index out of range");
    for (int64_t i = 0; i < dim * nf; ++i)
        require(bfacets[i] >= 0 && bfacets[i] < nv, MPET_ERR_INVALID, "facet vertex index out of range");
    // cells with ascending vertex ids (DOLFIN's ordered-mesh convention)
    std::vector<int32_t> sorted(cells, cells + cv * nc);
    for (int64_t k = 0; k < nc; ++k) std::sort(sorted.begin() + cv * k, sorted.begin() + cv * k + cv);
    c->dim = dim;
    c->nv = nv;
    c->nc = nc;
    c->nf = nf;
    c->J = J;
    c->x = c->pool.alloc<double>(3 * nv);
    c->cells = c->pool.alloc<int32_t>(cv * nc);
    c->bfacets = c->pool.alloc<int32_t>(dim * (nf > 0 ? nf : 1));
    c->markers = c->pool.alloc<int32_t>((1 + J) * (nf > 0 ? nf : 1));
    MPET_CUDA(cudaMemcpyAsync(c->x, xyz, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, c->stream));
    MPET_CUDA(cudaMemcpyAsync(c->cells, sorted.data(), sizeof(int32_t) * cv * nc, cudaMemcpyHostToDevice, c->stream));
    if (nf > 0) {
        MPET_CUDA(cudaMemcpyAsync(c->bfacets, bfacets, sizeof(int32_t) * dim * nf, cudaMemcpyHostToDevice, c->stream));
        MPET_CUDA(cudaMemcpyAsync(c->markers, markers, sizeof(int32_t) * (1 + J) * nf, cudaMemcpyHostToDevice,
                                  c->stream));
    }
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->mesh_ready = true;
    API_END(c)
}

int mpet_mesh_upload(mpet_ctx* c, int64_t nv, const double* xyz, int64_t nc, const int32_t* tets, int64_t nf,
                     const int32_t* bfacets, const int32_t* markers, int32_t J) {
    return mpet_mesh_upload_dim(c, 3, nv, xyz, nc, tets, nf, bfacets, markers, J);
}

// GMRES when asked, or (AUTO) when the transfer matrix S is not symmetric
static bool wants_gmres(const mpet_ctx* c, const mpet_params* p) {
    if (p->krylov == MPET_KRYLOV_GMRES) return true;
    if (p->krylov == MPET_KRYLOV_MINRES) return false;
    for (int a = 0; a < c->J; ++a)
        for (int b = 0; b < c->J; ++b)
            if (p->S[a * MPET_MAX_NETWORKS + b] != p->S[b * MPET_MAX_NETWORKS + a]) return true;
    return false;
}

static void check_params(const mpet_ctx* c, const mpet_params* p) {
    require(p != nullptr, MPET_ERR_INVALID, "params is NULL");
    require(p->num_networks == c->J, MPET_ERR_INVALID, "params.num_networks differs from the mesh upload");
    require(p->precision == MPET_PRECISION_FP64 || p->precision == MPET_PRECISION_MIXED, MPET_ERR_INVALID,
            "unknown precision");
    require(p->theta > 0.0 && p->theta <= 1.0, MPET_ERR_INVALID, "theta must be in (0, 1]");
    require(p->rtol > 0.0, MPET_ERR_INVALID, "rtol must be positive");
    require(p->formulation == MPET_FORM_MPET || p->formulation == MPET_FORM_TOTAL_PRESSURE, MPET_ERR_INVALID,
            "unknown formulation");
    require(p->inner_loop == 0 || p->inner_loop == 1, MPET_ERR_INVALID, "inner_loop must be 0 or 1");
    require(p->amg_cheb_degree_fine <= 32, MPET_ERR_INVALID, "amg_cheb_degree_fine must be at most 32");
    require(p->amg_cheb_degree_coarse <= 32, MPET_ERR_INVALID, "amg_cheb_degree_coarse must be at most 32");
    require(p->prec_u_order == 0 || p->prec_u_order == 1, MPET_ERR_INVALID, "prec_u_order must be 0 or 1");
    require(p->amg_cheb_coarse_level <= 16, MPET_ERR_INVALID, "amg_cheb_coarse_level must be at most 16");
    require(p->krylov >= MPET_KRYLOV_AUTO && p->krylov <= MPET_KRYLOV_GMRES && p->gmres_restart <= 64,
            MPET_ERR_INVALID, "unknown Krylov method or restart above 64");
    if (p->formulation == MPET_FORM_TOTAL_PRESSURE) {
        require(c->J >= 2, MPET_ERR_INVALID, "the total-pressure form needs p0 and at least one network");
        require(p->lmbda > 0.0, MPET_ERR_INVALID, "the total-pressure form needs lmbda > 0");
        bool field0 = p->alpha[0] == 1.0 && p->c[0] == 0.0 && p->K[0] == 0.0;
        for (int b = 0; b < c->J; ++b)
            field0 = field0 && p->S[b] == 0.0 && p->S[b * MPET_MAX_NETWORKS] == 0.0;
        require(field0, MPET_ERR_INVALID, "total-pressure field 0 needs alpha = 1, c = K = 0 and no transfer");
    }
}

int mpet_setup(mpet_ctx* c, const mpet_params* p) {
    API_BEGIN(c)
    require(c->mesh_ready, MPET_ERR_STATE, "mpet_mesh_upload must come first");
    require(!c->setup_done, MPET_ERR_STATE, "mpet_setup already done");
    check_params(c, p);
    c->prm = *p;
    c->gmres = wants_gmres(c, p);
    if (c->prm.inner_rtol <= 0) c->prm.inner_rtol = 3e-4;
    if (c->prm.amg_theta < 0) c->prm.amg_theta = 0.1;
    build_topology(c);
    build_pattern(c);
    build_bc(c);
    build_facets(c);
    c->A.v64 = c->pool.alloc<double>(c->nnz);
    c->dinv = c->pool.alloc<double>(c->N);
    c->Lu.v64 = c->pool.alloc<double>(c->Lu.nnz);
    for (int a = 0; a < c->J; ++a) c->Pp[a].v64 = c->pool.alloc<double>(c->Pp[a].nnz);
    alloc_krylov(c);
    MPET_CUDA(cudaMemsetAsync(c->A.v64, 0, sizeof(double) * c->nnz, c->stream));
    // optional copies of the system matrix for the SpMV variants, in order of
    // use, each only while a fifth of HBM stays free: node blocks, the FP32
    // CSR values, SELL-32
    const bool mixed = c->prm.precision == MPET_PRECISION_MIXED;
    build_node_blocks(c);
    if (mixed && device_fits(c, sizeof(float) * (size_t)c->nnz)) {
        c->A.v32 = c->pool.alloc<float>(c->nnz);
        MPET_CUDA(cudaMemsetAsync(c->A.v32, 0, sizeof(float) * c->nnz, c->stream));
    }
    if (!mixed || c->A.v32) build_sell(c, c->A, c->A.v32 != nullptr, true);
    refresh_system_copies(c);
    autotune_system(c);
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->setup_done = true;
    API_END(c)
}

int mpet_update_params(mpet_ctx* c, const mpet_params* p) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    check_params(c, p);
    require(p->precision == c->prm.precision, MPET_ERR_INVALID, "precision is fixed at setup");
    c->prm = *p;
    c->gmres = wants_gmres(c, p);
    if (c->prm.inner_rtol <= 0) c->prm.inner_rtol = 3e-4;
    c->assembled = false;
    c->precond_ready = false;
    c->u_hier_valid = false;
    API_END(c)
}

int mpet_get_sizes(mpet_ctx* c, int64_t* N, int64_t* nnz, int64_t* nnodes, int64_t* nedges) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    if (N) *N = c->N;
    if (nnz) *nnz = c->nnz;
    if (nnodes) *nnodes = c->nnodes;
    if (nedges) *nedges = c->ne;
    API_END(c)
}

int mpet_get_pattern(mpet_ctx* c, int64_t* rp, int32_t* ci) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    if (rp) MPET_CUDA(cudaMemcpyAsync(rp, c->A.rp, sizeof(int64_t) * (c->N + 1), cudaMemcpyDeviceToHost, c->stream));
    if (ci) MPET_CUDA(cudaMemcpyAsync(ci, c->A.ci, sizeof(int32_t) * c->nnz, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    API_END(c)
}

int mpet_get_edges(mpet_ctx* c, int64_t* edges) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    std::vector<int64_t> k(c->ne);
    MPET_CUDA(cudaMemcpyAsync(k.data(), c->edge_key, sizeof(int64_t) * c->ne, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    for (int64_t e = 0; e < c->ne; ++e) {
        edges[2 * e] = k[e] / c->nv;
        edges[2 * e + 1] = k[e] % c->nv;
    }
    API_END(c)
}

int mpet_assemble(mpet_ctx* c, double dt, int32_t apply_bc) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(dt > 0.0, MPET_ERR_INVALID, "dt must be positive");
    launch_assemble_matrix(c, dt, apply_bc != 0, c->A.v32 != nullptr);
    launch_robin_matrix(c, dt);
    refresh_system_copies(c);
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->assembled = true;
    c->bc_cols_zeroed = false;
    c->q_dirty = true;
    c->asm_dt = dt;
    API_END(c)
}

int mpet_get_values(mpet_ctx* c, double* vals) {
    API_BEGIN(c)
    require(c->assembled, MPET_ERR_STATE, "mpet_assemble must come first");
    MPET_CUDA(cudaMemcpyAsync(vals, c->A.v64, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    API_END(c)
}

int mpet_get_bc_count(mpet_ctx* c, int32_t field, int64_t* count) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(field >= 0 && field <= c->J && count, MPET_ERR_INVALID, "bad field");
    *count = c->bc_off[field + 1] - c->bc_off[field];
    API_END(c)
}

__global__ void k_bc_coords(const int32_t* __restrict__ dofs, int64_t n, int64_t Nu, int64_t nv, int dim,
                            const double* __restrict__ x, const int64_t* __restrict__ ekey, double* coords) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t d = dofs[i];
    int64_t node = d < Nu ? d / dim : (d - Nu) % nv;
    for (int k = 0; k < 3; ++k) {
        double v;
        if (node < nv) {
            v = x[3 * node + k];
        } else {
            int64_t key = ekey[node - nv];
            v = 0.5 * (x[3 * (key / nv) + k] + x[3 * (key % nv) + k]);
        }
        coords[3 * i + k] = v;
    }
}

int mpet_get_bc(mpet_ctx* c, int32_t field, int32_t* dofs, double* coords) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(field >= 0 && field <= c->J, MPET_ERR_INVALID, "bad field");
    const int64_t off = c->bc_off[field], n = c->bc_off[field + 1] - off;
    if (n > 0) {
        if (dofs)
            MPET_CUDA(cudaMemcpyAsync(dofs, c->bc_dofs + off, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, c->stream));
        if (coords) {
            k_bc_coords<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(c->bc_dofs + off, n, c->Nu, c->nv, c->dim, c->x,
                                                                        c->edge_key, coords);
            MPET_CHECK_LAUNCH();
        }
    }
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    API_END(c)
}

int mpet_set_bc_values(mpet_ctx* c, int32_t field, const double* vals) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(field >= 0 && field <= c->J, MPET_ERR_INVALID, "bad field");
    const int64_t off = c->bc_off[field], n = c->bc_off[field + 1] - off;
    if (n > 0) {
        if (vals)
            MPET_CUDA(cudaMemcpyAsync(c->bc_vals + off, vals, sizeof(double) * n, cudaMemcpyDefault, c->stream));
        else
            MPET_CUDA(cudaMemsetAsync(c->bc_vals + off, 0, sizeof(double) * n, c->stream));
    }
    API_END(c)
}

int mpet_set_sources(mpet_ctx* c, const double* f, const double* g) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    c->f_nodes = f;
    c->g_vert = g;
    API_END(c)
}

int mpet_set_cell_permeability(mpet_ctx* c, const double* K_cells) {
    API_BEGIN(c)
    require(!c->setup_done || c->prm.formulation == MPET_FORM_MPET, MPET_ERR_INVALID,
            "built for the MPET form only");
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    c->K_cells = K_cells;
    c->assembled = false;
    c->precond_ready = false;
    API_END(c)
}

int mpet_set_rigid_modes(mpet_ctx* c, int32_t nz, const double* Z) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(nz >= 0 && nz <= 6 && (nz == 0 || Z), MPET_ERR_INVALID, "nz must be in 0..6");
    require(c->ninst == 0, MPET_ERR_INVALID, "rigid modes are not built for batches");
    require(nz == 0 || c->bc_off[1] == c->bc_off[0], MPET_ERR_INVALID,
            "rigid-motion modes need a displacement without Dirichlet DOFs");
    if (nz > 0 && !c->rigid_Z) {
        c->rigid_Z = c->pool.alloc<double>(6 * c->Nu);
        c->rigid_MZ = c->pool.alloc<double>(6 * c->Nu);
        c->rigid_b = c->pool.alloc<double>(c->N);
    }
    for (int i = 0; i < nz; ++i) {
        MPET_CUDA(cudaMemcpyAsync(c->rigid_Z + (int64_t)i * c->Nu, Z + (int64_t)i * c->Nu, sizeof(double) * c->Nu,
                                  cudaMemcpyDeviceToDevice, c->stream));
        launch_mass_u(c, c->rigid_Z + (int64_t)i * c->Nu, c->rigid_MZ + (int64_t)i * c->Nu);
    }
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->nrigid = nz;
    for (int i = 0; i < 6; ++i) c->rigid_r[i] = 0.0;
    API_END(c)
}

int mpet_get_rigid_multipliers(mpet_ctx* c, double* r) {
    API_BEGIN(c)
    require(r, MPET_ERR_INVALID, "NULL argument");
    for (int i = 0; i < c->nrigid; ++i) r[i] = c->rigid_r[i];
    API_END(c)
}

int mpet_set_pressure_constraints(mpet_ctx* c, int32_t nq, const int32_t* networks) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(c->ninst == 0 && !c->gmres, MPET_ERR_INVALID,
            "pressure constraints are built for single instances solved by MINRES");
    require(nq >= 0 && nq <= c->J && (nq == 0 || networks), MPET_ERR_INVALID, "nq must be in 0..J");
    for (int k = 0; k < nq; ++k) {
        const int a = networks[k];
        require(a >= 0 && a < c->J, MPET_ERR_INVALID, "network index out of range");
        for (int q = 0; q < k; ++q) require(networks[q] != a, MPET_ERR_INVALID, "network listed twice");
        require(c->bc_off[2 + a] == c->bc_off[1 + a], MPET_ERR_INVALID,
                "a constant-pressure constraint needs a network without Dirichlet DOFs");
    }
    // P1 load vector int phi_v = sum over the vertex's cells |T| / (dim + 1), and the diameter
    const int nvc = c->dim + 1;
    std::vector<double> geo((size_t)c->nc * 16), xyz((size_t)c->nv * 3);
    std::vector<int32_t> cells((size_t)c->nc * nvc);
    MPET_CUDA(cudaMemcpyAsync(geo.data(), c->geo, sizeof(double) * geo.size(), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaMemcpyAsync(xyz.data(), c->x, sizeof(double) * xyz.size(), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaMemcpyAsync(cells.data(), c->cells, sizeof(int32_t) * cells.size(), cudaMemcpyDeviceToHost,
                              c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<double> load(c->nv, 0.0);
    for (int64_t e = 0; e < c->nc; ++e)
        for (int r = 0; r < nvc; ++r) load[cells[(size_t)e * nvc + r]] += geo[16 * e + 12] / nvc;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t v = 0; v < c->nv; ++v)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], xyz[3 * v + k]);
            hi[k] = std::max(hi[k], xyz[3 * v + k]);
        }
    double diam2 = 0.0;
    for (int k = 0; k < 3; ++k) diam2 += (hi[k] - lo[k]) * (hi[k] - lo[k]);
    if (!c->q_load) c->q_load = c->pool.alloc<double>(c->nv);
    MPET_CUDA(cudaMemcpyAsync(c->q_load, load.data(), sizeof(double) * c->nv, cudaMemcpyHostToDevice, c->stream));
    if (nq > 0 && (!c->q_W || nq > c->nq)) {
        c->q_W = c->pool.alloc<double>((int64_t)nq * c->N);
        c->q_N = c->pool.alloc<double>((int64_t)nq * c->N);
    }
    if (nq > 0 && !c->rigid_b) c->rigid_b = c->pool.alloc<double>(c->N);  // projected right-hand side
    c->q_nk = 0;
    for (int a = 0; a < MPET_MAX_NETWORKS; ++a) c->prec_p_shift[a] = 0.0;
    for (int k = 0; k < nq; ++k) {
        c->q_net[k] = networks[k];
        c->prec_p_shift[networks[k]] = diam2 > 0.0 ? c->prm.K[networks[k]] / diam2 : 0.0;
        c->q_lambda[k] = 0.0;
    }
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->nq = nq;
    c->q_dirty = true;
    c->precond_ready = false;
    API_END(c)
}

int mpet_get_pressure_multipliers(mpet_ctx* c, double* lambda_host) {
    API_BEGIN(c)
    require(lambda_host, MPET_ERR_INVALID, "NULL argument");
    for (int k = 0; k < c->nq; ++k) lambda_host[k] = c->q_lambda[k];
    API_END(c)
}

int mpet_set_cell_coefficients(mpet_ctx* c, const double* c_cells, const double* S_cells) {
    API_BEGIN(c)
    require(!c->setup_done || c->prm.formulation == MPET_FORM_MPET, MPET_ERR_INVALID,
            "built for the MPET form only");
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    c->c_cells = c_cells;
    c->S_cells = S_cells;
    c->assembled = false;
    c->precond_ready = false;
    API_END(c)
}

int mpet_set_batch(mpet_ctx* c, int32_t ninst, const int32_t* vertex_instance) {
    API_BEGIN(c)
    require(!c->setup_done || c->prm.formulation == MPET_FORM_MPET, MPET_ERR_INVALID,
            "built for the MPET form only");
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(c->dim == 3, MPET_ERR_INVALID, "batches are built for tetrahedral meshes");
    require(c->ninst == 0, MPET_ERR_STATE, "the batch partition is already set");
    require(c->nrigid == 0, MPET_ERR_STATE, "batches with rigid-motion modes are not built");
    require(ninst >= 1 && vertex_instance, MPET_ERR_INVALID, "need ninst >= 1 and an instance per vertex");
    setup_batch(c, ninst, vertex_instance);
    set_instances(c, ninst, vertex_instance);
    c->precond_ready = false;
    c->u_hier_valid = false;
    API_END(c)
}

int mpet_get_batch_relres(mpet_ctx* c, double* relres_host) {
    API_BEGIN(c)
    require(c->ninst > 0 && c->inst_host, MPET_ERR_STATE, "no batch solve yet");
    require(relres_host, MPET_ERR_INVALID, "NULL argument");
    batch_relres(c, relres_host);
    API_END(c)
}

int mpet_get_facet_data(mpet_ctx* c, int32_t* fnodes, double* area_normal) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    if (c->nf > 0) {
        if (fnodes)
            MPET_CUDA(cudaMemcpyAsync(fnodes, c->fnodes, sizeof(int32_t) * 6 * c->nf, cudaMemcpyDeviceToDevice,
                                      c->stream));
        if (area_normal)
            MPET_CUDA(cudaMemcpyAsync(area_normal, c->fgeo, sizeof(double) * 4 * c->nf, cudaMemcpyDeviceToDevice,
                                      c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
    }
    API_END(c)
}

int mpet_set_facet_data(mpet_ctx* c, int32_t kind, const double* values) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    switch (kind) {
        case MPET_FACET_TRACTION: c->f_traction = values; break;
        case MPET_FACET_FLUX: c->f_flux = values; break;
        case MPET_FACET_ROBIN_BETA: c->f_beta = values; break;
        case MPET_FACET_ROBIN_PRESSURE: c->f_probin = values; break;
        case MPET_FACET_ROBIN_BETA_MATRIX: c->f_beta_matrix = values; break;
        default: fail(MPET_ERR_INVALID, "unknown facet data kind");
    }
    API_END(c)
}

int mpet_rhs(mpet_ctx* c, double dt, const double* up_prev, double* b) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(up_prev && b, MPET_ERR_INVALID, "NULL vector");
    launch_rhs(c, dt, up_prev, b);
    API_END(c)
}

int mpet_setup_preconditioner(mpet_ctx* c, double dt) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(dt > 0.0, MPET_ERR_INVALID, "dt must be positive");
    destroy_minres_graph(c);
    using clk = std::chrono::steady_clock;
    auto since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
    auto t0 = clk::now();
    setup_network_modes(c, dt);
    launch_assemble_prec_blocks(c, dt);
    // the displacement block w (grad u, grad v) depends on neither dt nor K, c, S: its
    // hierarchy is kept from the last set-up unless the parameters changed
    const bool reuse_u = c->u_hier_valid && c->prm.prec_u_form != 1;
    if (c->prm.prec_u_form != 1 && !reuse_u) launch_mf_cells(c, dt);
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    c->setup_ms[0] = since(t0);  // block assembly on the GPU
    t0 = clk::now();
    const bool fp32 = c->prm.precision == MPET_PRECISION_MIXED;
    auto fetch = [&](const Csr& d, HostCsr& h) {
        h.n = d.n;
        h.m = d.m;
        h.rp.resize(d.n + 1);
        h.ci.resize(d.nnz);
        h.v.resize(d.nnz);
        MPET_CUDA(cudaMemcpyAsync(h.rp.data(), d.rp, sizeof(int64_t) * (d.n + 1), cudaMemcpyDeviceToHost, c->stream));
        MPET_CUDA(cudaMemcpyAsync(h.ci.data(), d.ci, sizeof(int32_t) * d.nnz, cudaMemcpyDeviceToHost, c->stream));
        MPET_CUDA(cudaMemcpyAsync(h.v.data(), d.v64, sizeof(double) * d.nnz, cudaMemcpyDeviceToHost, c->stream));
        MPET_CUDA(cudaStreamSynchronize(c->stream));
        // the pattern arrays of the P1 blocks cover all P2 nodes: keep the vertex rows
        if (h.rp[0] != 0) fail(MPET_ERR_STATE, "unexpected row pointer base");
    };
    const int cs = c->prm.amg_coarse_size > 0 ? c->prm.amg_coarse_size : 500;
    bool elast = false;
    if (c->prm.prec_u_form == 1) {
        try {
            elast = setup_u_elasticity(c, fp32);
        } catch (const Error&) {
            // e.g. a coarsest elasticity operator that is not definite: the Laplacian form stands in
            cudaGetLastError();
            elast = false;
        }
        c->u_elast = elast;
    }
    const bool build_u = !elast && !reuse_u;
    if (c->amg_device) {
        // every hierarchy built where its block lies (amg_device.cu)
        double ms[2], build = 0.0, finish = 0.0;
        const double theta = c->prm.amg_theta;
        for (double& x : c->amg_phase_ms) x = 0.0;
        if (build_u) {
            c->u_elast = false;
            amg_setup_device(c, c->amg_u, c->Lu, c->prm.amg_p2_to_p1 != 0, theta, cs, 12, 4, fp32, ms);
            build += ms[0];
            finish += ms[1];
            c->u_hier_valid = true;
        }
        for (int a = 0; a < c->J; ++a) {
            amg_setup_device(c, c->amg_p[a], c->Pp[a], false, theta, cs, 12, 1, fp32, ms);
            build += ms[0];
            finish += ms[1];
        }
        if (c->ninst > 0) build_skip_maps(c);
        c->setup_ms[1] = 0.0;     // nothing downloaded
        c->setup_ms[2] = build;   // hierarchies (device)
        c->setup_ms[3] = finish;  // FP32 copies, layouts, autotuning
        c->precond_ready = true;
        c->prec_dt = dt;
        return MPET_OK;
    }
    // downloads (and the P1-in-P2 embedding), then the host set-ups of all
    // hierarchies concurrently (threads sharing the host cores), then uploads
    HostCsr hu, P0;
    bool use_p0 = false;
    if (build_u) {
        c->u_elast = false;
        fetch(c->Lu, hu);
        if (c->prm.amg_p2_to_p1) {
            use_p0 = true;
            // First level of the displacement hierarchy: the P1 functions that
            // vanish on the displacement Dirichlet boundary, embedded in P2
            // (vertex values copied, edge-midpoint values averaged).
            std::vector<int64_t> ek(c->ne);
            std::vector<uint8_t> bc(c->nnodes);
            MPET_CUDA(cudaMemcpyAsync(ek.data(), c->edge_key, sizeof(int64_t) * c->ne, cudaMemcpyDeviceToHost,
                                      c->stream));
            MPET_CUDA(cudaMemcpyAsync(bc.data(), c->node_bc, c->nnodes, cudaMemcpyDeviceToHost, c->stream));
            MPET_CUDA(cudaStreamSynchronize(c->stream));
            std::vector<int64_t> cidx(c->nv, -1);
            int64_t m = 0;
            for (int64_t v = 0; v < c->nv; ++v)
                if (!bc[v]) cidx[v] = m++;
            P0.n = c->nnodes;
            P0.m = m;
            P0.rp.assign(c->nnodes + 1, 0);
            for (int64_t i = 0; i < c->nnodes; ++i) {
                int64_t cnt = 0;
                if (!bc[i]) {
                    if (i < c->nv) cnt = 1;
                    else cnt = (cidx[ek[i - c->nv] / c->nv] >= 0) + (cidx[ek[i - c->nv] % c->nv] >= 0);
                }
                P0.rp[i + 1] = P0.rp[i] + cnt;
            }
            P0.ci.resize(P0.rp[c->nnodes]);
            P0.v.resize(P0.rp[c->nnodes]);
            for (int64_t i = 0; i < c->nnodes; ++i) {
                int64_t p = P0.rp[i];
                if (bc[i]) continue;
                if (i < c->nv) {
                    P0.ci[p] = (int32_t)cidx[i];
                    P0.v[p] = 1.0;
                } else {
                    const int64_t lo = ek[i - c->nv] / c->nv, hi = ek[i - c->nv] % c->nv;
                    for (int64_t w : {lo, hi})
                        if (cidx[w] >= 0) {
                            P0.ci[p] = (int32_t)cidx[w];
                            P0.v[p] = 0.5;
                            ++p;
                        }
                }
            }
        }
    }
    std::vector<HostCsr> hp(c->J);
    for (int a = 0; a < c->J; ++a) fetch(c->Pp[a], hp[a]);
    c->setup_ms[1] = since(t0);  // downloads of the blocks
    t0 = clk::now();
    HostAmg hau;
    std::vector<HostAmg> hap(c->J);
    {
        const int ntask = c->J + (build_u ? 1 : 0);
        const int nth = std::max(1, host_threads() / ntask);
        std::vector<std::exception_ptr> errs(ntask);
        std::vector<std::thread> th;
        const double theta = c->prm.amg_theta;
        for (int a = 0; a < c->J; ++a)
            th.emplace_back([&, a] {
                try {
                    amg_setup_host(std::move(hp[a]), nullptr, theta, cs, 12, hap[a], nth);
                } catch (...) {
                    errs[a] = std::current_exception();
                }
            });
        if (build_u)
            th.emplace_back([&] {
                try {
                    amg_setup_host(std::move(hu), use_p0 ? &P0 : nullptr, theta, cs, 12, hau, nth, true);
                } catch (...) {
                    errs[c->J] = std::current_exception();
                }
            });
        for (auto& t : th) t.join();
        for (auto& e : errs)
            if (e) std::rethrow_exception(e);
    }
    c->setup_ms[2] = since(t0);  // host hierarchies (concurrent)
    t0 = clk::now();
    if (build_u) {
        upload_amg(c, c->amg_u, hau, 4, fp32);
        c->u_hier_valid = true;
    }
    for (int a = 0; a < c->J; ++a) upload_amg(c, c->amg_p[a], hap[a], 1, fp32);
    if (c->ninst > 0) build_skip_maps(c);
    c->setup_ms[3] = since(t0);  // uploads + autotuning
    c->precond_ready = true;
    c->prec_dt = dt;
    API_END(c)
}

int mpet_get_setup_timing(mpet_ctx* c, double* ms4) {
    API_BEGIN(c)
    require(ms4, MPET_ERR_INVALID, "NULL argument");
    for (int k = 0; k < 4; ++k) ms4[k] = c->setup_ms[k];
    API_END(c)
}

int mpet_get_prec_info(mpet_ctx* c, int32_t* u_elasticity) {
    API_BEGIN(c)
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(u_elasticity, MPET_ERR_INVALID, "NULL argument");
    *u_elasticity = c->u_elast ? 1 : 0;
    API_END(c)
}

int mpet_get_amg_info(mpet_ctx* c, int32_t block, int32_t* levels, int64_t* sizes, int64_t* nnz) {
    API_BEGIN(c)
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(block >= 0 && block <= c->J, MPET_ERR_INVALID, "bad block");
    const AmgHier& h = block == 0 ? c->amg_u : c->amg_p[block - 1];
    if (levels) *levels = (int32_t)h.lev.size();
    for (size_t k = 0; k < h.lev.size(); ++k) {
        if (sizes) sizes[k] = h.lev[k].A.n;
        if (nnz) nnz[k] = h.lev[k].A.nnz;
    }
    API_END(c)
}

int mpet_set_amg_setup(mpet_ctx* c, int32_t where) {
    API_BEGIN(c)
    require(where == 0 || where == 1, MPET_ERR_INVALID, "AMG set-up: 0 (host) or 1 (device)");
    c->amg_device = where == 1;
    c->u_hier_valid = false;
    c->precond_ready = false;
    API_END(c)
}

int mpet_get_amg_variants(mpet_ctx* c, int32_t block, int32_t* a_variant, int32_t* p_variant, int32_t* r_variant) {
    API_BEGIN(c)
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(block >= 0 && block <= c->J, MPET_ERR_INVALID, "bad block");
    const AmgHier& h = block == 0 ? c->amg_u : c->amg_p[block - 1];
    for (size_t k = 0; k < h.lev.size(); ++k) {
        const AmgLevel& L = h.lev[k];
        if (a_variant) a_variant[k] = L.mf ? 16 : (L.nb_uu ? 8 : L.A.variant);
        if (p_variant) p_variant[k] = k + 1 < h.lev.size() ? L.P.variant : -1;
        if (r_variant) r_variant[k] = k + 1 < h.lev.size() ? L.R.variant : -1;
    }
    API_END(c)
}

int mpet_get_amg_setup_phases(mpet_ctx* c, double* ms8) {
    API_BEGIN(c)
    require(ms8, MPET_ERR_INVALID, "NULL argument");
    for (int k = 0; k < 8; ++k) ms8[k] = c->amg_phase_ms[k];
    API_END(c)
}

int mpet_get_amg_matrix(mpet_ctx* c, int32_t block, int32_t level, int32_t which, int64_t* n, int64_t* m,
                        int64_t* nnz, int64_t* rp, int32_t* ci, double* v) {
    API_BEGIN(c)
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(block >= 0 && block <= c->J, MPET_ERR_INVALID, "bad block");
    require(which == 0 || which == 1, MPET_ERR_INVALID, "which: 0 (operator) or 1 (prolongation)");
    const AmgHier& h = block == 0 ? c->amg_u : c->amg_p[block - 1];
    require(level >= 0 && level < (int32_t)h.lev.size(), MPET_ERR_INVALID, "bad level");
    require(!(which == 1 && level + 1 == (int32_t)h.lev.size()), MPET_ERR_INVALID, "the coarsest level has no P");
    const Csr& d = which == 0 ? h.lev[level].A : h.lev[level].P;
    require(d.rp != nullptr && d.v64 != nullptr, MPET_ERR_STATE, "this level has no stored matrix");
    if (n) *n = d.n;
    if (m) *m = d.m;
    if (nnz) *nnz = d.nnz;
    if (rp) MPET_CUDA(cudaMemcpyAsync(rp, d.rp, sizeof(int64_t) * (d.n + 1), cudaMemcpyDeviceToHost, c->stream));
    if (ci && d.nnz) MPET_CUDA(cudaMemcpyAsync(ci, d.ci, sizeof(int32_t) * d.nnz, cudaMemcpyDeviceToHost, c->stream));
    if (v && d.nnz) MPET_CUDA(cudaMemcpyAsync(v, d.v64, sizeof(double) * d.nnz, cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    API_END(c)
}

int mpet_profile_vcycle(mpet_ctx* c, int32_t block, int32_t reps, int32_t* nlev, double* ms, double* bytes) {
    API_BEGIN(c)
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(block >= 0 && block <= c->J, MPET_ERR_INVALID, "bad block");
    require(reps >= 1 && nlev && ms && bytes, MPET_ERR_INVALID, "reps >= 1 and non-NULL outputs");
    destroy_minres_graph(c);
    int n = 0;
    profile_vcycle(c, block, reps, &n, ms, bytes);
    *nlev = n;
    API_END(c)
}

int mpet_solve(mpet_ctx* c, const double* b, double* x, mpet_stats* st) {
    API_BEGIN(c)
    require(c->assembled, MPET_ERR_STATE, "mpet_assemble must come first");
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(b && x, MPET_ERR_INVALID, "NULL vector");
    int s = solve_system(c, b, x, st);
    if (s != MPET_OK) {
        c->err = solve_status_message(s);
        return s;
    }
    API_END(c)
}

int mpet_step(mpet_ctx* c, double dt, const double* up_prev, double* up, mpet_stats* st) {
    API_BEGIN(c)
    require(c->assembled, MPET_ERR_STATE, "mpet_assemble must come first");
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(up_prev && up && up_prev != up, MPET_ERR_INVALID, "up_prev and up must be distinct device arrays");
    double* b = c->ob ? c->ob : (c->ob = c->pool.alloc<double>(c->N));
    launch_rhs(c, dt, up_prev, b);
    if (up != up_prev)
        MPET_CUDA(cudaMemcpyAsync(up, up_prev, sizeof(double) * c->N, cudaMemcpyDeviceToDevice, c->stream));
    int s = solve_system(c, b, up, st);
    if (s != MPET_OK) {
        c->err = solve_status_message(s);
        return s;
    }
    API_END(c)
}

int mpet_apply_preconditioner(mpet_ctx* c, int32_t precision, const void* r, void* z) {
    API_BEGIN(c)
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(r && z && r != z, MPET_ERR_INVALID, "r and z must be distinct device arrays");
    const bool mixed = c->prm.precision == MPET_PRECISION_MIXED;
    require(precision == (mixed ? MPET_PRECISION_MIXED : MPET_PRECISION_FP64), MPET_ERR_INVALID,
            "the hierarchy holds FP32 values in mixed precision and FP64 values otherwise");
    apply_preconditioner(c, precision, r, z);
    API_END(c)
}

int mpet_residual(mpet_ctx* c, const double* b, const double* x, double* r, double* norms) {
    API_BEGIN(c)
    require(c->assembled, MPET_ERR_STATE, "mpet_assemble must come first");
    require(b && x && r && norms, MPET_ERR_INVALID, "NULL argument");
    residual_norms(c, b, x, r, norms);
    API_END(c)
}

int mpet_spmv(mpet_ctx* c, int32_t precision, const void* x, void* y) {
    API_BEGIN(c)
    require(c->assembled, MPET_ERR_STATE, "mpet_assemble must come first");
    if (precision == MPET_PRECISION_MIXED) {
        require(c->A.v32 != nullptr, MPET_ERR_STATE, "no FP32 values (setup precision is FP64)");
        spmv<float>(c, c->A, 1, (const float*)x, (float*)y);
    } else {
        spmv<double>(c, c->A, 1, (const double*)x, (double*)y);
    }
    API_END(c)
}

int mpet_apply_symmetric(mpet_ctx* c, double* b, const double* xbc) {
    API_BEGIN(c)
    require(c->assembled, MPET_ERR_STATE, "mpet_assemble must come first");
    launch_zero_bc_columns(c, b, xbc);
    c->bc_cols_zeroed = true;
    convert_values_to_f32(c);
    refresh_system_copies(c);
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    API_END(c)
}

int mpet_get_spmv_tuning(mpet_ctx* c, double* ms7, int32_t* chosen) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    if (ms7)
        for (int v = 0; v < 7; ++v) ms7[v] = c->spmv_variant_ms[v];
    if (chosen) *chosen = c->A.variant;
    API_END(c)
}

int mpet_get_spmv_tuning_fp64(mpet_ctx* c, double* ms7, int32_t* chosen) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    const bool own = c->A.variant64 >= 0;
    if (ms7)
        for (int v = 0; v < 7; ++v) ms7[v] = own ? c->spmv_variant_ms64[v] : c->spmv_variant_ms[v];
    if (chosen) *chosen = own ? c->A.variant64 : c->A.variant;
    API_END(c)
}

int mpet_set_hierarchy_spmv_variant(mpet_ctx* c, int32_t variant) {
    API_BEGIN(c)
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require((variant >= 0 && variant <= 8) || variant == 32, MPET_ERR_INVALID, "variant out of range");
    destroy_minres_graph(c);
    auto set = [&](mpet::Csr& M) { M.variant = spmv_variant_available(M, variant) ? variant : 0; };
    auto hier = [&](mpet::AmgHier& h) {
        for (auto& L : h.lev) {
            set(L.A);
            set(L.P);
            set(L.R);
        }
    };
    hier(c->amg_u);
    for (int a = 0; a < c->J; ++a) hier(c->amg_p[a]);
    API_END(c)
}

int mpet_get_node_block_info(mpet_ctx* c, int64_t* blocks, int64_t* stored_values) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    if (blocks) *blocks = c->A_nb.nblocks;
    if (stored_values) *stored_values = c->A_nb.nvals;
    API_END(c)
}

int mpet_set_spmv_variant(mpet_ctx* c, int32_t variant) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(spmv_variant_available(c->A, variant), MPET_ERR_INVALID, "SpMV variant not available for this matrix");
    destroy_minres_graph(c);
    c->A.variant = variant;
    c->A.variant64 = -1;  // the forced variant serves both precisions
    API_END(c)
}

int mpet_set_prec_matrix_free(mpet_ctx* c, int32_t mode) {
    API_BEGIN(c)
    require(mode >= -1 && mode <= 1, MPET_ERR_INVALID, "mode: -1 (autotuned), 0 (CSR) or 1 (matrix-free)");
    c->mf_mode = mode;
    c->precond_ready = false;
    c->u_hier_valid = false;
    API_END(c)
}

int mpet_get_prec_matrix_free(mpet_ctx* c, int32_t* used, float* ms2) {
    API_BEGIN(c)
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    if (used) *used = (!c->u_elast && !c->amg_u.lev.empty() && c->amg_u.lev[0].mf) ? 1 : 0;
    if (ms2) {
        ms2[0] = c->mf_ms[0];
        ms2[1] = c->mf_ms[1];
    }
    API_END(c)
}

int mpet_set_element_kernel(mpet_ctx* c, int32_t kind) {
    API_BEGIN(c)
    require(kind == 0 || kind == 1, MPET_ERR_INVALID, "element kernel: 0 (FP64 CUDA cores) or 1 (tensor cores)");
    c->elem_kernel = kind;
    c->assembled = false;
    API_END(c)
}

int mpet_set_wait_limit(mpet_ctx* c, int32_t polls) {
    API_BEGIN(c)
    require(polls >= 0, MPET_ERR_INVALID, "wait limit must be >= 0");
    c->mbar_spin_limit = polls > 0 ? polls : 0;
    API_END(c)
}

int mpet_set_batch_skip(mpet_ctx* c, int32_t on) {
    API_BEGIN(c)
    require(on == 0 || on == 1, MPET_ERR_INVALID, "batch skip: 0 or 1");
    c->batch_skip = on == 1;
    destroy_minres_graph(c);
    API_END(c)
}

int mpet_get_timing(mpet_ctx* c, double* inner_ms, int64_t* inner_iterations, double* solve_ms, int64_t* launches) {
    API_BEGIN(c)
    if (inner_ms) *inner_ms = c->t_inner_ms;
    if (inner_iterations) *inner_iterations = c->n_inner_its;
    if (solve_ms) *solve_ms = c->t_solve_ms;
    if (launches) *launches = c->n_launch;
    API_END(c)
}

int mpet_error_indicators(mpet_ctx* c, double dt, const double* up, const double* up_prev, const double* f_nodes,
                          const double* f_prev_nodes, const double* g_vert, int64_t n_ifacets,
                          const int32_t* ifacets, const int32_t* cell_facets, double* eta_p, double* eta_u,
                          double* eta_u_dt, double* r4p) {
    API_BEGIN(c)
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(c->prm.formulation == MPET_FORM_MPET, MPET_ERR_INVALID, "built for the MPET form only");
    require(!c->K_cells && !c->c_cells && !c->S_cells && c->ninst == 0, MPET_ERR_INVALID,
            "indicators take scalar K, c, S and a single instance");
    require(dt > 0.0, MPET_ERR_INVALID, "dt must be positive");
    require(up && up_prev && cell_facets && eta_p && eta_u && eta_u_dt && r4p && n_ifacets >= 0 &&
                (n_ifacets == 0 || ifacets),
            MPET_ERR_INVALID, "NULL argument");
    require(launch_error_indicators(c, dt, up, up_prev, f_nodes, f_prev_nodes, g_vert, n_ifacets, ifacets,
                                    cell_facets, eta_p, eta_u, eta_u_dt, r4p) == 0,
            MPET_ERR_INVALID, "interior-facet tables do not match the mesh");
    API_END(c)
}

int mpet_pressure_misfit(mpet_ctx* c, const double* up, const double* p_target, double* loss, double* dloss) {
    API_BEGIN(c)
    require(!c->setup_done || c->prm.formulation == MPET_FORM_MPET, MPET_ERR_INVALID,
            "built for the MPET form only");
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(c->dim == 3, MPET_ERR_INVALID, "the adjoint is built for tetrahedral meshes");
    require(up && p_target && loss, MPET_ERR_INVALID, "NULL argument");
    if (!c->adj_loss) c->adj_loss = c->pool.alloc<double>(1);
    launch_misfit(c, up, p_target, dloss, c->adj_loss);
    MPET_CUDA(cudaMemcpyAsync(loss, c->adj_loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MPET_CUDA(cudaStreamSynchronize(c->stream));
    API_END(c)
}

static void require_adjoint_ok(mpet_ctx* c) {
    require(c->dim == 3, MPET_ERR_INVALID, "the adjoint is built for tetrahedral meshes");
    require(!(c->prm.theta < 1.0 && (c->f_beta || c->f_beta_matrix)), MPET_ERR_INVALID,
            "Robin terms are not differentiated for theta < 1");
}

int mpet_adjoint_rhs(mpet_ctx* c, double dt, const double* lam, double* out) {
    API_BEGIN(c)
    require(!c->gmres, MPET_ERR_INVALID, "the adjoint needs a symmetric system (symmetric S)");
    require(!c->setup_done || c->prm.formulation == MPET_FORM_MPET, MPET_ERR_INVALID,
            "built for the MPET form only");
    require(c->setup_done, MPET_ERR_STATE, "mpet_setup must come first");
    require(lam && out && lam != out, MPET_ERR_INVALID, "lam and out must be distinct device arrays");
    require_adjoint_ok(c);
    launch_adjoint_rhs(c, dt, lam, out);
    API_END(c)
}

int mpet_adjoint_step(mpet_ctx* c, double dt, const double* seed, const double* up_prev, const double* up,
                      double* lam, double* grad_K, mpet_stats* st) {
    API_BEGIN(c)
    require(!c->gmres, MPET_ERR_INVALID, "the adjoint needs a symmetric system (symmetric S)");
    require(!c->setup_done || c->prm.formulation == MPET_FORM_MPET, MPET_ERR_INVALID,
            "built for the MPET form only");
    require(c->assembled, MPET_ERR_STATE, "mpet_assemble must come first");
    require(c->precond_ready, MPET_ERR_STATE, "mpet_setup_preconditioner must come first");
    require(seed && lam && lam != seed, MPET_ERR_INVALID, "seed and lam must be distinct device arrays");
    require(!grad_K || (up_prev && up), MPET_ERR_INVALID, "the gradient needs up_prev and up");
    require_adjoint_ok(c);
    for (int a = 0; a < c->J; ++a)
        for (int b = 0; b < a; ++b)
            require(c->prm.S[a * MPET_MAX_NETWORKS + b] == c->prm.S[b * MPET_MAX_NETWORKS + a], MPET_ERR_INVALID,
                    "A^T differs from A for a non-symmetric S");
    if (!c->adj_b) c->adj_b = c->pool.alloc<double>(c->N);
    MPET_CUDA(cudaMemcpyAsync(c->adj_b, seed, sizeof(double) * c->N, cudaMemcpyDeviceToDevice, c->stream));
    launch_zero_bc_rows(c, c->adj_b);
    MPET_CUDA(cudaMemsetAsync(lam, 0, sizeof(double) * c->N, c->stream));
    int s = solve_system(c, c->adj_b, lam, st, true);
    if (s != MPET_OK) {
        c->err = solve_status_message(s);
        return s;
    }
    if (grad_K) launch_adjoint_grad(c, dt, lam, up_prev, up, grad_K);
    API_END(c)
}

}  // extern "C"
