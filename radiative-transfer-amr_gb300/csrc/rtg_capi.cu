// extern "C" entry points of librtg (declared in include/rtg.h).
#include <cstring>
#include <map>
#include <mutex>
#include <functional>
#include <string>
#include <vector>

#include "rtg_internal.h"

namespace rtg {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

std::atomic<long long>& launch_counter() {
    static std::atomic<long long> n{0};
    return n;
}

void raise_smem_limit(const void* func, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> done;
    int dev = 0;
    RTG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = done[std::make_pair(dev, func)];
    if (bytes <= cur) return;
    RTG_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
}

namespace {

template <typename T>
T* upload(rtg_handle* h, const std::vector<T>& v) {
    void* p = nullptr;
    const size_t bytes = sizeof(T) * std::max<size_t>(v.size(), 1);
    RTG_CUDA(cudaMalloc(&p, bytes));
    h->allocs.push_back(p);
    h->table_bytes += (int64_t)bytes;
    if (!v.empty()) RTG_CUDA(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return (T*)p;
}

std::vector<float> to_f32(const std::vector<double>& v) {
    std::vector<float> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = (float)v[i];
    return o;
}

__global__ void gather_kernel(const double* __restrict__ x, const int64_t* __restrict__ idx,
                              double* __restrict__ out, int64_t n) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        out[k] = x[idx[k]];
}

__global__ void scatter_kernel(const double* __restrict__ xi, const int64_t* __restrict__ idx,
                               double* __restrict__ out, int64_t n) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        out[idx[k]] = xi[k];
}

int grid_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 152 * 8); }

// Run fn, turning exceptions into a status code and the thread's error string.
int guard(const char* what, const std::function<void()>& fn) {
    try {
        fn();
        return RTG_OK;
    } catch (const RtgError& e) {
        set_error(std::string(what) + ": " + e.msg);
        return e.code;
    } catch (const std::exception& e) {
        set_error(std::string(what) + ": " + e.what());
        return RTG_ERR_ARG;
    }
}
}  // namespace
}  // namespace rtg

using namespace rtg;

extern "C" {

int rtg_abi_version(void) { return RTG_ABI_VERSION; }

int64_t rtg_launch_count(void) { return (int64_t)rtg::launch_counter().load(); }

const char* rtg_last_error(void) { return g_err.c_str(); }

int rtg_quad_nodes(int kind, int n, double* nodes, double* weights) {
    return guard("rtg_quad_nodes", [&] {
        if (n < 1 || n > kMaxNodes) throw RtgError{RTG_ERR_SIZE, "n outside [1, 16]"};
        if (!nodes || !weights) throw RtgError{RTG_ERR_ARG, "null output"};
        if (kind == 0)
            quad_lgl(n, nodes, weights);
        else if (kind == 1)
            quad_lg(n, nodes, weights);
        else
            throw RtgError{RTG_ERR_ARG, "kind must be 0 (LGL) or 1 (LG)"};
    });
}

int rtg_create(const rtg_mesh_desc* mesh, const rtg_coeffs* coeffs, int device, rtg_handle** out) {
    if (!out) {
        set_error("rtg_create: null output handle");
        return RTG_ERR_ARG;
    }
    *out = nullptr;
    rtg_handle* h = new rtg_handle();
    const int rc = guard("rtg_create", [&] {
        h->device = device;
        RTG_CUDA(cudaSetDevice(device));
        build_tables(mesh, coeffs, h->host);
        HostTables& t = h->host;
        ColDev* cols = upload(h, t.cols);
        ElemDev* elems = upload(h, t.elems);
        CplDev* cpls = upload(h, t.cpls);
        int64_t* woff = upload(h, t.W_off);
        CplGeo* cgeo = upload(h, t.cgeo);
        h->v64.cgeo = cgeo;
        h->v32.cgeo = cgeo;
        OpView<double>& a = h->v64;
        a.cols = cols;
        a.elems = elems;
        a.cpls = cpls;
        a.W_off = woff;
        a.kw = upload(h, t.kw);
        a.sw = upload(h, t.sw);
        a.ang = upload(h, t.ang);
        a.W = upload(h, t.W);
        std::vector<double> wt(t.W.size());
        for (size_t sg = 0; sg + 1 < t.W_off.size(); ++sg) {
            const int64_t o = t.W_off[sg];
            const int n = t.sig_nth[sg];
            for (int r = 0; r < n; ++r)
                for (int c = 0; c < n; ++c) wt[o + (int64_t)c * n + r] = t.W[o + (int64_t)r * n + c];
        }
        a.WT = upload(h, wt);
        a.G = upload(h, t.G);
        a.lglw = upload(h, t.lglw);
        a.mort = upload(h, t.mort);
        a.econst = upload(h, t.econst);
        a.colc = upload(h, t.colc);
        a.cplc = upload(h, t.cplc);
        a.ncols = (int32_t)t.cols.size();
        a.nelem = (int32_t)t.elems.size();
        OpView<float>& b = h->v32;
        b.cols = cols;
        b.elems = elems;
        b.cpls = cpls;
        b.W_off = woff;
        b.kw = upload(h, to_f32(t.kw));
        b.sw = upload(h, to_f32(t.sw));
        b.ang = upload(h, to_f32(t.ang));
        b.W = upload(h, to_f32(t.W));
        b.WT = upload(h, to_f32(wt));
        b.G = upload(h, to_f32(t.G));
        b.lglw = upload(h, to_f32(t.lglw));
        b.mort = upload(h, to_f32(t.mort));
        b.econst = upload(h, to_f32(t.econst));
        b.colc = upload(h, to_f32(t.colc));
        b.cplc = upload(h, to_f32(t.cplc));
        b.ncols = a.ncols;
        b.nelem = a.nelem;
        // index of every unknown in the full vector
        std::vector<int64_t> idx;
        idx.reserve((size_t)t.ndof_interior);
        for (const ElemDev& E : t.elems) {
            const ColDev& C = t.cols[E.col];
            const int bm = E.flags >> 4;
            for (int i = 0; i < C.nx; ++i)
                for (int j = 0; j < C.ny; ++j) {
                    const bool bd = ((bm & 1) && i == C.nx - 1) || ((bm & 2) && j == C.ny - 1) ||
                                    ((bm & 4) && i == 0) || ((bm & 8) && j == 0);
                    if (bd) continue;
                    for (int r = 0; r < E.nth; ++r) idx.push_back(E.dof_off + ((int64_t)i * C.ny + j) * E.nth + r);
                }
        }
        h->d_interior_index = upload(h, idx);
    });
    if (rc != RTG_OK) {
        rtg_destroy(h);
        return rc;
    }
    *out = h;
    return RTG_OK;
}

void rtg_destroy(rtg_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    free_batch(h);
    free_coarse(h);
    free_nn(h);
    free_amr(h);
    free_workspace(h);
    free_sweep(h);
    free_apply_plans(h);
    for (void* p : h->allocs) cudaFree(p);
    delete h;
}

int rtg_get_info(const rtg_handle* h, rtg_info* info) {
    return guard("rtg_get_info", [&] {
        if (!h || !info) throw RtgError{RTG_ERR_ARG, "null argument"};
        const HostTables& t = h->host;
        rtg_info o{};
        o.ndof = t.ndof;
        o.ndof_interior = t.ndof_interior;
        o.ncols = (int32_t)t.cols.size();
        o.nelem = (int32_t)t.elems.size();
        o.ncoupling = (int32_t)t.cpls.size();
        o.nsig = (int32_t)t.sig_nth.size();
        o.max_col_ndof = t.max_col_ndof;
        o.max_nth_col = t.max_nth_col;
        o.table_bytes = h->table_bytes;
        // algorithmic bytes: read x, write y, read kappa and sigma at the spatial nodes
        int64_t nodes = 0, flops = 0;
        for (const ColDev& C : t.cols) {
            nodes += (int64_t)C.nx * C.ny;
            flops += (int64_t)C.ndof * 2 * (C.nx + C.ny + C.nth_col + 1);
        }
        o.bytes_per_apply_fp64 = t.ndof * 16 + nodes * 16;
        o.bytes_per_apply_fp32 = t.ndof * 8 + nodes * 8;
        o.flops_per_apply = flops;
        *info = o;
    });
}

int rtg_apply(rtg_handle* h, uint32_t flags, int prec, const void* x, void* y, void* stream) {
    return guard("rtg_apply", [&] {
        if (!h || !x || !y) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (x == y) throw RtgError{RTG_ERR_ARG, "x and y alias"};
        if (!(flags & (RTG_MASS | RTG_SCAT | RTG_IC | RTG_BC | RTG_SYSTEM)))
            throw RtgError{RTG_ERR_ARG, "no operator component selected"};
        cudaStream_t s = (cudaStream_t)stream;
        if (prec == RTG_FP64)
            launch_apply<double>(h, h->v64, flags, (const double*)x, (double*)y, s);
        else if (prec == RTG_FP32)
            launch_apply<float>(h, h->v32, flags, (const float*)x, (float*)y, s);
        else
            throw RtgError{RTG_ERR_ARG, "unknown precision"};
    });
}

int rtg_precondition(rtg_handle* h, int prec, const void* r, void* z, void* stream) {
    return guard("rtg_precondition", [&] {
        if (!h || !r || !z) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (r == z) throw RtgError{RTG_ERR_ARG, "r and z alias"};
        cudaStream_t s = (cudaStream_t)stream;
        if (prec == RTG_FP64)
            apply_sweep<double>(h, (const double*)r, (double*)z, s);
        else if (prec == RTG_FP32)
            apply_sweep<float>(h, (const float*)r, (float*)z, s);
        else
            throw RtgError{RTG_ERR_ARG, "unknown precision"};
    });
}

int rtg_nn_rows(rtg_handle* h, int64_t* rows) {
    return guard("rtg_nn_rows", [&] {
        if (!h || !rows) throw RtgError{RTG_ERR_ARG, "null argument"};
        *rows = nn_rows(h);
    });
}

int rtg_nn_set_params(rtg_handle* h, const float* params, void* stream) {
    return guard("rtg_nn_set_params", [&] {
        if (!h || !params) throw RtgError{RTG_ERR_ARG, "null argument"};
        nn_set_params(h, params, (cudaStream_t)stream);
    });
}

int rtg_nn_features(rtg_handle* h, float* feat, void* stream) {
    return guard("rtg_nn_features", [&] {
        if (!h || !feat) throw RtgError{RTG_ERR_ARG, "null argument"};
        nn_features(h, feat, (cudaStream_t)stream);
    });
}

int rtg_nn_moments(rtg_handle* h, int prec, const void* z, float* mom, float* scale, void* stream) {
    return guard("rtg_nn_moments", [&] {
        if (!h || !z || !mom || !scale) throw RtgError{RTG_ERR_ARG, "null argument"};
        cudaStream_t s = (cudaStream_t)stream;
        if (prec == RTG_FP64)
            nn_moments<double>(h, (const double*)z, mom, scale, s);
        else if (prec == RTG_FP32)
            nn_moments<float>(h, (const float*)z, mom, scale, s);
        else
            throw RtgError{RTG_ERR_ARG, "unknown precision"};
    });
}

int rtg_nn_forward(const float* params, const float* feat, int64_t rows, float* coef, void* stream) {
    return guard("rtg_nn_forward", [&] {
        if (rows < 0) throw RtgError{RTG_ERR_ARG, "negative row count"};
        if (rows > 0 && (!params || !feat || !coef)) throw RtgError{RTG_ERR_ARG, "null argument"};
        nn_forward(params, feat, rows, coef, (cudaStream_t)stream);
    });
}

int rtg_nn_correct(rtg_handle* h, int prec, const float* coef, void* z, void* stream) {
    return guard("rtg_nn_correct", [&] {
        if (!h || !coef || !z) throw RtgError{RTG_ERR_ARG, "null argument"};
        cudaStream_t s = (cudaStream_t)stream;
        if (prec == RTG_FP64)
            nn_correct<double>(h, coef, (double*)z, s);
        else if (prec == RTG_FP32)
            nn_correct<float>(h, coef, (float*)z, s);
        else
            throw RtgError{RTG_ERR_ARG, "unknown precision"};
    });
}

int rtg_nn_targets(rtg_handle* h, int prec, const void* z, const void* e, const float* scale, float weight,
                   float* stats, void* stream) {
    return guard("rtg_nn_targets", [&] {
        if (!h || !z || !e || !scale || !stats) throw RtgError{RTG_ERR_ARG, "null argument"};
        cudaStream_t s = (cudaStream_t)stream;
        if (prec == RTG_FP64)
            nn_stats<double>(h, (const double*)z, (const double*)e, scale, weight, stats, s);
        else if (prec == RTG_FP32)
            nn_stats<float>(h, (const float*)z, (const float*)e, scale, weight, stats, s);
        else
            throw RtgError{RTG_ERR_ARG, "unknown precision"};
    });
}

int64_t rtg_nn_work_floats(void) { return nn_work_floats(); }

int rtg_nn_loss_grad(const float* params, const float* feat, const float* mom, const float* stats, int64_t rows,
                     float* work, float* grad, double* loss, void* stream) {
    return guard("rtg_nn_loss_grad", [&] {
        if (rows < 0) throw RtgError{RTG_ERR_ARG, "negative row count"};
        if (!params || !work || !grad || (rows > 0 && (!feat || !mom || !stats)))
            throw RtgError{RTG_ERR_ARG, "null argument"};
        nn_loss_grad(params, feat, mom, stats, rows, work, grad, loss, (cudaStream_t)stream);
    });
}

int rtg_nn_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1,
                float beta2, float eps, float wd, void* stream) {
    return guard("rtg_nn_adam", [&] {
        if (!params || !grad || !m || !v) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (step < 1) throw RtgError{RTG_ERR_ARG, "step counts from 1"};
        nn_adam(params, grad, m, v, step, lr, beta1, beta2, eps, wd, (cudaStream_t)stream);
    });
}

int rtg_nn_precondition(rtg_handle* h, int prec, const void* r, void* z, void* stream) {
    return guard("rtg_nn_precondition", [&] {
        if (!h || !r || !z) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (r == z) throw RtgError{RTG_ERR_ARG, "r and z alias"};
        cudaStream_t s = (cudaStream_t)stream;
        if (prec == RTG_FP64) {
            apply_sweep<double>(h, (const double*)r, (double*)z, s);
            apply_learned<double>(h, (double*)z, s);
        } else if (prec == RTG_FP32) {
            apply_sweep<float>(h, (const float*)r, (float*)z, s);
            apply_learned<float>(h, (float*)z, s);
        } else {
            throw RtgError{RTG_ERR_ARG, "unknown precision"};
        }
    });
}

int rtg_error_angular_jump(rtg_handle* h, const double* u, double* cell_err2, double* col_err2, void* stream) {
    return guard("rtg_error_angular_jump", [&] {
        if (!h || !u || !cell_err2) throw RtgError{RTG_ERR_ARG, "null argument"};
        error_angular_jump(h, u, cell_err2, col_err2, (cudaStream_t)stream);
    });
}

int rtg_error_spatial_jump(rtg_handle* h, const double* u, double* col_err2, void* stream) {
    return guard("rtg_error_spatial_jump", [&] {
        if (!h || !u || !col_err2) throw RtgError{RTG_ERR_ARG, "null argument"};
        error_spatial_jump(h, u, col_err2, (cudaStream_t)stream);
    });
}

int rtg_hp_steer(rtg_handle* h, const double* u, double* col_lp, double* cell_lp, void* stream) {
    return guard("rtg_hp_steer", [&] {
        if (!h || !u) throw RtgError{RTG_ERR_ARG, "null argument"};
        hp_steer(h, u, col_lp, cell_lp, (cudaStream_t)stream);
    });
}

int rtg_sweep_info(rtg_handle* h, int* levels, int* lagged, int64_t* inverse_entries, void* stream) {
    return guard("rtg_sweep_info", [&] {
        if (!h) throw RtgError{RTG_ERR_ARG, "null argument"};
        cudaStream_t s = (cudaStream_t)stream;
        if (levels) *levels = sweep_levels_count(h, s);
        if (lagged) *lagged = sweep_lagged_count(h, s);
        if (inverse_entries) *inverse_entries = sweep_inverse_entries(h, s);
    });
}

int rtg_sweep_maps(rtg_handle* h, int prec, int* onephase, int64_t* map_entries, int64_t* upwind_entries,
                   void* stream) {
    return guard("rtg_sweep_maps", [&] {
        if (!h) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (prec != RTG_FP32 && prec != RTG_FP64) throw RtgError{RTG_ERR_ARG, "unknown precision"};
        sweep_maps(h, prec, onephase, map_entries, upwind_entries, (cudaStream_t)stream);
    });
}

int rtg_sweep_trace(rtg_handle* h, int prec, const void* r, void* z, uint64_t* trace, int32_t* level,
                    void* stream) {
    return guard("rtg_sweep_trace", [&] {
        if (!h || !r || !z || !trace) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (r == z) throw RtgError{RTG_ERR_ARG, "r and z alias"};
        cudaStream_t s = (cudaStream_t)stream;
        unsigned long long* tr = reinterpret_cast<unsigned long long*>(trace);
        if (prec == RTG_FP64)
            apply_sweep<double>(h, (const double*)r, (double*)z, s, tr);
        else if (prec == RTG_FP32)
            apply_sweep<float>(h, (const float*)r, (float*)z, s, tr);
        else
            throw RtgError{RTG_ERR_ARG, "unknown precision"};
        if (level) sweep_levels(h, level, s);
    });
}

int rtg_apply_tuning(rtg_handle* h, int32_t* table, int cap_rows, int* nclasses, void* stream) {
    return guard("rtg_apply_tuning", [&] {
        if (!h || !nclasses || (cap_rows > 0 && !table)) throw RtgError{RTG_ERR_ARG, "null argument"};
        *nclasses = apply_tuning(h, table, cap_rows, (cudaStream_t)stream);
    });
}

int rtg_apply_shape(rtg_handle* h, int prec, const int32_t* shape) {
    return guard("rtg_apply_shape", [&] {
        if (!h) throw RtgError{RTG_ERR_ARG, "null handle"};
        if (prec != RTG_FP64 && prec != RTG_FP32) throw RtgError{RTG_ERR_ARG, "prec must be RTG_FP64 or RTG_FP32"};
        // captured graphs hold the old plan's launches: finish the work in
        // flight and drop them with the plan
        RTG_CUDA(cudaSetDevice(h->device));
        RTG_CUDA(cudaDeviceSynchronize());
        free_workspace(h);
        free_batch(h);
        apply_shape(h, prec, shape);
    });
}

int rtg_interior_mask(rtg_handle* h, uint8_t* mask, void* stream) {
    return guard("rtg_interior_mask", [&] {
        if (!h || !mask) throw RtgError{RTG_ERR_ARG, "null argument"};
        launch_interior_mask(h, mask, (cudaStream_t)stream);
    });
}

int rtg_mask_vector(rtg_handle* h, int part, const double* x, double* out, void* stream) {
    return guard("rtg_mask_vector", [&] {
        if (!h || !x || !out) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (part != 0 && part != 1) throw RtgError{RTG_ERR_ARG, "part must be 0 or 1"};
        launch_mask_vector(h, part, x, out, (cudaStream_t)stream);
    });
}

int rtg_split_vector(rtg_handle* h, const double* x, double* x_int, void* stream) {
    return guard("rtg_split_vector", [&] {
        if (!h || !x || !x_int) throw RtgError{RTG_ERR_ARG, "null argument"};
        const int64_t n = h->host.ndof_interior;
        gather_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(x, h->d_interior_index, x_int, n), count_launch();
        RTG_CUDA(cudaGetLastError());
    });
}

int rtg_merge_vectors(rtg_handle* h, const double* x_int, const double* g, double* x, void* stream) {
    return guard("rtg_merge_vectors", [&] {
        if (!h || !x_int || !g || !x) throw RtgError{RTG_ERR_ARG, "null argument"};
        cudaStream_t s = (cudaStream_t)stream;
        launch_mask_vector(h, 1, g, x, s);
        const int64_t n = h->host.ndof_interior;
        scatter_kernel<<<grid_for(n), 256, 0, s>>>(x_int, h->d_interior_index, x, n), count_launch();
        RTG_CUDA(cudaGetLastError());
    });
}

int rtg_weight_forcing(rtg_handle* h, const double* fvals, double* out, void* stream) {
    return guard("rtg_weight_forcing", [&] {
        if (!h || !fvals || !out) throw RtgError{RTG_ERR_ARG, "null argument"};
        launch_weight_forcing(h, fvals, out, (cudaStream_t)stream);
    });
}

int rtg_solve_batched(rtg_handle* h, int nbatch, const int64_t* inst_off, const double* f, const double* g,
                      double* u, const rtg_solve_opts* opts, rtg_solve_info* infos, void* stream) {
    int inner = RTG_OK;
    const int rc = guard("rtg_solve_batched", [&] {
        if (!h || !inst_off || !f || !g || !u || !opts) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (opts->restart < 1 || opts->restart > 60) throw RtgError{RTG_ERR_ARG, "restart outside [1, 60]"};
        inner = solve_batched(h, nbatch, inst_off, f, g, u, opts, infos, (cudaStream_t)stream);
    });
    return rc != RTG_OK ? rc : inner;
}

int rtg_solve(rtg_handle* h, const double* f, const double* g, double* u, const rtg_solve_opts* opts,
              rtg_solve_info* info, double* hist, int hist_cap, void* stream) {
    int inner = RTG_OK;
    const int rc = guard("rtg_solve", [&] {
        if (!h || !f || !g || !u || !opts) throw RtgError{RTG_ERR_ARG, "null argument"};
        if (opts->restart < 1 || opts->restart > 60) throw RtgError{RTG_ERR_ARG, "restart outside [1, 60]"};
        if (opts->method != 0 && opts->method != 1) throw RtgError{RTG_ERR_ARG, "unknown method"};
        if (!(opts->rtol >= 0.) || !(opts->atol >= 0.)) throw RtgError{RTG_ERR_ARG, "bad tolerance"};
        inner = solve(h, f, g, u, opts, info, hist, hist_cap, (cudaStream_t)stream);
    });
    return rc != RTG_OK ? rc : inner;
}

int rtg_solve_hessenberg(rtg_handle* h, double* R, int cap, int32_t* n, void* stream) {
    return guard("rtg_solve_hessenberg", [&] {
        if (!h || !n) throw RtgError{RTG_ERR_ARG, "null argument"};
        int nn = 0;
        last_hessenberg(h, R, cap, &nn, (cudaStream_t)stream);
        *n = nn;
    });
}

}  // extern "C"
