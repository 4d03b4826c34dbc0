// Internal definitions of librtg: operator tables on the host and device.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "rtg.h"

namespace rtg {

constexpr int kMaxNodes = 16;          // nodes per direction supported
constexpr double kSmall = 1.e-14;      // 10*EPS drop rule of the (M - S) blocks
constexpr double kBcTol = 1.e-15;      // drop rule of the face terms

void set_error(const std::string& msg);

// Opt a kernel in to `bytes` of dynamic shared memory.  The attribute belongs
// to the function, process-wide, so several handles share it: it is only ever
// raised (per device), never lowered below what another handle launched with.
// The default limit is 48 KB minus the kernel's static shared memory, so any
// launch with dynamic shared memory goes through here.
void raise_smem_limit(const void* func, size_t bytes);

// Kernels launched by the library since it was loaded: every launch statement
// ends with count_launch() (comma operator, so it stays one statement).
std::atomic<long long>& launch_counter();
inline void count_launch() { launch_counter().fetch_add(1, std::memory_order_relaxed); }

struct RtgError {
    int code;
    std::string msg;
};

// check the launch just made (launch errors are reported by the next
// cudaGetLastError, so every launch site checks its own)
#define RTG_LAUNCHED(what)                                                                    \
    do {                                                                                      \
        cudaError_t e_ = cudaGetLastError();                                                  \
        if (e_ != cudaSuccess)                                                                \
            throw ::rtg::RtgError{RTG_ERR_CUDA, std::string("launch of ") + (what) + " (" +    \
                                                    __FILE__ + ":" + RTG_STR(__LINE__) + "): " + \
                                                    cudaGetErrorString(e_)};                  \
    } while (0)
#define RTG_STR2(x) #x
#define RTG_STR(x) RTG_STR2(x)
#define RTG_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            throw ::rtg::RtgError{RTG_ERR_CUDA, std::string(#call) + " (" + __FILE__ + ":" + \
                                                    RTG_STR(__LINE__) + "): " +              \
                                                    cudaGetErrorString(e_)};                 \
    } while (0)

// Per column.
struct ColDev {
    double dx, dy;
    int64_t dof_off;      // first DOF
    int32_t nx, ny;
    int32_t node_off;     // into kw/sw/cw tables (nx*ny entries)
    int32_t elem_begin, elem_end;
    int32_t sig;          // angular mesh id
    int32_t nth_col;      // angular nodes in the column
    int32_t ndof;         // nx*ny*nth_col
    int32_t pad;
};

// Per element (column, leaf cell).
struct ElemDev {
    int64_t dof_off;
    double dth;
    int32_t col;
    int32_t nth;
    int32_t ang;          // offset of this cell's angular table (7*nth doubles)
    int32_t row;          // first angular row of the cell in the column mesh
    int32_t flags;        // bits 0-3 face F outflow, bits 4-7 face F inflow boundary
    int32_t cpl_begin, cpl_end;
    int32_t pad;
};

// Face coupling of an element to one neighbour element.
struct CplDev {
    double dcoeff;        // (dy dth/4) on x-faces, (dx dth/4) on y-faces
    int32_t face;
    int32_t nbr;          // neighbour element
    int32_t es;           // spatial mortar offset ([m1][m0] row-major)
    int32_t et;           // angular mortar offset ([nth1][nth0] row-major)
};

// Where a coupling reads its neighbour's facing node line: entry (jj, a) of
// the line is x[base + jj*stride + a], jj < m1, a < nth1.
struct CplGeo {
    int64_t base;
    int32_t stride;
    int32_t m1;
    int32_t nth1;
    int32_t pad;
};

// Device-side view passed to kernels by value.
template <typename T>
struct OpView {
    const ColDev* cols;
    const ElemDev* elems;
    const CplDev* cpls;
    const T* kw;          // wx wy kappa per node
    const T* sw;          // wx wy sigma per node
    const T* ang;         // per-cell angular tables: wth, wth sin, wth cos, ThF[4]
    const T* W;           // angular scattering matrices per signature
    const int64_t* W_off; // per signature
    const T* G;           // G[n][p][i] = l'_p(x_i) w_i for n nodes, offset n*n*... see gofs
    const T* lglw;        // [kMaxNodes+1][kMaxNodes] LGL weights
    const T* mort;        // spatial + angular mortar matrices
    const T* econst;      // per element: dx dy dth/8, dx dth/4, dy dth/4, 0
    const T* colc;        // per column: dx dy / 8
    const T* cplc;        // per coupling: dcoeff
    const CplGeo* cgeo;   // per coupling: neighbour line addressing
    int32_t ncols;
    int32_t nelem;
    const int32_t* skip = nullptr;   // per column: nonzero = leave the column out (batched solve)
    const int* stop = nullptr;       // nonzero: the launch does nothing (a finished Krylov iteration)
    const T* WT = nullptr;           // W transposed per signature: WT[c][R] = W[R][c]
};

// The sentinel of the sweep's published-value protocol, as raw bits
// (signalling NaNs with a payload; loads and stores move bits, never FP
// values): z holds it until the element that owns a value publishes it.
template <typename T>
struct Sentinel;
template <>
struct Sentinel<float> {
    using U = unsigned int;
    static constexpr U bits = 0x7FBADBADu;
};
template <>
struct Sentinel<double> {
    using U = unsigned long long;
    static constexpr U bits = 0x7FF4BADBADBADBADull;
};

#ifdef __CUDACC__
// Asynchronous global -> shared copies (cp.async): many in flight per thread,
// no registers held; cp_async_wait_all() before the barrier that publishes them.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
template <int kBytes>
__device__ __forceinline__ void cp_async_small(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(src), "n"(kBytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// a / b for 0 <= a < 2^22, given rb = 1/b rounded to nearest float: (a + 1/2)/b
// lies at least 1/(2b) from an integer and the two roundings move it by at
// most (a + 1/2) 2^-23 / b < 1/(2b), so truncation gives the exact quotient.
__device__ __forceinline__ int small_div(int a, float rb) { return (int)(((float)a + 0.5f) * rb); }
#endif

struct HostTables {
    std::vector<ColDev> cols;
    std::vector<ElemDev> elems;
    std::vector<CplDev> cpls;
    std::vector<CplGeo> cgeo;
    std::vector<double> kw, sw, ang, W, G, lglw, mort, econst, colc, cplc;
    std::vector<int64_t> W_off;
    std::vector<int32_t> sig_nth;
    std::vector<int32_t> col_nbr8;   // [ncols][8] distinct neighbour columns, -1 padded
    std::vector<int32_t> col_nbr_raw;  // [ncols][4 faces][2] neighbour columns as given, -1 none
    std::vector<int32_t> col_free;   // [ncols] faces without a neighbour
    std::vector<double> col_pos;     // [ncols][4] x0, y0, x1, y1
    std::vector<double> cell_pos;    // [nelem][2] th0, th1
    std::vector<int32_t> cell_lv, cell_idx;   // [nelem] angular level and index
    int64_t ndof = 0, ndof_interior = 0;
    int32_t nnodes = 0;              // spatial nodes over all columns
    int32_t max_col_ndof = 0, max_nth_col = 0, max_cells_col = 0;
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct Workspace;  // Krylov workspace (rtg_krylov.cu)
struct Sweep;      // sweep preconditioner (rtg_sweep.cu)
struct ApplyPlan;  // column partition of the apply kernels (rtg_apply.cu)
struct BatchWs;    // batched-solve workspace (rtg_batch.cu)
struct NNWs;       // learned correction of the sweep (rtg_nn.cu)
struct Coarse;     // coarse-space correction of the two-level preconditioner (rtg_coarse.cu)
struct AmrTables;  // error indicators and hp steering (rtg_amr.cu)

}  // namespace rtg

struct rtg_handle {
    int device = 0;
    rtg::HostTables host;
    // device copies (FP64 and FP32 variants of the value tables)
    rtg::OpView<double> v64{};
    rtg::OpView<float> v32{};
    std::vector<void*> allocs;
    int64_t table_bytes = 0;
    int64_t* d_interior_index = nullptr;   // [ndof_interior] full index of each unknown
    rtg::Workspace* ws = nullptr;
    rtg::Sweep* sweep = nullptr;
    rtg::ApplyPlan* plan64 = nullptr;
    rtg::ApplyPlan* plan32 = nullptr;
    rtg::BatchWs* bws = nullptr;
    rtg::NNWs* nn = nullptr;
    // precond 3: outcome of the trial that decides whether the learned
    // correction stays in the solve, per inner precision (0 FP64, 1 FP32):
    // 0 not run yet, 1 kept, 2 the sweep alone reduced the residual faster
    int nn_trial[2] = {0, 0};
    // set when a bounded wait of the tensor-core scattering gave up: its
    // copies or MMAs may still have been in flight when the CTA released its
    // shared memory and tensor memory, so neither this handle nor the values it
    // produced are trusted; every later apply or solve on it fails
    bool poisoned = false;
    rtg::Coarse* coarse = nullptr;
    rtg::AmrTables* amr = nullptr;
};

namespace rtg {

// Host builders (rtg_build.cpp)
void quad_lgl(int n, double* x, double* w);
void quad_lg(int n, double* x, double* w);
void build_tables(const rtg_mesh_desc* m, const rtg_coeffs* c, HostTables& t);

// Kernel launchers (rtg_apply.cu)
template <typename T>
void launch_apply(const rtg_handle* h, const OpView<T>& v, uint32_t flags, const T* x, T* y,
                  cudaStream_t s);
void launch_interior_mask(const rtg_handle* h, uint8_t* mask, cudaStream_t s);
void launch_mask_vector(const rtg_handle* h, int part, const double* x, double* out,
                        cudaStream_t s);
void launch_weight_forcing(const rtg_handle* h, const double* f, double* out, cudaStream_t s);
void free_apply_plans(rtg_handle* h);
// RTG_ERR_TIMEOUT (and the handle poisoned) if a tensor-core wait of the FP32
// apply gave up since the plan was built, else RTG_OK; one device read
int apply_status(rtg_handle* h, cudaStream_t s);
// FP32 apply autotuning table (tunes on first use): rows of [nx, ny, nth_b,
// cap, ns per candidate cap]; returns the number of degree classes
int apply_tuning(rtg_handle* h, int32_t* out, int cap_rows, cudaStream_t s);
int apply_shape(rtg_handle* h, int prec, const int32_t* shape);

// Sweep preconditioner (rtg_sweep.cu): z = P^{-1} r
template <typename T>
void apply_sweep(rtg_handle* h, const T* r, T* z, cudaStream_t s);
// prefilled: the caller has written the sentinel over z and reset the claim
// counter (sweep_counter) in an earlier launch on the same stream
template <typename T>
void apply_sweep(rtg_handle* h, const T* r, T* z, cudaStream_t s, unsigned long long* trace,
                 const int32_t* skip = nullptr, const int* stop = nullptr, bool prefilled = false);
unsigned int* sweep_counter(rtg_handle* h, cudaStream_t s);
void sweep_levels(rtg_handle* h, int32_t* level, cudaStream_t s);
void sweep_maps(rtg_handle* h, int prec, int* onephase, int64_t* map_entries, int64_t* upwind, cudaStream_t s);
Sweep* get_sweep(rtg_handle* h, cudaStream_t s);
int sweep_levels_count(rtg_handle* h, cudaStream_t s);
int sweep_lagged_count(rtg_handle* h, cudaStream_t s);
int64_t sweep_inverse_entries(rtg_handle* h, cudaStream_t s);
int sweep_status(rtg_handle* h, cudaStream_t s);
void free_sweep(rtg_handle* h);

// Learned correction of the sweep (rtg_nn.cu)
NNWs* get_nn(rtg_handle* h);
void free_nn(rtg_handle* h);
int64_t nn_rows(rtg_handle* h);
void nn_set_params(rtg_handle* h, const float* params, cudaStream_t s);
bool nn_has_params(rtg_handle* h);
void nn_features(rtg_handle* h, float* feat, cudaStream_t s);
template <typename T>
void nn_moments(rtg_handle* h, const T* z, float* mom, float* scale, cudaStream_t s);
void nn_forward(const float* params, const float* feat, int64_t rows, float* coef, cudaStream_t s);
template <typename T>
void nn_correct(rtg_handle* h, const float* coef, T* z, cudaStream_t s, const int* stop = nullptr);
template <typename T>
void nn_stats(rtg_handle* h, const T* z, const T* err, const float* scale, float weight, float* S, cudaStream_t s);
int64_t nn_work_floats();
void nn_loss_grad(const float* params, const float* feat, const float* mom, const float* stats, int64_t rows,
                  float* work, float* grad, double* loss, cudaStream_t s);
void nn_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float b1, float b2,
             float eps, float wd, cudaStream_t s);
template <typename T>
void apply_learned(rtg_handle* h, T* z, cudaStream_t s, const int* stop = nullptr);

// Two-level preconditioner (rtg_coarse.cu): column diffusion correction
void build_coarse(rtg_handle* h, cudaStream_t s);
void free_coarse(rtg_handle* h);

// Error indicators and hp steering (rtg_amr.cu)
void free_amr(rtg_handle* h);
void error_angular_jump(rtg_handle* h, const double* u, double* cell_err2, double* col_err2, cudaStream_t s);
void error_spatial_jump(rtg_handle* h, const double* u, double* col_err2, cudaStream_t s);
void hp_steer(rtg_handle* h, const double* u, double* col_lp, double* cell_lp, cudaStream_t s);
int64_t error_jump_pairs(rtg_handle* h);
int coarse_size(rtg_handle* h);
void coarse_operator(rtg_handle* h, double* out);
template <typename T>
void apply_coarse(rtg_handle* h, const T* v, T* z, cudaStream_t s);

// Solver (rtg_krylov.cu)
int solve(rtg_handle* h, const double* f, const double* g, double* u, const rtg_solve_opts* o,
          rtg_solve_info* info, double* hist, int hist_cap, cudaStream_t s);
void free_workspace(rtg_handle* h);
int last_hessenberg(rtg_handle* h, double* R, int cap, int* n, cudaStream_t s);

// Batched solve (rtg_batch.cu)
int solve_batched(rtg_handle* h, int nb, const int64_t* inst_off, const double* f, const double* g, double* u,
                  const rtg_solve_opts* o, rtg_solve_info* infos, cudaStream_t s);
void free_batch(rtg_handle* h);

}  // namespace rtg
