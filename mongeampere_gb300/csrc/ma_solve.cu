// ma_solve.cu -- the damped Newton OT solve.
//
// MA::ot_solve (include/MA/optimal_transport.hpp:89-193) restated on the device:
//   * f(w) = kantorovich(w) - <nu, w>, gradient m(w) - nu, Hessian H(w);
//   * eps0 = min(min m(w0), min nu) / 2; a non-positive eps0 is MA_EMPTY_CELL (:137-148);
//   * Newton direction of solve_laplacian_matrix (:41-87): H with its last row and
//     column removed, d[n-1] = 0 -- here by conjugate gradients in one cooperative
//     kernel (no host round trip per iteration), preconditioned by an aggregation
//     multigrid V-cycle (ma_amg.cu) or by the diagonal;
//   * backtracking: accept w0 + a d when min m >= eps0 and |g| <= (1 - a/2) |g0|,
//     else halve a (:158-176), bounded at a = 2^-40;
//   * stop when |g|_2 < eps_g (:150), or max_i |g_i| / nu_i <= eps_g.
#include <cooperative_groups.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "ma_runtime.h"

namespace cg = cooperative_groups;

namespace ma {

// ---------------------------------------------------------------------------
// vector kernels
// ---------------------------------------------------------------------------
__global__ void k_grad(const double* m, const double* nu, int n, double* g)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) g[i] = m[i] - nu[i];
}

__global__ void k_axpy_to(const double* w0, const double* d, double a, int n, double* w)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w[i] = w0[i] + a * d[i];
}

// inverse diagonal of H (0 for the gauge row and for empty rows)
__global__ void k_dinv(const int* rowptr, const int* col, const double* val, int n, double* dinv)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 0.0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
        if (col[k] == i) d = val[k];
    dinv[i] = (i == n - 1 || d == 0.0) ? 0.0 : 1.0 / d;
}

__global__ void k_min_nu(const double* nu, int n, double* out)
{
    __shared__ double sh[256];
    double m = INFINITY;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmin(m, nu[i]);
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sh[0];
}

// ---------------------------------------------------------------------------
// cooperative Jacobi-PCG on H[:n-1, :n-1]
// ---------------------------------------------------------------------------
struct PcgArgs {
    int n;
    const int* rowptr;
    const int* col;
    const double* val;
    const double* dinv;
    const double* b;  // right-hand side (component n-1 ignored)
    double* x;
    double* r;
    double* z;
    double* p;
    double* q;
    double* part;     // 3 * gridDim.x partial sums
    double* out;      // [iterations, |r|, |b|]
    double rtol;
    int maxiter;
};

constexpr int kPcgThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
        for (int k = 0; k < kPcgThreads / 32; k++) s += sh[k];
        sh[32] = s;
    }
    __syncthreads();
    s = sh[32];
    __syncthreads();
    return s;
}

// every block reduces the per-block partials in the same order: identical values
// in all blocks, so every block takes the same branch
__device__ __forceinline__ double grid_total(const double* part, int nb, double* sh)
{
    double v = 0.0;
    for (int k = threadIdx.x; k < nb; k += kPcgThreads) v += part[k];
    return block_sum(v, sh);
}

__global__ void __launch_bounds__(kPcgThreads) k_pcg(PcgArgs a)
{
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[40];
    const int nb = gridDim.x;
    const int m = a.n - 1;  // active unknowns: 0 .. n-2
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;

    double l_rz = 0.0, l_bb = 0.0;
    for (int i = tid; i < a.n; i += stride) {
        double bi = (i < m) ? a.b[i] : 0.0;
        double zi = a.dinv[i] * bi;
        a.x[i] = 0.0;
        a.r[i] = bi;
        a.z[i] = zi;
        a.p[i] = zi;
        l_rz += bi * zi;
        l_bb += bi * bi;
    }
    double s_rz = block_sum(l_rz, sh), s_bb = block_sum(l_bb, sh);
    if (threadIdx.x == 0) {
        a.part[blockIdx.x] = s_rz;
        a.part[nb + blockIdx.x] = s_bb;
    }
    grid.sync();
    double rz = grid_total(a.part, nb, sh);
    double bb = grid_total(a.part + nb, nb, sh);
    double bnorm = sqrt(bb);
    double tol = a.rtol * bnorm;
    int it = 0;
    double rr = bb;
    grid.sync();
    while (it < a.maxiter && sqrt(rr) > tol && rz > 0.0) {
        // q = H p and p.q
        double l_pq = 0.0;
        for (int i = tid; i < a.n; i += stride) {
            double s = 0.0;
            if (i < m) {
                for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; k++) {
                    int j = a.col[k];
                    if (j < m) s += a.val[k] * a.p[j];
                }
            }
            a.q[i] = s;
            l_pq += s * a.p[i];
        }
        double s_pq = block_sum(l_pq, sh);
        if (threadIdx.x == 0) a.part[blockIdx.x] = s_pq;
        grid.sync();
        double pq = grid_total(a.part, nb, sh);
        if (!(pq > 0.0)) break;
        double alpha = rz / pq;
        double l_rz2 = 0.0, l_rr = 0.0;
        for (int i = tid; i < a.n; i += stride) {
            double xi = a.x[i] + alpha * a.p[i];
            double ri = a.r[i] - alpha * a.q[i];
            double zi = a.dinv[i] * ri;
            a.x[i] = xi;
            a.r[i] = ri;
            a.z[i] = zi;
            l_rz2 += ri * zi;
            l_rr += ri * ri;
        }
        double s1 = block_sum(l_rz2, sh), s2 = block_sum(l_rr, sh);
        if (threadIdx.x == 0) {
            a.part[nb + blockIdx.x] = s1;
            a.part[2 * nb + blockIdx.x] = s2;
        }
        grid.sync();
        double rz2 = grid_total(a.part + nb, nb, sh);
        rr = grid_total(a.part + 2 * nb, nb, sh);
        double beta = rz2 / rz;
        rz = rz2;
        for (int i = tid; i < a.n; i += stride) a.p[i] = a.z[i] + beta * a.p[i];
        it++;
        grid.sync();
    }
    if (tid == 0) {
        a.out[0] = (double)it;
        a.out[1] = sqrt(rr);
        a.out[2] = bnorm;
    }
}

// solve H[:n-1,:n-1] x = b (b, x device vectors of length n; x[n-1] = 0)
static ma_status pcg_solve(Ctx* c, int n, const double* b, double* x, double rtol, int maxiter, int* iters,
                           double* relres, int precond)
{
    if (precond == MA_PRECOND_MULTIGRID && amg_levels(n) >= 2)
        return amg_pcg_solve(c, n, b, x, rtol, maxiter, iters, relres);
    cudaStream_t s = c->stream;
    MA_CUDA(c, c->cg_r.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_z.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_p.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_q.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_dinv.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_scal.ensure(sizeof(double) * 8));
    static int max_blocks = 0;
    if (max_blocks == 0) {
        int per_sm = 0, sms = 0;
        MA_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kPcgThreads, 0));
        MA_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
        max_blocks = per_sm * sms;
    }
    int want = (n + kPcgThreads - 1) / kPcgThreads;
    int nb = want < max_blocks ? want : max_blocks;
    if (nb < 1) nb = 1;
    MA_CUDA(c, c->cg_part.ensure(sizeof(double) * 3 * nb));
    k_dinv<<<(n + 255) / 256, 256, 0, s>>>(c->rowptr.as<int>(), c->col.as<int>(), c->val.as<double>(), n,
                                             c->cg_dinv.as<double>());
    PcgArgs a;
    a.n = n;
    a.rowptr = c->rowptr.as<int>();
    a.col = c->col.as<int>();
    a.val = c->val.as<double>();
    a.dinv = c->cg_dinv.as<double>();
    a.b = b;
    a.x = x;
    a.r = c->cg_r.as<double>();
    a.z = c->cg_z.as<double>();
    a.p = c->cg_p.as<double>();
    a.q = c->cg_q.as<double>();
    a.part = c->cg_part.as<double>();
    a.out = c->cg_scal.as<double>();
    a.rtol = rtol;
    a.maxiter = maxiter;
    void* args[] = {&a};
    {
        ProfScope ps(c, &c->profile.pcg_ms, &c->profile.pcg_launches);
        MA_CUDA(c, cudaLaunchCooperativeKernel((void*)k_pcg, dim3(nb), dim3(kPcgThreads), args, 0, s));
    }
    c->launches += 2;
    MA_CUDA(c, cudaMemcpyAsync(c->hstat + 8, c->cg_scal.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaStreamSynchronize(s));
    if (iters) *iters = (int)c->hstat[8];
    c->profile.pcg_iters += (int64_t)c->hstat[8];
    if (relres) *relres = c->hstat[10] > 0 ? c->hstat[9] / c->hstat[10] : 0.0;
    return MA_OK;
}

// ---------------------------------------------------------------------------
// Newton linear solve without any allocation
// ---------------------------------------------------------------------------
// Some callers cannot let a library allocate device memory: applications that
// hand all device memory to their own pool or arena up front and forbid any
// allocation outside it, and latency-critical loops where the device-wide
// synchronisation of cudaMalloc/cudaFree is not acceptable.  For them the
// Jacobi-PCG work vectors live in this fixed array, reserved when the library is
// loaded and kept by every GPU that loads it until the process exits.
constexpr int64_t kStaticMaxN = (int64_t)1 << 18;  // largest system: 262,144 sites
constexpr int kStaticMaxBlocks = 4096;              // per-block partial sums of the CG kernel
constexpr size_t kStaticDoubles = 5 * (size_t)kStaticMaxN + 3 * (size_t)kStaticMaxBlocks + 8;
static __device__ __align__(256) double g_static_pcg[kStaticDoubles];  // 10.1 MB

// per-device address of g_static_pcg and the co-resident block count of k_pcg,
// looked up once per device with that device current
struct StaticSetup {
    bool done = false;
    double* base = nullptr;
    int max_blocks = 0;
};
static std::mutex g_static_mutex;
static StaticSetup g_static_setup[64];

static ma_status static_setup(int dev, StaticSetup* out)
{
    if (dev < 0 || dev >= 64) return MA_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_static_mutex);
    StaticSetup& st = g_static_setup[dev];
    if (!st.done) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_static_pcg) != cudaSuccess) {
            cudaGetLastError();
            return MA_ERR_CUDA;
        }
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kPcgThreads, 0) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return MA_ERR_CUDA;
        }
        st.base = static_cast<double*>(ptr);
        st.max_blocks = per_sm * sms < kStaticMaxBlocks ? per_sm * sms : kStaticMaxBlocks;
        st.done = true;
    }
    *out = st;
    return MA_OK;
}

}  // namespace ma

using namespace ma;

extern "C" {

ma_status ma_laplacian_solve_static(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                                    const double* g, double* d, double rtol, int64_t maxiter, int64_t* iters,
                                    void* stream)
{
    if (n < 1 || !rowptr || !col || !val || !g || !d) return MA_ERR_INVALID_ARGUMENT;
    if (n > kStaticMaxN) return MA_ERR_BUFFER_TOO_SMALL;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return MA_ERR_NO_DEVICE;
    }
    StaticSetup su;
    ma_status st = static_setup(dev, &su);
    if (st != MA_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int ni = (int)n;
    double* base = su.base;
    double* dinv = base;
    double* r = base + kStaticMaxN;
    double* z = base + 2 * kStaticMaxN;
    double* p = base + 3 * kStaticMaxN;
    double* q = base + 4 * kStaticMaxN;
    double* part = base + 5 * kStaticMaxN;
    double* out = part + 3 * kStaticMaxBlocks;
    k_dinv<<<(ni + 255) / 256, 256, 0, s>>>(rowptr, col, val, ni, dinv);
    int want = (ni + kPcgThreads - 1) / kPcgThreads;
    int nb = want < su.max_blocks ? want : su.max_blocks;
    if (nb < 1) nb = 1;
    PcgArgs a;
    a.n = ni;
    a.rowptr = rowptr;
    a.col = col;
    a.val = val;
    a.dinv = dinv;
    a.b = g;
    a.x = d;
    a.r = r;
    a.z = z;
    a.p = p;
    a.q = q;
    a.part = part;
    a.out = out;
    a.rtol = rtol > 0 ? rtol : 1e-10;
    a.maxiter = maxiter > 0 ? (int)maxiter : 20000;
    void* args[] = {&a};
    if (cudaLaunchCooperativeKernel((void*)k_pcg, dim3(nb), dim3(kPcgThreads), args, 0, s) != cudaSuccess) {
        cudaGetLastError();
        return MA_ERR_CUDA;
    }
    double res[3] = {0, 0, 0};
    if (cudaMemcpyAsync(res, out, sizeof(res), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return MA_ERR_CUDA;
    }
    if (iters) *iters = (int64_t)res[0];
    return MA_OK;
}

void ma_solve_opts_default(ma_solve_opts* o)
{
    if (!o) return;
    o->eps_g = 1e-7;
    o->maxiter = 100;
    o->stop_rule = MA_STOP_GRAD_NORM;
    o->precision = MA_FP64;
    o->verbose = 0;
    o->cg_rtol = 0.0;  // adaptive forcing
    o->cg_maxiter = 20000;
    o->precond = MA_PRECOND_MULTIGRID;
}

ma_status ma_laplacian_solve(ma_ctx* cp, const double* g, double* d, ma_mem mem, double rtol, int64_t maxiter,
                             int64_t* iters)
{
    Ctx* c = cp;
    if (!c || !g || !d) return MA_ERR_INVALID_ARGUMENT;
    if (!c->have_h) return fail(c, MA_ERR_INVALID_ARGUMENT, "no Hessian has been computed");
    cudaSetDevice(c->device);
    int n = c->n;
    MA_CUDA(c, c->g.ensure(sizeof(double) * n));
    MA_CUDA(c, c->dirn.ensure(sizeof(double) * n));
    const double* dg = g;
    if (mem == MA_MEM_HOST) {
        MA_CUDA(c, cudaMemcpyAsync(c->g.p, g, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        dg = c->g.as<double>();
    }
    double* dd = (mem == MA_MEM_HOST) ? c->dirn.as<double>() : d;
    int it = 0;
    double rr = 0;
    ma_status st = pcg_solve(c, n, dg, dd, rtol > 0 ? rtol : 1e-10, maxiter > 0 ? (int)maxiter : 20000, &it, &rr,
                             MA_PRECOND_MULTIGRID);
    if (st != MA_OK) return st;
    if (mem == MA_MEM_HOST) {
        MA_CUDA(c, cudaMemcpyAsync(d, dd, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        MA_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    if (iters) *iters = it;
    return MA_OK;
}

ma_status ma_ot_solve(ma_ctx* cp, const ma_mesh* mp, int64_t n64, const double* x, const double* y, const double* nu,
                      double* w_inout, ma_mem mem, const ma_solve_opts* opts, ma_stats* stats)
{
    Ctx* c = cp;
    const Mesh* m = mp;
    if (!c || !m || !x || !y || !nu || !w_inout || n64 < 1 || n64 > ((int64_t)1 << 30)) return MA_ERR_INVALID_ARGUMENT;
    ma_solve_opts o;
    ma_solve_opts_default(&o);
    if (opts) o = *opts;
    const bool adaptive = !(o.cg_rtol > 0);
    if (o.cg_maxiter <= 0) o.cg_maxiter = 20000;
    const int n = (int)n64;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    ma_stats S{};
    // inputs on the device
    const double *dx = x, *dy = y, *dnu = nu;
    if (mem == MA_MEM_HOST) {
        MA_CUDA(c, c->hx.ensure(sizeof(double) * n));
        MA_CUDA(c, c->hy.ensure(sizeof(double) * n));
        MA_CUDA(c, c->hnu.ensure(sizeof(double) * n));
        MA_CUDA(c, cudaMemcpyAsync(c->hx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        MA_CUDA(c, cudaMemcpyAsync(c->hy.p, y, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        MA_CUDA(c, cudaMemcpyAsync(c->hnu.p, nu, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        dx = c->hx.as<double>();
        dy = c->hy.as<double>();
        dnu = c->hnu.as<double>();
    }
    MA_CUDA(c, c->wcur.ensure(sizeof(double) * n));
    MA_CUDA(c, c->w0.ensure(sizeof(double) * n));
    MA_CUDA(c, c->dirn.ensure(sizeof(double) * n));
    MA_CUDA(c, c->g.ensure(sizeof(double) * n));
    double* w = c->wcur.as<double>();
    MA_CUDA(c, cudaMemcpyAsync(w, w_inout, sizeof(double) * n,
                               mem == MA_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    ma_status st = build_site_index(c, m, n, dx, dy, w);
    if (st != MA_OK) return st;

    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // mixed precision: evaluations with FP32 piece integrals until their residual
    // meets the stopping rule, then FP64 evaluations (and FP64 Newton steps if the
    // FP64 residual is not yet below it): the stopping test is always made on FP64
    // masses
    bool mixed_phase = o.precision == MA_MIXED;
    // the FP32 integrals are good to about 1e-5 of a cell's mass: below this relative
    // residual the mixed evaluations stop helping the Newton iteration
    constexpr double kMixedFloor = 1e-4;
    auto timed_eval = [&](const double* wv, bool trial) -> ma_status {
        cudaEventRecord(e0, s);
        EvalFlags f;
        f.hessian = true;
        f.nu = dnu;
        f.abort_on_empty = trial;
        f.mixed = mixed_phase;
        if (!mixed_phase) S.neval_fp64++;
        ma_status r = run_eval(c, m, n, wv, f);
        if (r != MA_OK) return r;
        cudaEventRecord(e1, s);
        if (c->aborted) {
            // value, -, min mass, |g|, max rel: the trial is rejected on its min mass
            c->hstat[0] = NAN;
            c->hstat[2] = 0.0;
            c->hstat[3] = INFINITY;
            c->hstat[4] = INFINITY;
        } else {
            MA_CUDA(c, cudaMemcpyAsync(c->hstat, c->stat_out.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        MA_CUDA(c, cudaStreamSynchronize(s));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        S.t_eval_ms += ms;
        S.neval++;
        return MA_OK;
    };
    auto converged = [&](double gn, double mr) {
        return o.stop_rule == MA_STOP_MAX_REL ? (mr <= o.eps_g) : (gn < o.eps_g);
    };

    ma_status result = MA_OK;
    MA_CUDA(c, c->cg_scal.ensure(sizeof(double) * 8));
    k_min_nu<<<1, 256, 0, s>>>(dnu, n, c->cg_scal.as<double>() + 7);
    c->launches += 1;
    MA_CUDA(c, cudaMemcpyAsync(c->hstat + 15, c->cg_scal.as<double>() + 7, sizeof(double), cudaMemcpyDeviceToHost, s));
    if ((st = timed_eval(w, false)) != MA_OK) {
        result = st;
        goto done;
    }
    {
        double fx = c->hstat[0], minm = c->hstat[2], gn = c->hstat[3], mr = c->hstat[4];
        double minnu = c->hstat[15];
        double eps0 = std::fmin(minm, minnu) / 2.0;
        if (!(eps0 > 0)) {
            result = fail(c, MA_EMPTY_CELL, "computed minimum mass is non-positive: a Laguerre cell is empty");
            S.grad_norm = gn;
            S.max_rel_err = mr;
            S.value = fx;
            goto done;
        }
        int64_t niter = 0;
        const double g0 = gn > 0 ? gn : 1.0;
        for (;;) {
            if (converged(gn, mr) || (mixed_phase && mr <= kMixedFloor)) {
                if (!mixed_phase) break;
                // the mixed residual has converged: check (and finish) in FP64
                mixed_phase = false;
                if ((st = timed_eval(w, false)) != MA_OK) {
                    result = st;
                    break;
                }
                fx = c->hstat[0];
                minm = c->hstat[2];
                gn = c->hstat[3];
                mr = c->hstat[4];
                continue;
            }
            if (niter > o.maxiter) {
                result = MA_MAXITER;
                break;
            }
            niter++;
            // Newton direction: d = -H_s^{-1} g_s
            k_grad<<<(n + 255) / 256, 256, 0, s>>>(c->mass.as<double>(), dnu, n, c->g.as<double>());
            c->launches += 1;
            cudaEventRecord(e0, s);
            int it = 0;
            double rr = 0;
            // inexact Newton: the linear solve only needs to beat the current residual
            double rtol = adaptive ? std::fmin(1e-3, std::fmax(1e-12, 0.1 * gn / g0)) : o.cg_rtol;
            if ((st = pcg_solve(c, n, c->g.as<double>(), c->dirn.as<double>(), rtol, (int)o.cg_maxiter, &it,
                                &rr, o.precond)) != MA_OK) {
                result = st;
                break;
            }
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            S.t_linsolve_ms += ms;
            S.cg_iters += it;
            MA_CUDA(c, cudaMemcpyAsync(c->w0.p, w, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            double alpha = 1.0, n0 = gn;
            bool ok = false;
            while (true) {
                // w = w0 - alpha * solution
                k_axpy_to<<<(n + 255) / 256, 256, 0, s>>>(c->w0.as<double>(), c->dirn.as<double>(), -alpha, n, w);
                c->launches += 1;
                if ((st = timed_eval(w, true)) != MA_OK) {
                    result = st;
                    break;
                }
                fx = c->hstat[0];
                minm = c->hstat[2];
                gn = c->hstat[3];
                mr = c->hstat[4];
                if (minm >= eps0 && gn <= (1.0 - alpha / 2.0) * n0) {
                    ok = true;
                    break;
                }
                alpha *= 0.5;
                S.linesearch_halvings++;
                if (o.verbose)
                    fprintf(stderr, "subit %lld: min(masses)=%.17g\n", (long long)niter, minm);
                if (alpha < 0x1p-40) break;
            }
            if (result != MA_OK) break;
            if (!ok && mixed_phase) {
                // the mixed residual is at its noise level: redo this step in FP64
                mixed_phase = false;
                MA_CUDA(c, cudaMemcpyAsync(w, c->w0.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
                if ((st = timed_eval(w, false)) != MA_OK) {
                    result = st;
                    break;
                }
                fx = c->hstat[0];
                minm = c->hstat[2];
                gn = c->hstat[3];
                mr = c->hstat[4];
                continue;
            }
            if (!ok) {
                result = fail(c, MA_LINESEARCH_FAIL, "line search failed");
                break;
            }
            if (o.verbose)
                fprintf(stderr, "it %lld: f=%.17g |df|=%.17g max_rel=%.3g tau=%g eval=%zu cg=%d\n", (long long)niter, fx,
                        gn, mr, alpha, S.neval, it);
        }
        S.niter = (size_t)niter;
        S.grad_norm = gn;
        S.max_rel_err = mr;
        S.value = fx;
    }
done:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (result == MA_OK || result == MA_MAXITER || result == MA_LINESEARCH_FAIL) {
        cudaMemcpyAsync(w_inout, w, sizeof(double) * n,
                        mem == MA_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s);
        cudaStreamSynchronize(s);
    }
    if (stats) *stats = S;
    return result;
}

}  // extern "C"
