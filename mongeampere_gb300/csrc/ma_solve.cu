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

#include <algorithm>
#include <cmath>
#include <climits>
#include <cstdio>
#include <mutex>
#include <utility>
#include <vector>

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
                           double* relres, int precond, int reuse = 0)
{
    if (precond == MA_PRECOND_MULTIGRID && amg_levels(n) >= 2)
        return amg_pcg_solve(c, n, b, x, rtol, maxiter, reuse, iters, relres);
    cudaStream_t s = c->stream;
    MA_CUDA(c, c->cg_r.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_z.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_p.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_q.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_dinv.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_scal.ensure(sizeof(double) * 8));
    int max_blocks = 0;
    {
        int per_sm = 0, sms = 0;
        MA_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kPcgThreads, 0));
        MA_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
        max_blocks = per_sm * sms;
        if (c->grid_share > 1) max_blocks = std::max(1, max_blocks / c->grid_share);
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
    MA_CUDA(c, ctx_sync(c));
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

// The Newton iteration of MA::ot_solve on one set of sites (device arrays; w in/out).
constexpr double kForcing = 1e-2;  // relative CG residual of a Newton direction (cg_rtol = 0)
constexpr int kAggRefresh = 8;  // Newton steps per multigrid aggregation (the sites do not move; the
                                // Hessian's strengths drift: on the 100,000-site workload 8 steps cost
                                // 11 more CG iterations a solve than 4 and save 3 ms of setup)

// fp64_finish = false: a mixed-precision solve may stop on its mixed residual (the
// intermediate stages of the continuation, whose tolerance is far above the FP32 noise)
// report_value = false: a stage whose value nobody reads (a continuation stage before
// the last, a coarse multiscale level); its evaluations leave out the value's integrals
// and S.value is NaN.
static ma_status newton_core(Ctx* c, const Mesh* m, int n, const double* dx, const double* dy, const double* dnu,
                             double* w, const ma_solve_opts& o, ma_stats& S, bool fp64_finish = true,
                             bool report_value = true)
{
    cudaStream_t s = c->stream;
    const bool default_forcing = !(o.cg_rtol > 0);
    MA_CUDA(c, c->w0.ensure(sizeof(double) * n));
    MA_CUDA(c, c->dirn.ensure(sizeof(double) * n));
    MA_CUDA(c, c->g.ensure(sizeof(double) * n));
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
    // The FP32 integrals leave a noise of 1e-5 to 1e-4 of a cell's mass in the masses
    // (measured up to 3e-4 max-relative at 1M sites): from this relative residual on,
    // where only the quadratically convergent last steps remain, the evaluations are
    // FP64.  Above it the noise cannot decide a line search; a mixed line search that
    // fails all the same is redone in FP64.
    constexpr double kMixedFloor = 1e-2;
    // Only the value of the last evaluation is reported, so the FP64 evaluations leave
    // out the value's integrals (a third of a piece's FP64 edge terms) until the
    // accepted point is within kValueNear of the stopping tolerance; the first
    // evaluation has them (an empty cell there ends the solve with its value), the
    // mixed integrals always do, and a solve whose last evaluation lacks them ends
    // with one FP64 evaluation of the final weights.  fx_valid: fx is the value.
    constexpr double kValueNear = 1e3;
    bool fx_valid = false;
    auto near_end = [&](double gn, double mr) {
        return o.stop_rule == MA_STOP_MAX_REL ? (mr <= kValueNear * o.eps_g) : (gn <= kValueNear * o.eps_g);
    };
    auto timed_eval = [&](const double* wv, bool trial, bool value) -> ma_status {
        cudaEventRecord(e0, s);
        EvalFlags f;
        f.hessian = true;
        f.nu = dnu;
        f.abort_on_empty = trial;
        f.mixed = mixed_phase;
        f.value = value;
        fx_valid = value || f.mixed;
        if (!f.mixed) S.neval_fp64++;
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
        MA_CUDA(c, ctx_sync(c));
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
    if ((st = timed_eval(w, false, report_value)) != MA_OK) {
        result = st;
        goto core_done;
    }
    {
        double fx = c->hstat[0], minm = c->hstat[2], gn = c->hstat[3], mr = c->hstat[4];
        double minnu = c->hstat[15];
        double eps0 = std::fmin(minm, minnu) / 2.0;
        if (!(eps0 > 0)) {
            result = fail(c, MA_EMPTY_CELL, "computed minimum mass is non-positive: a Laguerre cell is empty");
            S.grad_norm = gn;
            S.max_rel_err = mr;
            S.value = fx_valid ? fx : NAN;
            goto core_done;
        }
        int64_t niter = 0;
        for (;;) {
            if (converged(gn, mr) || (mixed_phase && mr <= kMixedFloor)) {
                if (!mixed_phase || (!fp64_finish && converged(gn, mr))) break;
                // the mixed residual has converged: check (and finish) in FP64
                mixed_phase = false;
                if ((st = timed_eval(w, false, report_value)) != MA_OK) {
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
                // the reference's loop test `niter++ <= maxiter` (optimal_transport.hpp:150-151)
                // counts this last, failed test too: Statistics::niter = maxiter + 2
                result = MA_MAXITER;
                niter++;
                break;
            }
            niter++;
            // Newton direction: d = -H_s^{-1} g_s
            k_grad<<<(n + 255) / 256, 256, 0, s>>>(c->mass.as<double>(), dnu, n, c->g.as<double>());
            c->launches += 1;
            cudaEventRecord(e0, s);
            int it = 0;
            double rr = 0;
            // inexact Newton with a constant forcing term: directions to 1e-2 relative
            // residual keep the reference's Newton and evaluation counts (measured on the
            // 64^2 / 1,000-site, 512^2 / 100,000-site and 2048^2 / 1M-site workloads)
            // while tighter solves only cost CG iterations
            double rtol = default_forcing ? kForcing : o.cg_rtol;
            // the multigrid's aggregates are rebuilt every kAggRefresh Newton steps of
            // this solve; the steps between rebuild only its Galerkin matrices
            const int reuse = (niter - 1) % kAggRefresh != 0;
            if ((st = pcg_solve(c, n, c->g.as<double>(), c->dirn.as<double>(), rtol, (int)o.cg_maxiter, &it,
                                &rr, o.precond, reuse)) != MA_OK) {
                result = st;
                break;
            }
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            S.t_linsolve_ms += ms;
            S.cg_iters += it;
            if (!(rr <= rtol * (1.0 + 1e-12))) S.cg_noconv++;  // rr = |r| / |g| of the direction
            MA_CUDA(c, cudaMemcpyAsync(c->w0.p, w, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            double alpha = 1.0, n0 = gn;
            const bool want_value = report_value && near_end(gn, mr);
            bool ok = false;
            while (true) {
                // w = w0 - alpha * solution
                k_axpy_to<<<(n + 255) / 256, 256, 0, s>>>(c->w0.as<double>(), c->dirn.as<double>(), -alpha, n, w);
                c->launches += 1;
                if ((st = timed_eval(w, true, want_value)) != MA_OK) {
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
                if ((st = timed_eval(w, false, report_value)) != MA_OK) {
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
                fprintf(stderr, "it %lld: |df|=%.17g max_rel=%.3g tau=%g eval=%zu cg=%d\n", (long long)niter, gn, mr,
                        alpha, S.neval, it);
        }
        S.niter = (size_t)niter;
        S.grad_norm = gn;
        S.max_rel_err = mr;
        if (report_value && !fx_valid && (result == MA_OK || result == MA_MAXITER)) {
            // the value at the final weights: the same weights evaluated again, in FP64
            // and with the value's integrals
            mixed_phase = false;
            if ((st = timed_eval(w, false, true)) != MA_OK) {
                result = st;
                goto core_done;
            }
            fx = c->hstat[0];
        }
        S.value = fx_valid ? fx : NAN;  // no value after a failed line search
    }
core_done:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return result;
}

// ---------------------------------------------------------------------------
// multiscale initial guess (Merigot, "A multiscale approach to optimal transport",
// 2011): the sites are coarsened by groups of kMsGroup consecutive sites in Morton
// order (nu-weighted centroid, summed target mass) down to about kMsCoarse sites;
// the coarsest problem is solved from w = 0, and each finer level starts from
//     w_i = w_c + 2 (x_i - x_c) . (x_c - z_c)
// (c the parent of i, z_c the rho-centroid of c's Laguerre cell at the coarse
// solution): within a group the power diagram is the group's Voronoi diagram moved
// by z_c - x_c, i.e. placed where the parent's cell is (for clustered sites the
// cells lie far from their sites).  The guess is scaled back towards 0 while a cell
// would be empty; each level is solved to kMsLevelTol before the finest is solved to
// the caller's tolerance.  The Newton iteration on every level is the reference's;
// only the initial guess of the finest one changes, which MA::ot_solve takes as an
// argument.
// ---------------------------------------------------------------------------
constexpr int kMsGroup = 8;
constexpr int kMsCoarse = 4000;
constexpr double kMsLevelTol = 1e-2;

static uint64_t morton2(double x, double y, double x0, double y0, double sx, double sy)
{
    auto spread = [](uint64_t v) {
        v &= 0xFFFFFull;
        v = (v | (v << 16)) & 0x0000FFFF0000FFFFull;
        v = (v | (v << 8)) & 0x00FF00FF00FF00FFull;
        v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0Full;
        v = (v | (v << 2)) & 0x3333333333333333ull;
        v = (v | (v << 1)) & 0x5555555555555555ull;
        return v;
    };
    const double fx = std::min(std::max((x - x0) * sx, 0.0), 1048575.0);
    const double fy = std::min(std::max((y - y0) * sy, 0.0), 1048575.0);
    return spread((uint64_t)fx) | (spread((uint64_t)fy) << 1);
}

struct MsLevel {
    std::vector<double> x, y, nu;
    std::vector<int> parent;  // aggregate (site of the next coarser level) of each site
};

// has the evaluation at w an empty cell?  (a cheap evaluation that stops at the first)
static ma_status has_empty_cell(Ctx* c, const Mesh* m, int n, const double* w, bool* empty)
{
    EvalFlags f;
    f.hessian = true;
    f.abort_on_empty = true;
    ma_status st = run_eval(c, m, n, w, f);
    if (st != MA_OK) return st;
    *empty = c->aborted;
    return MA_OK;
}

static ma_status multiscale_solve(Ctx* c, const Mesh* m, int n, const double* dx, const double* dy,
                                  const double* dnu, double* w, const ma_solve_opts& o, ma_stats& S)
{
    cudaStream_t s = c->stream;
    std::vector<MsLevel> L(1);
    L[0].x.resize(n);
    L[0].y.resize(n);
    L[0].nu.resize(n);
    MA_CUDA(c, cudaMemcpyAsync(L[0].x.data(), dx, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaMemcpyAsync(L[0].y.data(), dy, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaMemcpyAsync(L[0].nu.data(), dnu, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, ctx_sync(c));
    while ((int)L.back().x.size() > kMsCoarse) {
        MsLevel& f = L.back();
        const size_t nf = f.x.size();
        double x0 = f.x[0], x1 = f.x[0], y0 = f.y[0], y1 = f.y[0];
        for (size_t i = 0; i < nf; i++) {
            x0 = std::min(x0, f.x[i]);
            x1 = std::max(x1, f.x[i]);
            y0 = std::min(y0, f.y[i]);
            y1 = std::max(y1, f.y[i]);
        }
        const double sx = x1 > x0 ? 1048576.0 / (x1 - x0) : 0.0, sy = y1 > y0 ? 1048576.0 / (y1 - y0) : 0.0;
        std::vector<std::pair<uint64_t, int>> key(nf);
        for (size_t i = 0; i < nf; i++) key[i] = {morton2(f.x[i], f.y[i], x0, y0, sx, sy), (int)i};
        std::sort(key.begin(), key.end());
        const size_t nc = (nf + kMsGroup - 1) / kMsGroup;
        MsLevel cl;
        cl.x.assign(nc, 0.0);
        cl.y.assign(nc, 0.0);
        cl.nu.assign(nc, 0.0);
        f.parent.assign(nf, 0);
        for (size_t r = 0; r < nf; r++) {
            const int i = key[r].second, J = (int)(r / kMsGroup);
            f.parent[i] = J;
            cl.x[J] += f.nu[i] * f.x[i];
            cl.y[J] += f.nu[i] * f.y[i];
            cl.nu[J] += f.nu[i];
        }
        for (size_t J = 0; J < nc; J++) {
            cl.x[J] /= cl.nu[J];
            cl.y[J] /= cl.nu[J];
        }
        L.push_back(std::move(cl));
    }
    std::vector<double> wl(L.back().x.size(), 0.0);
    for (int l = (int)L.size() - 1; l >= 0; l--) {
        const int nl = (int)L[l].x.size();
        const double *lx = dx, *ly = dy, *lnu = dnu;
        double* lw = w;
        if (l > 0) {
            MA_CUDA(c, c->ms_x.ensure(sizeof(double) * nl));
            MA_CUDA(c, c->ms_y.ensure(sizeof(double) * nl));
            MA_CUDA(c, c->ms_nu.ensure(sizeof(double) * nl));
            MA_CUDA(c, c->ms_w.ensure(sizeof(double) * nl));
            MA_CUDA(c, cudaMemcpyAsync(c->ms_x.p, L[l].x.data(), sizeof(double) * nl, cudaMemcpyHostToDevice, s));
            MA_CUDA(c, cudaMemcpyAsync(c->ms_y.p, L[l].y.data(), sizeof(double) * nl, cudaMemcpyHostToDevice, s));
            MA_CUDA(c, cudaMemcpyAsync(c->ms_nu.p, L[l].nu.data(), sizeof(double) * nl, cudaMemcpyHostToDevice, s));
            lx = c->ms_x.as<double>();
            ly = c->ms_y.as<double>();
            lnu = c->ms_nu.as<double>();
            lw = c->ms_w.as<double>();
        }
        // the initial guess: the prolonged weights, scaled towards 0 while a cell is empty
        std::vector<double> wt(nl);
        double t = 1.0;
        for (int tries = 0;; tries++) {
            for (int i = 0; i < nl; i++) wt[i] = t * wl[i];
            MA_CUDA(c, cudaMemcpyAsync(lw, wt.data(), sizeof(double) * nl, cudaMemcpyHostToDevice, s));
            MA_CUDA(c, ctx_sync(c));
            if (t == 0.0) break;
            ma_status st = build_site_index(c, m, nl, lx, ly, lw);
            if (st != MA_OK) return st;
            bool empty = false;
            if ((st = has_empty_cell(c, m, nl, lw, &empty)) != MA_OK) return st;
            if (!empty) break;
            t = tries < 12 ? 0.5 * t : 0.0;
        }
        ma_solve_opts ol = o;
        if (l > 0) {
            ol.stop_rule = MA_STOP_MAX_REL;
            ol.eps_g = kMsLevelTol;
            ol.verbose = 0;
        }
        ma_stats Sl{};
        ma_status st = newton_core(c, m, nl, lx, ly, lnu, lw, ol, Sl, true, l == 0);
        if (o.verbose)
            fprintf(stderr, "multiscale level %d: %d sites, guess scale %g, status %d, %zu Newton steps, max_rel %.3g\n",
                    l, nl, t, (int)st, Sl.niter, Sl.max_rel_err);
        S.niter += Sl.niter;
        S.neval += Sl.neval;
        S.neval_fp64 += Sl.neval_fp64;
        S.cg_noconv += Sl.cg_noconv;
        S.cg_iters += Sl.cg_iters;
        S.linesearch_halvings += Sl.linesearch_halvings;
        S.t_eval_ms += Sl.t_eval_ms;
        S.t_linsolve_ms += Sl.t_linsolve_ms;
        S.grad_norm = Sl.grad_norm;
        S.max_rel_err = Sl.max_rel_err;
        S.value = Sl.value;
        if (l == 0) return st;
        if (st != MA_OK && st != MA_MAXITER) return st;
        // the coarse solution and the centroids of its cells
        std::vector<double> wc(nl), mo(6 * (size_t)nl);
        {
            EvalFlags f;
            f.hessian = false;
            f.moments = 1;
            if ((st = build_site_index(c, m, nl, lx, ly, lw)) != MA_OK) return st;
            if ((st = run_eval(c, m, nl, lw, f)) != MA_OK) return st;
        }
        MA_CUDA(c, cudaMemcpyAsync(wc.data(), lw, sizeof(double) * nl, cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, cudaMemcpyAsync(mo.data(), c->mom.p, sizeof(double) * 6 * nl, cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, ctx_sync(c));
        const MsLevel& F = L[l - 1];
        const MsLevel& Cl = L[l];
        const std::vector<int>& par = F.parent;
        wl.assign(par.size(), 0.0);
        for (size_t i = 0; i < par.size(); i++) {
            const int J = par[i];
            const double mJ = mo[6 * (size_t)J];
            const double zx = mJ > 0 ? mo[6 * (size_t)J + 1] / mJ : Cl.x[J];
            const double zy = mJ > 0 ? mo[6 * (size_t)J + 2] / mJ : Cl.y[J];
            wl[i] = wc[J] + 2.0 * ((F.x[i] - Cl.x[J]) * (Cl.x[J] - zx) + (F.y[i] - Cl.y[J]) * (Cl.y[J] - zy));
        }
    }
    return MA_OK;
}

// ---------------------------------------------------------------------------
// continuation in the target masses (no counterpart in the reference, whose ot_solve
// takes the initial weights as an argument): from the masses m0 of the initial weights,
// the targets nu_t = m0 + t (nu - m0) are reached stage by stage, each stage the
// reference's damped Newton warm-started from the previous one, with t chosen so that no
// cell's target changes by more than a factor kContFactor from one stage to the next.
// At t = 0 the initial weights solve the problem exactly, so every stage starts from a
// point with no empty cell, which the reference's Kitagawa-Merigot-Thibert rule needs
// (its eps0 = min(m_start, nu_t) / 2 is taken per stage).  For sites far from
// equilibrium (clustered sites on a spread-out density) the damped Newton from w = 0
// cuts every step to a few 2^-11; here the stages are damped too, but converge.
// ---------------------------------------------------------------------------
constexpr double kContFactor = 2.0;
constexpr double kContStageTol = 1e-1;  // max relative residual of an intermediate stage (on the clustered
                                        // 1M-site workload 1e-2 / 5e-2 / 1e-1: 744 / 725 / 711 Newton steps)
constexpr int64_t kContStageIters = 5;  // an intermediate stage may take this many times maxiter

static ma_status continuation_solve(Ctx* c, const Mesh* m, int n, const double* dx, const double* dy,
                                    const double* dnu, double* w, const ma_solve_opts& o, ma_stats& S)
{
    cudaStream_t s = c->stream;
    ma_status st = build_site_index(c, m, n, dx, dy, w);
    if (st != MA_OK) return st;
    {
        EvalFlags f;
        f.hessian = false;
        if ((st = run_eval(c, m, n, w, f)) != MA_OK) return st;
        S.neval++;
        S.neval_fp64++;
    }
    std::vector<double> m0(n), nu(n), nut(n);
    MA_CUDA(c, cudaMemcpyAsync(m0.data(), c->mass.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaMemcpyAsync(nu.data(), dnu, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, ctx_sync(c));
    for (int i = 0; i < n; i++)
        if (!(m0[i] > 0.0))
            return fail(c, MA_EMPTY_CELL, "computed minimum mass is non-positive: a Laguerre cell is empty");
    MA_CUDA(c, c->ms_nu.ensure(sizeof(double) * n));
    double t = 0.0;
    for (int stage = 0;; stage++) {
        // the largest t' with m_t' / m_t in [1 / kContFactor, kContFactor] for every cell
        double tn = 1.0;
        for (int i = 0; i < n; i++) {
            const double d = nu[i] - m0[i], mt = m0[i] + t * d;
            if (d > 0.0)
                tn = std::min(tn, (kContFactor * mt - m0[i]) / d);
            else if (d < 0.0)
                tn = std::min(tn, (m0[i] - mt / kContFactor) / -d);
        }
        tn = std::min(1.0, std::max(tn, t + 1e-6 * (1.0 - t)));
        const bool last = tn >= 1.0;
        const double* target = dnu;
        ma_solve_opts os = o;
        if (!last) {
            for (int i = 0; i < n; i++) nut[i] = m0[i] + tn * (nu[i] - m0[i]);
            MA_CUDA(c, cudaMemcpyAsync(c->ms_nu.p, nut.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
            target = c->ms_nu.as<double>();
            os.stop_rule = MA_STOP_MAX_REL;
            os.eps_g = kContStageTol;
            os.maxiter = o.maxiter * kContStageIters;
        }
        ma_stats Sl{};
        st = newton_core(c, m, n, dx, dy, target, w, os, Sl, last, last);
        if (o.verbose)
            fprintf(stderr, "continuation stage %d: t = %.6g, status %d, %zu Newton steps, %zu evaluations, max_rel %.3g\n",
                    stage, tn, (int)st, Sl.niter, Sl.neval, Sl.max_rel_err);
        S.niter += Sl.niter;
        S.neval += Sl.neval;
        S.neval_fp64 += Sl.neval_fp64;
        S.cg_iters += Sl.cg_iters;
        S.cg_noconv += Sl.cg_noconv;
        S.linesearch_halvings += Sl.linesearch_halvings;
        S.t_eval_ms += Sl.t_eval_ms;
        S.t_linsolve_ms += Sl.t_linsolve_ms;
        S.grad_norm = Sl.grad_norm;
        S.max_rel_err = Sl.max_rel_err;
        S.value = Sl.value;
        if (last || st != MA_OK) return st;
        t = tn;
    }
}

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
    a.maxiter = maxiter <= 0 ? 20000 : (maxiter > INT_MAX ? INT_MAX : (int)maxiter);
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
    // res[1] = |r|, res[2] = |g| of the last iterate: the CG stopped at maxiter or broke
    // down (p.Hp <= 0) unless the residual met the tolerance
    if (!(res[1] <= a.rtol * res[2])) return MA_CG_NOCONV;
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
    o->cg_rtol = 0.0;  // the default forcing term
    o->cg_maxiter = 20000;
    o->precond = MA_PRECOND_MULTIGRID;
    o->init = MA_INIT_GIVEN;
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
    const double tol = rtol > 0 ? rtol : 1e-10;
    const int mit = maxiter <= 0 ? 20000 : (maxiter > INT_MAX ? INT_MAX : (int)maxiter);
    ma_status st = pcg_solve(c, n, dg, dd, tol, mit, &it, &rr, MA_PRECOND_MULTIGRID);
    if (st != MA_OK) return st;
    if (mem == MA_MEM_HOST) {
        MA_CUDA(c, cudaMemcpyAsync(d, dd, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        MA_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    if (iters) *iters = it;
    if (!(rr <= tol * (1.0 + 1e-12)))
        return fail(c, MA_CG_NOCONV, "CG stopped at its iteration cap before reaching rtol");
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
    double* w = c->wcur.as<double>();
    MA_CUDA(c, cudaMemcpyAsync(w, w_inout, sizeof(double) * n,
                               mem == MA_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    ma_status result = o.init == MA_INIT_MULTISCALE     ? multiscale_solve(c, m, n, dx, dy, dnu, w, o, S)
                       : o.init == MA_INIT_CONTINUATION ? continuation_solve(c, m, n, dx, dy, dnu, w, o, S)
                                                        : newton_core(c, m, n, dx, dy, dnu, w, o, S);
    if (result == MA_OK || result == MA_MAXITER || result == MA_LINESEARCH_FAIL) {
        cudaMemcpyAsync(w_inout, w, sizeof(double) * n,
                        mem == MA_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s);
        ctx_sync(c);
    }
    if (stats) *stats = S;
    return result;
}

ma_status ma_w2_flow(ma_ctx* cp, const ma_mesh* mp, int64_t n64, double* x, double* y, const double* nu, double* w,
                     ma_mem mem, int64_t steps, double tau, const ma_solve_opts* opts, ma_stats* stats)
{
    // the iteration of tests/test_zeldovich.cpp:99-119 (and Lloyd's, lloyd.hpp:126-144,
    // for tau = -1): an OT solve, the cells' centroids c, then x <- x + tau (x - c).
    // The solve starts from the previous weights, or from zero when a moved site's
    // cell is empty there.
    Ctx* c = cp;
    if (!c || !mp || !x || !y || !nu || !w || n64 < 1 || steps < 0) return MA_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)n64;
    ma_stats total{};
    std::vector<double> hm(n), hf(2 * n), hx(n), hy(n), hw(n);
    for (int64_t k = 0; k < steps; k++) {
        ma_stats st{};
        ma_status r = ma_ot_solve(cp, mp, n64, x, y, nu, w, mem, opts, &st);
        if (r == MA_EMPTY_CELL) {
            // the moved sites left a cell empty at the previous weights: restart from
            // zero weights (Voronoi cells), as the reference's loop does every step
            if (mem == MA_MEM_DEVICE)
                MA_CUDA(c, cudaMemset(w, 0, sizeof(double) * n));
            else
                std::fill(w, w + n, 0.0);
            r = ma_ot_solve(cp, mp, n64, x, y, nu, w, mem, opts, &st);
        }
        total.niter += st.niter;
        total.neval += st.neval;
        total.neval_fp64 += st.neval_fp64;
        total.cg_noconv += st.cg_noconv;
        total.cg_iters += st.cg_iters;
        total.linesearch_halvings += st.linesearch_halvings;
        total.t_eval_ms += st.t_eval_ms;
        total.t_linsolve_ms += st.t_linsolve_ms;
        total.grad_norm = st.grad_norm;
        total.max_rel_err = st.max_rel_err;
        total.value = st.value;
        if (r != MA_OK) {
            if (stats) *stats = total;
            return r;
        }
        // the centroids, from host copies of the sites and weights
        const cudaMemcpyKind toh = mem == MA_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
        const cudaMemcpyKind fromh = mem == MA_MEM_DEVICE ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
        MA_CUDA(c, cudaMemcpy(hx.data(), x, sizeof(double) * n, toh));
        MA_CUDA(c, cudaMemcpy(hy.data(), y, sizeof(double) * n, toh));
        MA_CUDA(c, cudaMemcpy(hw.data(), w, sizeof(double) * n, toh));
        if ((r = ma_moments(cp, mp, n64, hx.data(), hy.data(), hw.data(), MA_MEM_HOST, hm.data(), hf.data(),
                            nullptr)) != MA_OK)
            return r;
        for (size_t i = 0; i < n; i++) {
            if (!(hm[i] > 0)) continue;  // an empty cell keeps its site
            const double cx = hf[2 * i] / hm[i], cy = hf[2 * i + 1] / hm[i];
            hx[i] += tau * (hx[i] - cx);
            hy[i] += tau * (hy[i] - cy);
        }
        MA_CUDA(c, cudaMemcpy(x, hx.data(), sizeof(double) * n, fromh));
        MA_CUDA(c, cudaMemcpy(y, hy.data(), sizeof(double) * n, fromh));
    }
    if (stats) *stats = total;
    return MA_OK;
}

}  // extern "C"
