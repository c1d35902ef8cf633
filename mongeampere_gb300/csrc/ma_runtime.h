// ma_runtime.h -- host-side state behind the C ABI (context, meshes, buffers).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ma.h"
#include "ma_internal.h"

namespace ma {

// grow-only device buffer
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need)
    {
        if (need <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t nb = need + need / 4 + 256;
        cudaError_t e = cudaMalloc(&p, nb);
        if (e == cudaSuccess) bytes = nb;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
};

struct Ctx;

struct Mesh {
    Ctx* ctx = nullptr;
    int kind = 0;  // 0 grid, 1 triangles
    double X0 = 0, Y0 = 0, X1 = 0, Y1 = 0;
    double total_mass = 0;
    // grid
    int nx = 0, ny = 0;
    DevBuf gx, gy, val, ihx, ihy;
    // triangles
    int nv = 0, nt = 0;
    DevBuf vx, vy, tri, lin, tbin, bin_start, bin_tri;
    int bnx = 0, bny = 0;
    double bx0 = 0, by0 = 0, bcw = 0, bch = 0;
    // host copies of the geometry (new vertex values keep it)
    std::vector<double> hgx, hgy, hvx, hvy;
    std::vector<int> htri;  // counter-clockwise
    MeshGridDev grid_dev() const;
    MeshTriDev tri_dev() const;
};

// aggregation multigrid hierarchy (levels 1.. of the Newton system)
struct AmgBuf {
    DevBuf rp, ci, va, dinv, b, xp, y;  // the level's matrix (levels >= 1) and work vectors
    DevBuf va32, dinv32;                // the FP32 copy of the matrix for the preconditioner
    DevBuf agg, mp, mem;             // its aggregates: row -> node of the next level, member lists
};
struct Amg {
    AmgBuf lev[16];
    DevBuf r1, xs, inv, cnt, rp0, ci0, va0, sp, eci, eva, flag, cinv, ys;
    DevBuf eva32, dinv32, r32a, r32b, q32, s32;  // the fine level's FP32 preconditioner data
    // aggregation scratch: the matching state, the first pass's aggregates and
    // their Galerkin matrix
    DevBuf mate, best, claim, mflag, mid, join, agg1, agg2, mp1, mem1, mfill, rp1, ci1, va1, dinv1, part, counts;
    // the aggregates in lev[].agg/mp/mem: built for the site index of epoch agg_epoch,
    // agg_nlev levels of agg_n[] rows
    int64_t agg_epoch = -1;
    int agg_nlev = 0;
    int agg_n[16] = {};
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = true;
    std::string last_error;
    int64_t launches = 0;

    // inputs (when given in host memory)
    DevBuf hx, hy, hw, hnu;
    // site index: Morton-sorted sites and their radix tree
    int n = 0;
    int64_t index_epoch = 0;  // counts site-index builds
    DevBuf mkeys, mkeys_tmp, hist, hist_scan, perm, sites, posf, scan_scratch, fill;
    DevBuf t_child, t_range, t_parent, t_leaf_parent, t_flag, t_box, t_boxf, t_mom, t_ab, t_nk;
    DevBuf keys, bboxd;  // ordered keys and their doubles
    // evaluation outputs
    DevBuf mass, vpart, mom, rowcnt, st_col, st_val, rowptr, col, val, status, redo, nredo, stat_partial, stat_out;
    DevBuf big_index, big_col, big_val, big_work;  // large-capacity pass
    DevBuf redo64;                                 // mixed form: cells redone in FP64
    DevBuf nb_cnt, nb_lab, cell_box;               // stage 1 -> stage 2
    bool prev_valid = false;                       // nb_cnt/nb_lab match the current site index
    DevBuf abortf;                                 // empty-cell flag of a line-search trial
    DevBuf vjp_cm, vjp_cf, vjp_gx, vjp_gy, vjp_gw, vjp_gr;  // adjoint staging (host callers)
    // materialised pieces of the last ma_pieces call
    DevBuf pc_cnt, pv_cnt, pc_base, pv_base, pc_site, pc_tri, pc_off, pc_xy, pc_edge;
    int64_t npieces = 0, npverts = 0;
    bool have_pieces = false;
    DevBuf raster_col, raster_img;  // rasterisation staging (host callers)
    // cells clipped to a polygon, of the last ma_polygon_cells call (original site order)
    DevBuf pg_poly, pg_cnt, pg_base, pg_off, pg_xy, pg_edge, pg_list, pg_work;
    int64_t pg_n = 0, pg_nv = 0;
    bool have_pgon = false;
    bool aborted = false;                          // the last evaluation stopped at an empty cell
    DevBuf counters;                               // stage-1 search counters (profiling)
    DevBuf info;  // status, nredo, nnz
    int64_t nnz = 0;
    bool have_h = false;
    // solver work vectors
    DevBuf wcur, w0, dirn, g, cg_r, cg_z, cg_p, cg_q, cg_dinv, cg_scal, cg_part;
    DevBuf ms_x, ms_y, ms_nu, ms_w;  // a coarse level of the multiscale initial guess
    // batches: worker contexts (one stream each) and the autotuned worker count
    std::vector<ma_ctx*> workers;
    int batch_workers = 0;
    int grid_share = 1;  // a batch worker's cooperative grids use 1 / grid_share of the GPU
    // a batch worker waits for its stream asleep (an event with cudaEventBlockingSync)
    // rather than spinning, so that more workers than host cores can share the cores
    bool blocking_sync = false;
    cudaEvent_t sync_event = nullptr;
    DevBuf tune_w;                // weight copies of the batch autotuner (device callers)
    std::vector<double> tune_wh;  //                                       (host callers)
    Amg amg;
    // profiling (CUDA events around the main kernels)
    bool prof = false;
    ma_profile profile{};
    cudaEvent_t pev[2] = {nullptr, nullptr};
    // pinned host mirror of small results
    double* hstat = nullptr;  // 16 doubles
    int* hinfo = nullptr;     // 8 ints
};

// wait for the context's stream: cudaStreamSynchronize, or asleep on an event for a
// context with blocking_sync
inline cudaError_t ctx_sync(Ctx* c)
{
    if (!c->blocking_sync) return cudaStreamSynchronize(c->stream);
    if (!c->sync_event) {
        cudaError_t e = cudaEventCreateWithFlags(&c->sync_event, cudaEventBlockingSync | cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaEventRecord(c->sync_event, c->stream);
    if (e != cudaSuccess) return e;
    return cudaEventSynchronize(c->sync_event);
}

// error helpers
ma_status fail(Ctx* c, ma_status s, const std::string& msg);
ma_status cuda_fail(Ctx* c, cudaError_t e, const char* what);

#define MA_CUDA(ctx, call)                                        \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return ::ma::cuda_fail(ctx, _e, #call); \
    } while (0)

// evaluation pipeline (device pointers)
ma_status build_site_index(Ctx* c, const Mesh* m, int n, const double* x, const double* y, const double* w);
ma_status build_site_index_box(Ctx* c, double X0, double Y0, double X1, double Y1, int n, const double* x,
                               const double* y, const double* w);
// caller arrays on the device: host arrays are copied into `buf`, device arrays used in place
ma_status stage_in(Ctx* c, DevBuf& buf, const double* src, int64_t n, ma_mem mem, const double** dst);
// adjoint of one evaluation: cotangents in, gradients out (device, original order)
struct VjpArgs {
    double cot_value = 0.0;
    const double* cot_mass = nullptr;  // n or null
    const double* cot_first = nullptr; // 2n (x, y per site) or null
    double* grad_x = nullptr;
    double* grad_y = nullptr;
    double* grad_w = nullptr;
    double* grad_rho = nullptr;  // mesh vertices (zeroed by the caller) or null
};

struct EvalFlags {
    bool hessian = true;
    const VjpArgs* vjp = nullptr;  // when set: the adjoint instead of the outputs
    bool pieces = false;           // materialise the pieces instead of the outputs
    bool mixed = false;            // FP32 piece integrals (cell sums, predicates and vertices of
                                   // the clip stay certified / FP64)
    int moments = 0;  // 0 none, 1 first, 2 second
    const double* nu = nullptr;  // when given, stat_out[0] = value - <nu, w>
    // Newton line-search trial: an empty cell already rejects the trial (its mass 0
    // is below eps0 > 0), so the evaluation stops at the first one and sets
    // Ctx::aborted instead of computing the rest
    bool abort_on_empty = false;
    // the Kantorovich value's integrals (int rho |x - x_i|^2, a third of an FP64 piece's
    // edge terms): a Newton solve needs the value of its last evaluation only
    bool value = true;
};
ma_status run_eval(Ctx* c, const Mesh* m, int n, const double* w, const EvalFlags& f);
// Newton linear solve H[:n-1,:n-1] x = b with the multigrid-preconditioned CG (ma_amg.cu);
// reuse != 0 keeps the aggregates of the last hierarchy built for the same site index
// (only the Galerkin matrices are rebuilt)
int amg_levels(int n);
ma_status amg_pcg_solve(Ctx* c, int n, const double* b, double* x, double rtol, int maxiter, int reuse, int* iters,
                        double* relres);

// bracket an enqueue with profiling events; the elapsed time is added after a sync
struct ProfScope {
    Ctx* c;
    double* ms;
    int64_t* cnt;  // nullable
    bool done = false;
    ProfScope(Ctx* c_, double* ms_, int64_t* cnt_) : c(c_), ms(ms_), cnt(cnt_)
    {
        if (c->prof) cudaEventRecord(c->pev[0], c->stream);
    }
    void end()
    {
        if (done) return;
        done = true;
        if (!c->prof) return;
        cudaEventRecord(c->pev[1], c->stream);
        cudaEventSynchronize(c->pev[1]);
        float t = 0;
        cudaEventElapsedTime(&t, c->pev[0], c->pev[1]);
        *ms += t;
        if (cnt) (*cnt)++;
    }
    ~ProfScope() { end(); }
};

}  // namespace ma

// the opaque handles of the C ABI
struct ma_ctx : public ma::Ctx {};
struct ma_mesh : public ma::Mesh {};
