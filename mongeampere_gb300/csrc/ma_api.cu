// ma_api.cu -- the C ABI: contexts, meshes, and one Laguerre evaluation
// (MA::kantorovich, include/MA/kantorovich.hpp:35-141; MA::first_moment /
// second_moment / lloyd, include/MA/lloyd.hpp:30-144).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ma_runtime.h"

using namespace ma;

namespace ma {

ma_status fail(Ctx* c, ma_status s, const std::string& msg)
{
    if (c) c->last_error = msg;
    return s;
}

ma_status cuda_fail(Ctx* c, cudaError_t e, const char* what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (c) c->last_error = m;
    if (e == cudaErrorMemoryAllocation) return MA_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MA_ERR_NO_DEVICE;
    return MA_ERR_CUDA;
}

MeshGridDev Mesh::grid_dev() const
{
    MeshGridDev d;
    d.nx = nx;
    d.ny = ny;
    d.gx = gx.as<double>();
    d.gy = gy.as<double>();
    d.val = val.as<double>();
    d.ihx = ihx.as<double>();
    d.ihy = ihy.as<double>();
    return d;
}

MeshTriDev Mesh::tri_dev() const
{
    MeshTriDev d;
    d.nv = nv;
    d.nt = nt;
    d.vx = vx.as<double>();
    d.vy = vy.as<double>();
    d.tri = tri.as<int>();
    d.lin = lin.as<double>();
    d.tbin = tbin.as<int4>();
    d.bnx = bnx;
    d.bny = bny;
    d.bx0 = bx0;
    d.by0 = by0;
    d.bcw = bcw;
    d.bch = bch;
    d.bin_start = bin_start.as<int>();
    d.bin_tri = bin_tri.as<int>();
    return d;
}


// Build the site index: Morton keys over the bounding box of sites and mesh, a radix
// sort, the radix tree and its node boxes.  Positions only: once per set of sites.
ma_status build_site_index(Ctx* c, const Mesh* m, int n, const double* x, const double* y, const double* w)
{
    return build_site_index_box(c, m->X0, m->Y0, m->X1, m->Y1, n, x, y, w);
}

// the same over the bounding box of the sites and of the box [X0, X1] x [Y0, Y1]
ma_status build_site_index_box(Ctx* c, double X0, double Y0, double X1, double Y1, int n, const double* x,
                               const double* y, const double* w)
{
    cudaStream_t s = c->stream;
    if (n >= (1 << 24)) return fail(c, MA_ERR_INVALID_ARGUMENT, "at most 2^24 - 1 sites per problem");
    MA_CUDA(c, c->keys.ensure(8 * sizeof(unsigned long long)));
    MA_CUDA(c, c->bboxd.ensure(8 * sizeof(double)));
    unsigned long long init[5] = {~0ull, 0ull, ~0ull, 0ull, 0ull};
    MA_CUDA(c, cudaMemcpyAsync(c->keys.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
    launch_bbox(x, y, nullptr, n, c->keys.as<unsigned long long>(), s);
    launch_key_to_double(c->keys.as<unsigned long long>(), c->bboxd.as<double>(), 4, s);
    c->launches += 2;
    MA_CUDA(c, cudaMemcpyAsync(c->hstat, c->bboxd.p, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, ctx_sync(c));
    double xmin = c->hstat[0], xmax = c->hstat[1], ymin = c->hstat[2], ymax = c->hstat[3];
    if (!(std::isfinite(xmin) && std::isfinite(xmax) && std::isfinite(ymin) && std::isfinite(ymax)))
        return fail(c, MA_ERR_INVALID_ARGUMENT, "non-finite site coordinates");
    xmin = std::min(xmin, X0);
    xmax = std::max(xmax, X1);
    ymin = std::min(ymin, Y0);
    ymax = std::max(ymax, Y1);
    int nb = radix_sort_blocks(n);
    size_t nn = (size_t)n;
    size_t ni = nn > 1 ? nn - 1 : 1;
    MA_CUDA(c, c->mkeys.ensure(sizeof(uint64_t) * nn));
    MA_CUDA(c, c->mkeys_tmp.ensure(sizeof(uint64_t) * nn));
    MA_CUDA(c, c->hist.ensure(sizeof(int) * 256 * (size_t)nb));
    MA_CUDA(c, c->hist_scan.ensure(sizeof(int) * (256 * (size_t)nb + 1)));
    MA_CUDA(c, c->perm.ensure(sizeof(int) * nn));
    MA_CUDA(c, c->sites.ensure(sizeof(SiteD) * nn));
    MA_CUDA(c, c->posf.ensure(sizeof(float2) * nn));
    size_t scr = std::max(scan_scratch_ints(256 * nb), scan_scratch_ints(n));
    MA_CUDA(c, c->scan_scratch.ensure(sizeof(int) * scr));
    MA_CUDA(c, c->t_child.ensure(sizeof(int2) * ni));
    MA_CUDA(c, c->t_range.ensure(sizeof(int2) * ni));
    MA_CUDA(c, c->t_parent.ensure(sizeof(int) * ni));
    MA_CUDA(c, c->t_leaf_parent.ensure(sizeof(int) * nn));
    MA_CUDA(c, c->t_flag.ensure(sizeof(int) * ni));
    MA_CUDA(c, c->t_box.ensure(sizeof(double4) * ni));
    MA_CUDA(c, c->t_boxf.ensure(sizeof(float4) * ni));
    MA_CUDA(c, c->t_mom.ensure(tree_mom_bytes(n)));
    MA_CUDA(c, c->t_ab.ensure(sizeof(double4) * ni));
    MA_CUDA(c, c->t_nk.ensure(sizeof(float4) * ni));
    launch_morton(x, y, n, xmin, ymin, xmax, ymax, c->mkeys.as<uint64_t>(), s);
    launch_radix_sort(c->mkeys.as<uint64_t>(), c->mkeys_tmp.as<uint64_t>(), n, c->hist.as<int>(),
                      c->hist_scan.as<int>(), c->scan_scratch.as<int>(), s);
    launch_perm_gather(c->mkeys.as<uint64_t>(), x, y, w, n, c->perm.as<int>(), c->sites.as<SiteD>(),
                       c->posf.as<float2>(), s);
    if (n == 1) {
        int minus1 = -1;
        MA_CUDA(c, cudaMemcpyAsync(c->t_leaf_parent.p, &minus1, sizeof(int), cudaMemcpyHostToDevice, s));
    }
    launch_tree(c->mkeys.as<uint64_t>(), n, c->t_child.as<int2>(), c->t_range.as<int2>(), c->t_parent.as<int>(),
                c->t_leaf_parent.as<int>(), s);
    launch_tree_boxes(c->sites.as<SiteD>(), n, c->t_child.as<int2>(), c->t_parent.as<int>(),
                      c->t_leaf_parent.as<int>(), c->t_flag.as<int>(), c->t_box.as<double4>(),
                      c->t_boxf.as<float4>(), s);
    c->launches += 1 + 8 * 5 + 1 + 2;
    c->n = n;
    c->index_epoch++;
    c->prev_valid = false;
    return MA_OK;
}

static ma_status ensure_eval_buffers(Ctx* c, int n, bool mom)
{
    MA_CUDA(c, c->mass.ensure(sizeof(double) * (size_t)n));
    MA_CUDA(c, c->vpart.ensure(sizeof(double) * (size_t)n));
    if (mom) MA_CUDA(c, c->mom.ensure(sizeof(double) * 6 * (size_t)n));
    MA_CUDA(c, c->rowcnt.ensure(sizeof(int) * (size_t)n));
    const size_t scap = (size_t)small_row_cap();
    MA_CUDA(c, c->st_col.ensure(sizeof(int) * scap * (size_t)n));
    MA_CUDA(c, c->st_val.ensure(sizeof(double) * scap * (size_t)n));
    MA_CUDA(c, c->big_index.ensure(sizeof(int) * (size_t)n));
    MA_CUDA(c, c->nb_cnt.ensure(sizeof(int) * (size_t)n));
    MA_CUDA(c, c->nb_lab.ensure(sizeof(int) * (size_t)stage1_cap() * (size_t)n));
    MA_CUDA(c, c->cell_box.ensure(sizeof(double4) * (size_t)n));
    MA_CUDA(c, c->rowptr.ensure(sizeof(int) * ((size_t)n + 1)));
    MA_CUDA(c, c->status.ensure(sizeof(uint32_t) * 4));
    MA_CUDA(c, c->redo.ensure(sizeof(int) * (size_t)n));
    MA_CUDA(c, c->nredo.ensure(sizeof(int) * 4));
    int nb = stats_blocks(n);
    MA_CUDA(c, c->stat_partial.ensure(sizeof(double) * 5 * (size_t)nb));
    MA_CUDA(c, c->stat_out.ensure(sizeof(double) * 16));
    MA_CUDA(c, c->keys.ensure(8 * sizeof(unsigned long long)));
    MA_CUDA(c, c->bboxd.ensure(8 * sizeof(double)));
    size_t guess = (size_t)n * 8 + 64;
    MA_CUDA(c, c->col.ensure(sizeof(int) * guess));
    MA_CUDA(c, c->val.ensure(sizeof(double) * guess));
    return MA_OK;
}

// main pass: stage 1 (cells) then stage 2 (pieces); cap_kind 1: large-capacity pass.
// mode: 0 evaluation, 1 with moments, 2 adjoint
static void launch_cells(Ctx* c, const Mesh* m, const CellArgs& a, int cap_kind, int mode)
{
    const bool mom = mode == 1;
    if (cap_kind == 0) {
        {
            ProfScope ps(c, &c->profile.cells_ms, &c->profile.cells_launches);
            launch_cells_stage1(a, c->stream);
        }
        {
            ProfScope ps(c, &c->profile.pieces_ms, &c->profile.pieces_launches);
            if (m->kind == 0)
                launch_pieces_grid(a, m->grid_dev(), mode, c->stream);
            else
                launch_pieces_tri(a, m->tri_dev(), mode, c->stream);
        }
        c->launches += 2;
    } else {
        if (m->kind == 0)
            launch_cells_large_grid(a, m->grid_dev(), mom, c->stream);
        else
            launch_cells_large_tri(a, m->tri_dev(), mom, c->stream);
        c->launches += 1;
    }
}

// One Laguerre evaluation for the sites of the current grid with weights w (device,
// original order).  Leaves mass, vpart (and mom), the CSR Hessian and the statistics
// in the context.
ma_status run_eval(Ctx* c, const Mesh* m, int n, const double* w, const EvalFlags& f)
{
    cudaStream_t s = c->stream;
    ma_status st = ensure_eval_buffers(c, n, f.moments > 0);
    if (st != MA_OK) return st;
    launch_update_weights(w, c->perm.as<int>(), n, c->sites.as<SiteD>(), s);
    {
        ProfScope ps(c, &c->profile.bounds_ms, &c->profile.bounds_launches);
        launch_tree_bounds(c->sites.as<SiteD>(), n, c->t_child.as<int2>(), c->t_range.as<int2>(),
                           c->t_parent.as<int>(), c->t_leaf_parent.as<int>(), c->t_flag.as<int>(),
                           c->t_box.as<double4>(), c->t_boxf.as<float4>(), c->t_mom.p,
                           c->t_ab.as<double4>(), c->t_nk.as<float4>(), s);
    }
    c->launches += 1 + tree_bounds_launches(n);
    MA_CUDA(c, cudaMemsetAsync(c->status.p, 0, sizeof(uint32_t) * 4, s));
    MA_CUDA(c, cudaMemsetAsync(c->nredo.p, 0, sizeof(int) * 4, s));
    MA_CUDA(c, cudaMemsetAsync(c->big_index.p, 0xFF, sizeof(int) * (size_t)n, s));

    CellArgs a;
    a.n = n;
    a.sites = c->sites.as<SiteD>();
    a.perm = c->perm.as<int>();
    a.tree.n = n;
    a.tree.child = c->t_child.as<int2>();
    a.tree.range = c->t_range.as<int2>();
    a.tree.box = c->t_box.as<double4>();
    a.tree.boxf = c->t_boxf.as<float4>();
    a.tree.ab = c->t_ab.as<double4>();
    a.tree.nk = c->t_nk.as<float4>();
    a.tree.posf = c->posf.as<float2>();
    a.tree.parent = c->t_parent.as<int>();
    a.tree.leaf_parent = c->t_leaf_parent.as<int>();
    a.X0 = m->X0;
    a.Y0 = m->Y0;
    a.X1 = m->X1;
    a.Y1 = m->Y1;
    a.mass = c->mass.as<double>();
    a.vpart = c->vpart.as<double>();
    a.value = f.value ? 1 : 0;
    a.mom = f.moments > 0 ? c->mom.as<double>() : nullptr;
    a.rowcnt = c->rowcnt.as<int>();
    a.st_col = c->st_col.as<int>();
    a.st_val = c->st_val.as<double>();
    a.scap = small_row_cap();
    a.status = c->status.as<uint32_t>();
    a.redo = c->redo.as<int>();
    a.nredo = c->nredo.as<int>();
    a.work = nullptr;
    a.nwork = 0;
    a.scratch = nullptr;
    a.cell_list = nullptr;
    a.ncell_list = 0;
    MA_CUDA(c, c->redo64.ensure(sizeof(int) * (size_t)n));
    a.redo64 = c->redo64.as<int>();
    a.nredo64 = c->nredo.as<int>() + 2;
    a.prev_valid = c->prev_valid ? 1 : 0;
    a.counters = nullptr;
    a.abort_flag = nullptr;
    c->aborted = false;
    if (f.abort_on_empty) {
        MA_CUDA(c, c->abortf.ensure(sizeof(int) * 4));
        MA_CUDA(c, cudaMemsetAsync(c->abortf.p, 0, sizeof(int), s));
        a.abort_flag = c->abortf.as<int>();
    }
    if (c->prof) {
        MA_CUDA(c, c->counters.ensure(12 * sizeof(unsigned long long)));
        MA_CUDA(c, cudaMemsetAsync(c->counters.p, 0, 12 * sizeof(unsigned long long), s));
        a.counters = c->counters.as<unsigned long long>();
    }
    a.nb_cnt = c->nb_cnt.as<int>();
    a.nb_lab = c->nb_lab.as<int>();
    a.cell_box = c->cell_box.as<double4>();
    a.big_index = c->big_index.as<int>();
    a.big_col = nullptr;
    a.big_val = nullptr;
    a.big_cap = large_row_cap();
    a.cot_value = 0.0;
    a.cot_mass = nullptr;
    a.cot_mom = nullptr;
    a.grad_x = a.grad_y = a.grad_w = a.grad_rho = nullptr;
    if (f.vjp) {
        a.cot_value = f.vjp->cot_value;
        a.cot_mass = f.vjp->cot_mass;
        a.cot_mom = f.vjp->cot_first;
        a.grad_x = f.vjp->grad_x;
        a.grad_y = f.vjp->grad_y;
        a.grad_w = f.vjp->grad_w;
        a.grad_rho = f.vjp->grad_rho;
    }
    a.pc_cnt = a.pv_cnt = nullptr;
    a.pc_base = a.pv_base = nullptr;
    a.out_site = a.out_tri = a.out_edge = nullptr;
    a.out_off = nullptr;
    a.out_xy = nullptr;
    if (f.pieces) {
        MA_CUDA(c, c->pc_cnt.ensure(sizeof(int) * ((size_t)n + 1)));
        MA_CUDA(c, c->pv_cnt.ensure(sizeof(int) * ((size_t)n + 1)));
        MA_CUDA(c, c->pc_base.ensure(sizeof(int) * ((size_t)n + 1)));
        MA_CUDA(c, c->pv_base.ensure(sizeof(int) * ((size_t)n + 1)));
        MA_CUDA(c, cudaMemsetAsync(c->pc_cnt.p, 0, sizeof(int) * ((size_t)n + 1), s));
        MA_CUDA(c, cudaMemsetAsync(c->pv_cnt.p, 0, sizeof(int) * ((size_t)n + 1), s));
        a.pc_cnt = c->pc_cnt.as<int>();
        a.pv_cnt = c->pv_cnt.as<int>();
    }
    const int mode = f.pieces ? 3 : (f.vjp ? (f.mixed ? 6 : 2) : (f.moments > 0 ? 1 : (f.mixed ? 5 : 0)));
    launch_cells(c, m, a, 0, mode);
    c->hinfo[2] = 0;
    if (mode == 5)
        MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 2, c->nredo.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaMemcpyAsync(c->hinfo, c->nredo.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 1, c->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    c->hinfo[3] = 0;
    if (a.abort_flag)
        MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 3, a.abort_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, ctx_sync(c));
    if (c->hinfo[3]) {
        // a line-search trial with an empty cell: nothing else is computed
        c->aborted = true;
        c->have_h = false;
        return MA_OK;
    }
    int nredo = c->hinfo[0];
    if (mode == 5 && c->hinfo[2] > 0) {
        // mixed: the cells whose certified FP32 mass error exceeds its bound, in FP64
        // (ordered on the stream before everything that reads the outputs)
        CellArgs r = a;
        r.cell_list = c->redo64.as<int>();
        r.ncell_list = c->hinfo[2];
        {
            ProfScope ps(c, &c->profile.pieces_ms, &c->profile.pieces_launches);
            if (m->kind == 0)
                launch_pieces_grid(r, m->grid_dev(), 0, s);
            else
                launch_pieces_tri(r, m->tri_dev(), 0, s);
        }
        c->launches += 1;
    }
    if (f.pieces) {
        // the count pass is done: offsets, then the emit pass over the same cells
        c->have_h = false;
        c->have_pieces = false;
        if ((uint32_t)c->hinfo[1] & ST_BAD_INPUT) return fail(c, MA_ERR_INVALID_ARGUMENT, "non-finite site or weight");
        // cells beyond stage 1's capacity or whose clips meet exact ties: counted (and
        // below emitted) one thread per cell with exact predicates
        CellArgs b = a;
        const MeshGridDev gd = m->grid_dev();
        const MeshTriDev td = m->tri_dev();
        if (nredo > 0) {
            b.abort_flag = nullptr;
            b.work = c->redo.as<int>();
            b.nwork = nredo;
            MA_CUDA(c, c->big_work.ensure(large_work_bytes() * (size_t)nredo));
            b.scratch = c->big_work.p;
            b.nredo = c->nredo.as<int>() + 1;
            {
                ProfScope ps(c, &c->profile.cells_large_ms, &c->profile.cells_large_launches);
                launch_cells_large_list(b, m->kind == 0 ? &gd : nullptr, m->kind == 0 ? nullptr : &td, false, s);
            }
            c->launches += 2;
            c->profile.large_sites += nredo;
            MA_CUDA(c, cudaMemcpyAsync(c->hinfo, c->nredo.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
            MA_CUDA(c, ctx_sync(c));
            if (c->hinfo[0] > 0)
                return fail(c, MA_ERR_CAPACITY, "a Laguerre cell has more vertices than the largest kernel capacity");
        }
        launch_scan(c->pc_cnt.as<int>(), c->pc_base.as<int>(), n, c->scan_scratch.as<int>(), s);
        launch_scan(c->pv_cnt.as<int>(), c->pv_base.as<int>(), n, c->scan_scratch.as<int>(), s);
        MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 4, c->pc_base.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 5, c->pv_base.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, ctx_sync(c));
        const int64_t np = c->hinfo[4], nv = c->hinfo[5];
        MA_CUDA(c, c->pc_site.ensure(sizeof(int) * (size_t)(np + 1)));
        MA_CUDA(c, c->pc_tri.ensure(sizeof(int) * (size_t)(np + 1)));
        MA_CUDA(c, c->pc_off.ensure(sizeof(int64_t) * (size_t)(np + 1)));
        MA_CUDA(c, c->pc_xy.ensure(sizeof(double) * 2 * (size_t)(nv + 1)));
        MA_CUDA(c, c->pc_edge.ensure(sizeof(int) * (size_t)(nv + 1)));
        a.pc_base = c->pc_base.as<int>();
        a.pv_base = c->pv_base.as<int>();
        a.out_site = c->pc_site.as<int>();
        a.out_tri = c->pc_tri.as<int>();
        a.out_off = c->pc_off.as<int64_t>();
        a.out_xy = c->pc_xy.as<double>();
        a.out_edge = c->pc_edge.as<int>();
        if (m->kind == 0)
            launch_pieces_grid(a, m->grid_dev(), 4, s);
        else
            launch_pieces_tri(a, m->tri_dev(), 4, s);
        c->launches += 5;
        if (nredo > 0) {
            b.pc_base = a.pc_base;
            b.pv_base = a.pv_base;
            b.out_site = a.out_site;
            b.out_tri = a.out_tri;
            b.out_off = a.out_off;
            b.out_xy = a.out_xy;
            b.out_edge = a.out_edge;
            launch_cells_large_list(b, m->kind == 0 ? &gd : nullptr, m->kind == 0 ? nullptr : &td, true, s);
            c->launches += 1;
        }
        MA_CUDA(c, cudaMemcpyAsync(c->pc_off.as<int64_t>() + np, &nv, sizeof(int64_t), cudaMemcpyHostToDevice, s));
        MA_CUDA(c, ctx_sync(c));
        c->npieces = np;
        c->npverts = nv;
        c->have_pieces = true;
        return MA_OK;
    }
    if (f.vjp) {
        c->have_h = false;
        if (nredo > 0)
            return fail(c, MA_ERR_CAPACITY,
                        "the adjoint handles cells of at most 48 neighbours whose pieces need no exact predicate");
        uint32_t vb = (uint32_t)c->hinfo[1];
        if (vb & ST_BAD_INPUT) return fail(c, MA_ERR_INVALID_ARGUMENT, "non-finite site or weight");
        return MA_OK;
    }
    if (nredo > 0) {
        // sites whose cell outgrew the small capacity: redo them with the large one
        CellArgs b = a;
        b.abort_flag = nullptr;  // every redone cell must complete: its mass is used
        b.work = c->redo.as<int>();
        b.nwork = nredo;
        MA_CUDA(c, c->fill.ensure(sizeof(int) * ((size_t)n + 4)));
        MA_CUDA(c, c->big_work.ensure(large_work_bytes() * (size_t)nredo));
        MA_CUDA(c, c->big_col.ensure(sizeof(int) * (size_t)large_row_cap() * nredo));
        MA_CUDA(c, c->big_val.ensure(sizeof(double) * (size_t)large_row_cap() * nredo));
        b.scratch = c->big_work.p;
        b.big_col = c->big_col.as<int>();
        b.big_val = c->big_val.as<double>();
        b.redo = c->fill.as<int>();
        b.nredo = c->nredo.as<int>() + 1;
        {
            ProfScope ps(c, &c->profile.cells_large_ms, &c->profile.cells_large_launches);
            launch_cells(c, m, b, 1, mode);
        }
        c->profile.large_sites += nredo;
        MA_CUDA(c, cudaMemcpyAsync(c->hinfo, c->nredo.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 1, c->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, ctx_sync(c));
        if (c->hinfo[0] > 0)
            return fail(c, MA_ERR_CAPACITY, "a Laguerre cell has more vertices than the largest kernel capacity");
    }
    if (a.counters) {
        unsigned long long cnt[12];
        MA_CUDA(c, cudaMemcpy(cnt, a.counters, sizeof(cnt), cudaMemcpyDeviceToHost));
        for (int q = 0; q < 6; q++) c->profile.search[q] += (int64_t)cnt[q];
        for (int q = 0; q < 4; q++) c->profile.mixed[q] += (int64_t)cnt[6 + q];
    }
    uint32_t stbits = (uint32_t)c->hinfo[1];
    c->prev_valid = true;
    if (stbits & ST_EXACT_OVERFLOW)
        return fail(c, MA_ERR_EXACT_OVERFLOW, "an exact predicate exceeded its expansion capacity");
    if (stbits & ST_BAD_INPUT) return fail(c, MA_ERR_INVALID_ARGUMENT, "non-finite site or weight");

    c->have_h = false;
    if (f.hessian) {
        launch_scan(c->rowcnt.as<int>(), c->rowptr.as<int>(), n, c->scan_scratch.as<int>(), s);
        c->launches += 2;
        MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 2, c->rowptr.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, ctx_sync(c));
        int64_t nnz = c->hinfo[2];
        MA_CUDA(c, c->col.ensure(sizeof(int) * (size_t)(nnz + 1)));
        MA_CUDA(c, c->val.ensure(sizeof(double) * (size_t)(nnz + 1)));
        launch_csr_compact(n, c->rowptr.as<int>(), c->rowcnt.as<int>(), c->st_col.as<int>(), c->st_val.as<double>(),
                           small_row_cap(), c->big_index.as<int>(), c->big_col.as<int>(), c->big_val.as<double>(),
                           large_row_cap(), c->col.as<int>(), c->val.as<double>(), s);
        c->launches += 1;
        c->nnz = nnz;
        c->have_h = true;
    }
    int nb = stats_blocks(n);
    launch_stats(c->mass.as<double>(), c->vpart.as<double>(), f.nu, w, n, c->stat_partial.as<double>(), nb,
                 c->stat_out.as<double>(), s);
    c->launches += 2;
    return MA_OK;
}

// stage caller arrays on the device: host arrays are copied into context buffers
ma_status stage_in(Ctx* c, DevBuf& buf, const double* src, int64_t n, ma_mem mem, const double** dst)
{
    if (mem == MA_MEM_DEVICE) {
        *dst = src;
        return MA_OK;
    }
    MA_CUDA(c, buf.ensure(sizeof(double) * (size_t)n));
    MA_CUDA(c, cudaMemcpyAsync(buf.p, src, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    *dst = buf.as<double>();
    return MA_OK;
}

}  // namespace ma

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

const char* ma_status_string(ma_status s)
{
    switch (s) {
    case MA_OK: return "ok";
    case MA_ERR_INVALID_ARGUMENT: return "invalid argument";
    case MA_ERR_NO_DEVICE: return "no usable CUDA device";
    case MA_ERR_CUDA: return "CUDA error";
    case MA_ERR_OUT_OF_MEMORY: return "out of device memory";
    case MA_ERR_CAPACITY: return "cell capacity exceeded";
    case MA_ERR_EXACT_OVERFLOW: return "exact predicate capacity exceeded";
    case MA_EMPTY_CELL: return "a Laguerre cell is empty";
    case MA_LINESEARCH_FAIL: return "line search failed";
    case MA_MAXITER: return "maximum number of iterations reached";
    case MA_ERR_BUFFER_TOO_SMALL: return "buffer too small";
    case MA_CG_NOCONV: return "conjugate gradients stopped before reaching the requested residual";
    }
    return "unknown status";
}

ma_status ma_ctx_create(int device, ma_ctx** out)
{
    if (!out) return MA_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return MA_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return MA_ERR_INVALID_ARGUMENT;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return MA_ERR_NO_DEVICE;
    if (prop.major != 10 || prop.minor != 3) return MA_ERR_NO_DEVICE;  // built for sm_103a only
    if (cudaSetDevice(device) != cudaSuccess) return MA_ERR_NO_DEVICE;
    ma_ctx* c = new ma_ctx();
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return MA_ERR_CUDA;
    }
    if (cudaMallocHost(&c->hstat, 16 * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&c->hinfo, 8 * sizeof(int)) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return MA_ERR_OUT_OF_MEMORY;
    }
    *out = c;
    return MA_OK;
}

void ma_ctx_destroy(ma_ctx* c)
{
    if (!c) return;
    for (ma_ctx* w : c->workers) ma_ctx_destroy(w);
    c->workers.clear();
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    DevBuf* bufs[] = {&c->counters, &c->nb_cnt, &c->nb_lab, &c->cell_box, &c->hx, &c->hy, &c->hw, &c->hnu, &c->abortf, &c->vjp_cm, &c->vjp_cf,
                      &c->vjp_gx, &c->vjp_gy, &c->vjp_gw, &c->vjp_gr, &c->pc_cnt, &c->pv_cnt,
                      &c->pc_base, &c->pv_base, &c->pc_site, &c->pc_tri, &c->pc_off, &c->pc_xy, &c->pc_edge,
                      &c->raster_col, &c->raster_img, &c->pg_poly, &c->pg_cnt, &c->pg_base, &c->pg_off,
                      &c->pg_xy, &c->pg_edge, &c->pg_list, &c->pg_work, &c->mkeys, &c->mkeys_tmp, &c->hist, &c->hist_scan,
                      &c->perm, &c->sites, &c->posf, &c->scan_scratch, &c->fill, &c->t_child, &c->t_range,
                      &c->t_parent, &c->t_leaf_parent, &c->t_flag, &c->t_box, &c->t_boxf, &c->t_mom, &c->t_ab, &c->t_nk,
                      &c->keys, &c->bboxd, &c->mass, &c->vpart, &c->mom, &c->rowcnt,
                      &c->st_col, &c->st_val, &c->rowptr, &c->col, &c->val, &c->status, &c->redo, &c->nredo,
                      &c->stat_partial, &c->stat_out, &c->info, &c->big_index, &c->big_col, &c->big_val, &c->big_work, &c->wcur, &c->w0, &c->dirn, &c->g, &c->cg_r,
                      &c->cg_z, &c->cg_p, &c->cg_q, &c->cg_dinv, &c->cg_scal, &c->cg_part,
                      &c->ms_x, &c->ms_y, &c->ms_nu, &c->ms_w, &c->tune_w};
    for (DevBuf* b : bufs) b->release();
    for (AmgBuf& l : c->amg.lev) {
        DevBuf* lb[] = {&l.rp, &l.ci, &l.va, &l.dinv, &l.b, &l.xp, &l.y, &l.agg, &l.mp, &l.mem};
        for (DevBuf* b : lb) b->release();
    }
    DevBuf* ab[] = {&c->amg.ys, &c->amg.r1, &c->amg.xs, &c->amg.inv, &c->amg.cnt, &c->amg.rp0, &c->amg.ci0, &c->amg.va0, &c->amg.sp, &c->amg.eci, &c->amg.eva,
                    &c->amg.flag, &c->amg.cinv, &c->amg.mate, &c->amg.best, &c->amg.claim, &c->amg.mflag,
                    &c->amg.mid, &c->amg.join, &c->amg.agg1, &c->amg.agg2, &c->amg.mp1, &c->amg.mem1,
                    &c->amg.mfill, &c->amg.rp1, &c->amg.ci1, &c->amg.va1, &c->amg.dinv1, &c->amg.part,
                    &c->amg.counts};
    for (DevBuf* b : ab) b->release();
    if (c->sync_event) cudaEventDestroy(c->sync_event);
    if (c->pev[0]) cudaEventDestroy(c->pev[0]);
    if (c->pev[1]) cudaEventDestroy(c->pev[1]);
    if (c->hstat) cudaFreeHost(c->hstat);
    if (c->hinfo) cudaFreeHost(c->hinfo);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

ma_status ma_ctx_set_stream(ma_ctx* c, void* stream)
{
    if (!c) return MA_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
    return MA_OK;
}

const char* ma_ctx_last_error(const ma_ctx* c) { return c ? c->last_error.c_str() : ""; }

int64_t ma_ctx_launch_count(const ma_ctx* c) { return c ? c->launches : 0; }

ma_status ma_ctx_profile(ma_ctx* c, int enable)
{
    if (!c) return MA_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (enable) {
        if (!c->pev[0]) {
            if (cudaEventCreate(&c->pev[0]) != cudaSuccess || cudaEventCreate(&c->pev[1]) != cudaSuccess)
                return MA_ERR_CUDA;
        }
        c->profile = ma_profile{};
    }
    c->prof = enable != 0;
    return MA_OK;
}

ma_status ma_ctx_profile_read(const ma_ctx* c, ma_profile* out)
{
    if (!c || !out) return MA_ERR_INVALID_ARGUMENT;
    *out = c->profile;
    return MA_OK;
}

// the linear interpolant of grid values integrates to area * mean of the three
// vertex values on each of the two triangles of a square
static double grid_total_mass(const std::vector<double>& gx, const std::vector<double>& gy, const double* values)
{
    const int nx = (int)gx.size(), ny = (int)gy.size();
    double tot = 0;
    for (int j = 0; j + 1 < ny; j++) {
        for (int i = 0; i + 1 < nx; i++) {
            double a = (gx[i + 1] - gx[i]) * (gy[j + 1] - gy[j]) / 2.0;
            double v00 = values[j * nx + i], v10 = values[j * nx + i + 1];
            double v01 = values[(j + 1) * nx + i], v11 = values[(j + 1) * nx + i + 1];
            tot += a * (v00 + v10 + v11) / 3.0 + a * (v00 + v11 + v01) / 3.0;
        }
    }
    return tot;
}

// per-triangle linear function (value at the first corner, gradient) of the
// vertex values, Linear_function of functions.hpp:55-80; returns the total mass
static double tri_linear(const std::vector<double>& vx, const std::vector<double>& vy, const std::vector<int>& t,
                         const double* values, std::vector<double>& lin)
{
    const size_t nt = t.size() / 3;
    lin.assign(3 * nt, 0.0);
    double tot = 0;
    for (size_t f = 0; f < nt; f++) {
        const int a = t[3 * f], b = t[3 * f + 1], d = t[3 * f + 2];
        const double e1x = vx[b] - vx[a], e1y = vy[b] - vy[a], e2x = vx[d] - vx[a], e2y = vy[d] - vy[a];
        const double det = e1x * e2y - e1y * e2x;
        const double f1 = values[b] - values[a], f2 = values[d] - values[a];
        lin[3 * f] = values[a];
        lin[3 * f + 1] = (f1 * e2y - f2 * e1y) / det;
        lin[3 * f + 2] = (e1x * f2 - e2x * f1) / det;
        tot += det / 2.0 * (values[a] + values[b] + values[d]) / 3.0;
    }
    return tot;
}

ma_status ma_mesh_set_values(ma_ctx* c, ma_mesh* m, const double* values, ma_mem mem)
{
    if (!c || !m || !values || m->ctx != c) return MA_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    const size_t nv = m->kind == 0 ? (size_t)m->nx * m->ny : (size_t)m->nv;
    std::vector<double> v(nv);
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    MA_CUDA(c, cudaMemcpy(v.data(), values, sizeof(double) * nv,
                          mem == MA_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
    if (m->kind == 0) {
        m->total_mass = grid_total_mass(m->hgx, m->hgy, v.data());
        MA_CUDA(c, cudaMemcpy(m->val.p, v.data(), sizeof(double) * nv, cudaMemcpyHostToDevice));
    } else {
        std::vector<double> lin;
        m->total_mass = tri_linear(m->hvx, m->hvy, m->htri, v.data(), lin);
        MA_CUDA(c, cudaMemcpy(m->lin.p, lin.data(), sizeof(double) * lin.size(), cudaMemcpyHostToDevice));
    }
    return MA_OK;
}

ma_status ma_mesh_create_grid(ma_ctx* c, int nx, int ny, const double* gx, const double* gy, const double* values,
                              ma_mesh** out)
{
    if (!c || !out || !gx || !gy || !values || nx < 2 || ny < 2) return MA_ERR_INVALID_ARGUMENT;
    for (int i = 0; i + 1 < nx; i++)
        if (!(gx[i + 1] > gx[i])) return fail(c, MA_ERR_INVALID_ARGUMENT, "gx must increase strictly");
    for (int j = 0; j + 1 < ny; j++)
        if (!(gy[j + 1] > gy[j])) return fail(c, MA_ERR_INVALID_ARGUMENT, "gy must increase strictly");
    cudaSetDevice(c->device);
    ma_mesh* m = new ma_mesh();
    m->ctx = c;
    m->kind = 0;
    m->nx = nx;
    m->ny = ny;
    m->X0 = gx[0];
    m->X1 = gx[nx - 1];
    m->Y0 = gy[0];
    m->Y1 = gy[ny - 1];
    std::vector<double> ihx(nx), ihy(ny);
    for (int i = 0; i + 1 < nx; i++) ihx[i] = 1.0 / (gx[i + 1] - gx[i]);
    for (int j = 0; j + 1 < ny; j++) ihy[j] = 1.0 / (gy[j + 1] - gy[j]);
    ihx[nx - 1] = 0;
    ihy[ny - 1] = 0;
    m->hgx.assign(gx, gx + nx);
    m->hgy.assign(gy, gy + ny);
    m->total_mass = grid_total_mass(m->hgx, m->hgy, values);
    cudaError_t e = cudaSuccess;
    if ((e = m->gx.ensure(sizeof(double) * nx)) != cudaSuccess ||
        (e = m->gy.ensure(sizeof(double) * ny)) != cudaSuccess ||
        (e = m->val.ensure(sizeof(double) * (size_t)nx * ny)) != cudaSuccess ||
        (e = m->ihx.ensure(sizeof(double) * nx)) != cudaSuccess ||
        (e = m->ihy.ensure(sizeof(double) * ny)) != cudaSuccess) {
        ma_mesh_destroy(m);
        return cuda_fail(c, e, "mesh allocation");
    }
    cudaMemcpy(m->gx.p, gx, sizeof(double) * nx, cudaMemcpyHostToDevice);
    cudaMemcpy(m->gy.p, gy, sizeof(double) * ny, cudaMemcpyHostToDevice);
    cudaMemcpy(m->val.p, values, sizeof(double) * (size_t)nx * ny, cudaMemcpyHostToDevice);
    cudaMemcpy(m->ihx.p, ihx.data(), sizeof(double) * nx, cudaMemcpyHostToDevice);
    e = cudaMemcpy(m->ihy.p, ihy.data(), sizeof(double) * ny, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        ma_mesh_destroy(m);
        return cuda_fail(c, e, "mesh upload");
    }
    *out = m;
    return MA_OK;
}

ma_status ma_mesh_create_image(ma_ctx* c, int width, int height, const double* pixels, ma_mesh** out)
{
    // image_to_pl_function (functions.hpp:82-120): an width x height grid of [-1, 1]^2,
    // vertex (i, j) at (-1 + 2 i / (width - 1), -1 + 2 j / (height - 1)) carrying
    // image(i, height - 1 - j) / 255 + 1e-3 (image rows top first)
    if (!c || !out || !pixels || width < 2 || height < 2) return MA_ERR_INVALID_ARGUMENT;
    std::vector<double> gx(width), gy(height), v((size_t)width * height);
    for (int i = 0; i < width; i++) gx[i] = -1.0 + i * (2.0 / (double)(width - 1));
    for (int j = 0; j < height; j++) gy[j] = -1.0 + j * (2.0 / (double)(height - 1));
    gx[width - 1] = 1.0;
    gy[height - 1] = 1.0;
    for (int j = 0; j < height; j++)
        for (int i = 0; i < width; i++)
            v[(size_t)j * width + i] = pixels[(size_t)(height - 1 - j) * width + i] / 255.0 + 1e-3;
    return ma_mesh_create_grid(c, width, height, gx.data(), gy.data(), v.data(), out);
}

ma_status ma_mesh_create_triangles(ma_ctx* c, int nv, const double* vx, const double* vy, const double* values,
                                   int nt, const int32_t* tri, ma_mesh** out)
{
    if (!c || !out || !vx || !vy || !values || !tri || nv < 3 || nt < 1) return MA_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    std::vector<int> t(tri, tri + 3 * (size_t)nt);
    std::vector<double> lin(3 * (size_t)nt);
    double X0 = vx[0], X1 = vx[0], Y0 = vy[0], Y1 = vy[0];
    for (int i = 0; i < nv; i++) {
        X0 = std::min(X0, vx[i]);
        X1 = std::max(X1, vx[i]);
        Y0 = std::min(Y0, vy[i]);
        Y1 = std::max(Y1, vy[i]);
    }
    double tot = 0;
    for (int f = 0; f < nt; f++) {
        int a = t[3 * f], b = t[3 * f + 1], d = t[3 * f + 2];
        if (a < 0 || b < 0 || d < 0 || a >= nv || b >= nv || d >= nv)
            return fail(c, MA_ERR_INVALID_ARGUMENT, "triangle index out of range");
        double e1x = vx[b] - vx[a], e1y = vy[b] - vy[a], e2x = vx[d] - vx[a], e2y = vy[d] - vy[a];
        double det = e1x * e2y - e1y * e2x;
        if (det == 0) return fail(c, MA_ERR_INVALID_ARGUMENT, "degenerate triangle");
        if (det < 0) {
            // counter-clockwise orientation, as the incremental builder's reorient_faces
            std::swap(t[3 * f + 1], t[3 * f + 2]);
            std::swap(b, d);
            std::swap(e1x, e2x);
            std::swap(e1y, e2y);
            det = -det;
        }
        double f1 = values[b] - values[a], f2 = values[d] - values[a];
        lin[3 * f] = values[a];
        lin[3 * f + 1] = (f1 * e2y - f2 * e1y) / det;
        lin[3 * f + 2] = (e1x * f2 - e2x * f1) / det;
        tot += det / 2.0 * (values[a] + values[b] + values[d]) / 3.0;
    }
    ma_mesh* m = new ma_mesh();
    m->ctx = c;
    m->kind = 1;
    m->nv = nv;
    m->nt = nt;
    m->X0 = X0;
    m->X1 = X1;
    m->Y0 = Y0;
    m->Y1 = Y1;
    m->total_mass = tot;
    m->hvx.assign(vx, vx + nv);
    m->hvy.assign(vy, vy + nv);
    m->htri = t;
    // bins: about two triangles per bin
    double W = std::max(X1 - X0, 1e-300), H = std::max(Y1 - Y0, 1e-300);
    double target = std::max(1.0, nt / 2.0);
    int bnx = std::max(1, (int)std::floor(std::sqrt(target * W / H)));
    int bny = std::max(1, (int)std::floor(target / bnx));
    bnx = std::min(bnx, 8192);
    bny = std::min(bny, 8192);
    m->bnx = bnx;
    m->bny = bny;
    m->bx0 = X0;
    m->by0 = Y0;
    m->bcw = W * (1 + 1e-9) / bnx;
    m->bch = H * (1 + 1e-9) / bny;
    std::vector<int4> tb(nt);
    std::vector<int> cnt((size_t)bnx * bny + 1, 0);
    auto clampb = [](int v, int n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); };
    for (int f = 0; f < nt; f++) {
        double tx0 = std::min({vx[t[3 * f]], vx[t[3 * f + 1]], vx[t[3 * f + 2]]});
        double tx1 = std::max({vx[t[3 * f]], vx[t[3 * f + 1]], vx[t[3 * f + 2]]});
        double ty0 = std::min({vy[t[3 * f]], vy[t[3 * f + 1]], vy[t[3 * f + 2]]});
        double ty1 = std::max({vy[t[3 * f]], vy[t[3 * f + 1]], vy[t[3 * f + 2]]});
        int4 r;
        r.x = clampb((int)std::floor((tx0 - m->bx0) / m->bcw) - 1, bnx);
        r.y = clampb((int)std::floor((ty0 - m->by0) / m->bch) - 1, bny);
        r.z = clampb((int)std::floor((tx1 - m->bx0) / m->bcw) + 1, bnx);
        r.w = clampb((int)std::floor((ty1 - m->by0) / m->bch) + 1, bny);
        tb[f] = r;
        for (int by = r.y; by <= r.w; by++)
            for (int bx = r.x; bx <= r.z; bx++) cnt[(size_t)by * bnx + bx + 1]++;
    }
    for (size_t b = 0; b < (size_t)bnx * bny; b++) cnt[b + 1] += cnt[b];
    std::vector<int> fillp(cnt.begin(), cnt.end() - 1), bt(cnt.back());
    for (int f = 0; f < nt; f++) {
        int4 r = tb[f];
        for (int by = r.y; by <= r.w; by++)
            for (int bx = r.x; bx <= r.z; bx++) bt[fillp[(size_t)by * bnx + bx]++] = f;
    }
    cudaError_t e = cudaSuccess;
    if ((e = m->vx.ensure(sizeof(double) * nv)) != cudaSuccess ||
        (e = m->vy.ensure(sizeof(double) * nv)) != cudaSuccess ||
        (e = m->tri.ensure(sizeof(int) * 3 * (size_t)nt)) != cudaSuccess ||
        (e = m->lin.ensure(sizeof(double) * 3 * (size_t)nt)) != cudaSuccess ||
        (e = m->tbin.ensure(sizeof(int4) * (size_t)nt)) != cudaSuccess ||
        (e = m->bin_start.ensure(sizeof(int) * cnt.size())) != cudaSuccess ||
        (e = m->bin_tri.ensure(sizeof(int) * (bt.size() + 1))) != cudaSuccess) {
        ma_mesh_destroy(m);
        return cuda_fail(c, e, "mesh allocation");
    }
    cudaMemcpy(m->vx.p, vx, sizeof(double) * nv, cudaMemcpyHostToDevice);
    cudaMemcpy(m->vy.p, vy, sizeof(double) * nv, cudaMemcpyHostToDevice);
    cudaMemcpy(m->tri.p, t.data(), sizeof(int) * 3 * (size_t)nt, cudaMemcpyHostToDevice);
    cudaMemcpy(m->lin.p, lin.data(), sizeof(double) * 3 * (size_t)nt, cudaMemcpyHostToDevice);
    cudaMemcpy(m->tbin.p, tb.data(), sizeof(int4) * (size_t)nt, cudaMemcpyHostToDevice);
    cudaMemcpy(m->bin_start.p, cnt.data(), sizeof(int) * cnt.size(), cudaMemcpyHostToDevice);
    e = cudaMemcpy(m->bin_tri.p, bt.data(), sizeof(int) * bt.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        ma_mesh_destroy(m);
        return cuda_fail(c, e, "mesh upload");
    }
    *out = m;
    return MA_OK;
}

void ma_mesh_destroy(ma_mesh* m)
{
    if (!m) return;
    if (m->ctx) cudaSetDevice(m->ctx->device);
    DevBuf* bufs[] = {&m->gx, &m->gy, &m->val, &m->ihx, &m->ihy, &m->vx, &m->vy, &m->tri, &m->lin,
                      &m->tbin, &m->bin_start, &m->bin_tri};
    for (DevBuf* b : bufs) b->release();
    delete m;
}

ma_status ma_mesh_total_mass(const ma_mesh* m, double* out)
{
    if (!m || !out) return MA_ERR_INVALID_ARGUMENT;
    *out = m->total_mass;
    return MA_OK;
}

static ma_status copy_out(ma_ctx* c, double* dst, const double* src, size_t count, ma_mem mem)
{
    if (!dst) return MA_OK;
    MA_CUDA(c, cudaMemcpyAsync(dst, src, sizeof(double) * count,
                               mem == MA_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
    return MA_OK;
}

ma_status ma_kantorovich(ma_ctx* c, const ma_mesh* m, int64_t n, const double* x, const double* y, const double* w,
                         ma_mem mem, ma_precision prec, double* value, double* g, int64_t* nnz)
{
    if (!c || !m || !x || !y || !w || n < 1 || n > (int64_t)1 << 30) return MA_ERR_INVALID_ARGUMENT;
    if (prec != MA_FP64 && prec != MA_MIXED) return MA_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    const double *dx, *dy, *dw;
    ma_status st;
    if ((st = stage_in(c, c->hx, x, n, mem, &dx)) != MA_OK) return st;
    if ((st = stage_in(c, c->hy, y, n, mem, &dy)) != MA_OK) return st;
    if ((st = stage_in(c, c->hw, w, n, mem, &dw)) != MA_OK) return st;
    if ((st = build_site_index(c, m, (int)n, dx, dy, dw)) != MA_OK) return st;
    EvalFlags f;
    f.hessian = true;
    f.mixed = prec == MA_MIXED;
    if ((st = run_eval(c, m, (int)n, dw, f)) != MA_OK) return st;
    if ((st = copy_out(c, g, c->mass.as<double>(), (size_t)n, mem)) != MA_OK) return st;
    MA_CUDA(c, cudaMemcpyAsync(c->hstat, c->stat_out.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    if (value) *value = c->hstat[0];
    if (nnz) *nnz = c->nnz;
    return MA_OK;
}

ma_status ma_kantorovich_vjp(ma_ctx* c, const ma_mesh* m, int64_t n, const double* x, const double* y,
                             const double* w, ma_mem mem, ma_precision prec, double cot_value, const double* cot_mass,
                             const double* cot_first, double* grad_x, double* grad_y, double* grad_w,
                             double* grad_rho)
{
    if (!c || !m || !x || !y || !w || !grad_x || !grad_y || !grad_w || n < 1 || n > (int64_t)1 << 30)
        return MA_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    const double *dx, *dy, *dw, *dcm = nullptr, *dcf = nullptr;
    ma_status st;
    if ((st = stage_in(c, c->hx, x, n, mem, &dx)) != MA_OK) return st;
    if ((st = stage_in(c, c->hy, y, n, mem, &dy)) != MA_OK) return st;
    if ((st = stage_in(c, c->hw, w, n, mem, &dw)) != MA_OK) return st;
    if (cot_mass && (st = stage_in(c, c->vjp_cm, cot_mass, n, mem, &dcm)) != MA_OK) return st;
    if (cot_first && (st = stage_in(c, c->vjp_cf, cot_first, 2 * n, mem, &dcf)) != MA_OK) return st;
    const int64_t nv = m->kind == 0 ? (int64_t)m->nx * m->ny : (int64_t)m->nv;
    VjpArgs v;
    v.cot_value = cot_value;
    v.cot_mass = dcm;
    v.cot_first = dcf;
    if (mem == MA_MEM_DEVICE) {
        v.grad_x = grad_x;
        v.grad_y = grad_y;
        v.grad_w = grad_w;
        v.grad_rho = grad_rho;
    } else {
        MA_CUDA(c, c->vjp_gx.ensure(sizeof(double) * (size_t)n));
        MA_CUDA(c, c->vjp_gy.ensure(sizeof(double) * (size_t)n));
        MA_CUDA(c, c->vjp_gw.ensure(sizeof(double) * (size_t)n));
        v.grad_x = c->vjp_gx.as<double>();
        v.grad_y = c->vjp_gy.as<double>();
        v.grad_w = c->vjp_gw.as<double>();
        if (grad_rho) {
            MA_CUDA(c, c->vjp_gr.ensure(sizeof(double) * (size_t)nv));
            v.grad_rho = c->vjp_gr.as<double>();
        }
    }
    if (v.grad_rho) MA_CUDA(c, cudaMemsetAsync(v.grad_rho, 0, sizeof(double) * (size_t)nv, c->stream));
    if ((st = build_site_index(c, m, (int)n, dx, dy, dw)) != MA_OK) return st;
    EvalFlags f;
    f.hessian = false;
    f.vjp = &v;
    f.mixed = prec == MA_MIXED;
    if ((st = run_eval(c, m, (int)n, dw, f)) != MA_OK) return st;
    if (mem == MA_MEM_HOST) {
        if ((st = copy_out(c, grad_x, v.grad_x, (size_t)n, mem)) != MA_OK) return st;
        if ((st = copy_out(c, grad_y, v.grad_y, (size_t)n, mem)) != MA_OK) return st;
        if ((st = copy_out(c, grad_w, v.grad_w, (size_t)n, mem)) != MA_OK) return st;
        if (grad_rho && (st = copy_out(c, grad_rho, v.grad_rho, (size_t)nv, mem)) != MA_OK) return st;
    }
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    return MA_OK;
}

ma_status ma_pieces(ma_ctx* c, const ma_mesh* m, int64_t n, const double* x, const double* y, const double* w,
                    ma_mem mem, int64_t* npieces, int64_t* nverts)
{
    if (!c || !m || !x || !y || !w || n < 1 || n > (int64_t)1 << 30) return MA_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    const double *dx, *dy, *dw;
    ma_status st;
    if ((st = stage_in(c, c->hx, x, n, mem, &dx)) != MA_OK) return st;
    if ((st = stage_in(c, c->hy, y, n, mem, &dy)) != MA_OK) return st;
    if ((st = stage_in(c, c->hw, w, n, mem, &dw)) != MA_OK) return st;
    if ((st = build_site_index(c, m, (int)n, dx, dy, dw)) != MA_OK) return st;
    EvalFlags f;
    f.hessian = false;
    f.pieces = true;
    if ((st = run_eval(c, m, (int)n, dw, f)) != MA_OK) return st;
    if (npieces) *npieces = c->npieces;
    if (nverts) *nverts = c->npverts;
    return MA_OK;
}

ma_status ma_pieces_copy(ma_ctx* c, int32_t* site, int32_t* tri, int64_t* off, double* xy, int32_t* edge, ma_mem mem)
{
    if (!c) return MA_ERR_INVALID_ARGUMENT;
    if (!c->have_pieces) return fail(c, MA_ERR_INVALID_ARGUMENT, "no pieces have been computed");
    cudaSetDevice(c->device);
    cudaMemcpyKind k = mem == MA_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t np = (size_t)c->npieces, nv = (size_t)c->npverts;
    if (site && np) MA_CUDA(c, cudaMemcpyAsync(site, c->pc_site.p, sizeof(int) * np, k, c->stream));
    if (tri && np) MA_CUDA(c, cudaMemcpyAsync(tri, c->pc_tri.p, sizeof(int) * np, k, c->stream));
    if (off) MA_CUDA(c, cudaMemcpyAsync(off, c->pc_off.p, sizeof(int64_t) * (np + 1), k, c->stream));
    if (xy && nv) MA_CUDA(c, cudaMemcpyAsync(xy, c->pc_xy.p, sizeof(double) * 2 * nv, k, c->stream));
    if (edge && nv) MA_CUDA(c, cudaMemcpyAsync(edge, c->pc_edge.p, sizeof(int) * nv, k, c->stream));
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    return MA_OK;
}

ma_status ma_hessian_copy(ma_ctx* c, int32_t* rowptr, int32_t* col, double* val, ma_mem mem)
{
    if (!c) return MA_ERR_INVALID_ARGUMENT;
    if (!c->have_h) return fail(c, MA_ERR_INVALID_ARGUMENT, "no Hessian has been computed");
    cudaSetDevice(c->device);
    cudaMemcpyKind k = mem == MA_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (rowptr) MA_CUDA(c, cudaMemcpyAsync(rowptr, c->rowptr.p, sizeof(int) * ((size_t)c->n + 1), k, c->stream));
    if (col) MA_CUDA(c, cudaMemcpyAsync(col, c->col.p, sizeof(int) * (size_t)c->nnz, k, c->stream));
    if (val) MA_CUDA(c, cudaMemcpyAsync(val, c->val.p, sizeof(double) * (size_t)c->nnz, k, c->stream));
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    return MA_OK;
}

static ma_status moments_impl(ma_ctx* c, const ma_mesh* m, int64_t n, const double* x, const double* y,
                              const double* w, ma_mem mem, int order)
{
    if (!c || !m || !x || !y || !w || n < 1 || n > (int64_t)1 << 30) return MA_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    const double *dx, *dy, *dw;
    ma_status st;
    if ((st = stage_in(c, c->hx, x, n, mem, &dx)) != MA_OK) return st;
    if ((st = stage_in(c, c->hy, y, n, mem, &dy)) != MA_OK) return st;
    if ((st = stage_in(c, c->hw, w, n, mem, &dw)) != MA_OK) return st;
    if ((st = build_site_index(c, m, (int)n, dx, dy, dw)) != MA_OK) return st;
    EvalFlags f;
    f.hessian = false;
    f.moments = order;
    return run_eval(c, m, (int)n, dw, f);
}

ma_status ma_moments(ma_ctx* c, const ma_mesh* m, int64_t n, const double* x, const double* y, const double* w,
                     ma_mem mem, double* mass, double* first, double* second)
{
    ma_status st = moments_impl(c, m, n, x, y, w, mem, second ? 2 : 1);
    if (st != MA_OK) return st;
    std::vector<double> mo(6 * (size_t)n);
    MA_CUDA(c, cudaMemcpyAsync(mo.data(), c->mom.p, sizeof(double) * 6 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<double> ms(n), f1(2 * (size_t)n), f2(3 * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        ms[i] = mo[6 * i];
        f1[2 * i] = mo[6 * i + 1];
        f1[2 * i + 1] = mo[6 * i + 2];
        f2[3 * i] = mo[6 * i + 3];
        f2[3 * i + 1] = mo[6 * i + 4];
        f2[3 * i + 2] = mo[6 * i + 5];
    }
    cudaMemcpyKind k = mem == MA_MEM_DEVICE ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
    if (mass) MA_CUDA(c, cudaMemcpy(mass, ms.data(), sizeof(double) * n, k));
    if (first) MA_CUDA(c, cudaMemcpy(first, f1.data(), sizeof(double) * 2 * n, k));
    if (second) MA_CUDA(c, cudaMemcpy(second, f2.data(), sizeof(double) * 3 * n, k));
    return MA_OK;
}

ma_status ma_lloyd(ma_ctx* c, const ma_mesh* m, int64_t n, const double* x, const double* y, const double* w,
                   ma_mem mem, double* mass, double* centroids)
{
    ma_status st = moments_impl(c, m, n, x, y, w, mem, 1);
    if (st != MA_OK) return st;
    std::vector<double> mo(6 * (size_t)n);
    MA_CUDA(c, cudaMemcpyAsync(mo.data(), c->mom.p, sizeof(double) * 6 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<double> ms(n), ce(2 * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        ms[i] = mo[6 * i];
        ce[2 * i] = mo[6 * i + 1] / mo[6 * i];
        ce[2 * i + 1] = mo[6 * i + 2] / mo[6 * i];
    }
    cudaMemcpyKind k = mem == MA_MEM_DEVICE ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
    if (mass) MA_CUDA(c, cudaMemcpy(mass, ms.data(), sizeof(double) * n, k));
    if (centroids) MA_CUDA(c, cudaMemcpy(centroids, ce.data(), sizeof(double) * 2 * n, k));
    return MA_OK;
}

}  // extern "C"
