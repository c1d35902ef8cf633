// ma_stage.cuh -- the cell stage: one Laguerre cell, clipped from a fixed polygon by a
// branch-and-bound walk over the site tree.  Shared by the evaluation's kernels
// (ma_cells.cu, where the fixed polygon is the mesh's bounding box) and by the
// polygon intersection (ma_polygon.cu, where it is the caller's polygon).
#pragma once

#include "ma_internal.h"

namespace ma {

// ---------------------------------------------------------------------------
// workspaces
// ---------------------------------------------------------------------------
template <int CAP>
struct Work {  // the whole cell in one thread (large-capacity pass)
    Slot slots[CAP];
    Poly<CAP> PA, PB;
    double hv[CAP];
    Nb64 nb[CAP];
    int map[CAP];
    int cols[CAP];
    double vals[CAP];
};

template <int CAP>
struct Work1 {  // stage 1: cell only
    Slot slots[CAP];
    Poly<CAP> PA, PB;
    int map[CAP];
};

template <int CAP>
__device__ __forceinline__ void compact_slots(Poly<CAP>& P, Slot* slots, int* map, int& ns)
{
    Bits<CAP> used;
    used.clear();
    for (int e = 0; e < P.n; e++)
        if (P.lab[e] >= 0) used.set(P.lab[e]);
    int m = 0;
    for (int s = 0; s < ns; s++) {
        if (used.get(s)) {
            map[s] = m;
            if (m != s) slots[m] = slots[s];
            m++;
        } else {
            map[s] = -1;
        }
    }
    for (int e = 0; e < P.n; e++)
        if (P.lab[e] >= 0) P.lab[e] = map[P.lab[e]];
    ns = m;
}

// Can no site of internal node nd cut polygon P?  With phi_j >= alpha + beta.x_j
// over the node and the node's box [c - h, c + h]:
//   pi_ij(p) / 2 = p.(x_j - x_i) + phi_i - phi_j
//              <= (p - beta).(c - x_i) + |p_x - beta_x| h_x + |p_y - beta_y| h_y - K,
//   K = alpha + beta.x_i - phi_i,
// convex in p, so it suffices that it is negative at every vertex of P.  Everything is
// FP32 with bounded rounding.  K comes from the node's expansion about its box centre c
// (nk, written with the bounds): with d = x_i - c and g = beta - c,
//   K = A + g.d - |d|^2 / 2 + w_i / 2,   A = alpha + beta.c - |c|^2 / 2 (rounded down),
// whose terms are all small where the test is close; x_i - beta = d - g.  The box enters
// relative to the FP32 site position, with the conversion errors absorbed into a wider
// box.
__device__ __forceinline__ bool node_harmless_v(const float* pux, const float* puy, const float* pur, int pn,
                                                float ox, float oy, float owh, float oxa, const float4 bf,
                                                const float4 nk)
{
    if (!(nk.x > -INFINITY)) return false;
    const float ccx = 0.5f * (bf.x + bf.z), ccy = 0.5f * (bf.y + bf.w);
    const float dx = ox - ccx, dy = oy - ccy;
    const float gdx = nk.y * dx, gdy = nk.z * dy, dd = 0.5f * (dx * dx + dy * dy);
    const float fK = nk.x + (gdx + gdy) - dd + owh;
    const float sg = fabsf(nk.y) + fabsf(nk.z), sd = fabsf(dx) + fabsf(dy);
    const float fke = 1e-6f * (fabsf(nk.x) + fabsf(gdx) + fabsf(gdy) + dd + fabsf(owh)) +
                      1.2e-7f * (sg + sd) * (oxa + sd) + 1e-37f;
    const float fex = dx - nk.y, fey = dy - nk.z;
    const float cx = -dx, cy = -dy;
    float hx = 0.5f * (bf.z - bf.x), hy = 0.5f * (bf.w - bf.y);
    float wx = 1.2e-7f * (fabsf(bf.x) + fabsf(bf.z) + 2.0f * fabsf(ox)) + 1e-37f;
    float wy = 1.2e-7f * (fabsf(bf.y) + fabsf(bf.w) + 2.0f * fabsf(oy)) + 1e-37f;
    hx = hx * 1.000001f + wx;
    hy = hy * 1.000001f + wy;
    const float L = fabsf(cx) + fabsf(cy) + hx + hy;
    const float e0 = 1.2e-7f * (fabsf(fex) + fabsf(fey) + sd + sg + 2.0f * oxa);
    for (int v = 0; v < pn; v++) {
        float qx = fex + pux[v], qy = fey + puy[v];
        float T = qx * cx + qy * cy + fabsf(qx) * hx + fabsf(qy) * hy - fK;
        float S = fabsf(qx * cx) + fabsf(qy * cy) + fabsf(qx) * hx + fabsf(qy) * hy + fabsf(fK);
        float err = 1e-6f * S + (pur[v] + e0) * L * 1.0001f + fke + 1e-36f;
        if (!(T + err < 0.0f)) return false;
    }
    return true;
}

template <int CAP>
__device__ __forceinline__ bool node_harmless(const Poly<CAP>& P, float ox, float oy, float owh, float oxa,
                                              const float4 bf, const float4 nk)
{
    return node_harmless_v(P.ux, P.uy, P.ur, P.n, ox, oy, owh, oxa, bf, nk);
}

// ---------------------------------------------------------------------------
// the cell stage: branch and bound over the site tree
// ---------------------------------------------------------------------------
constexpr int kCapSmall = 48;
constexpr int kSeedCap = kCapSmall;  // neighbour-list stride between the stages

struct CellOut {
    bool overflow;
    bool empty;
    bool aborted;  // another cell was found empty and the evaluation is abandoned
    uint32_t st;
    int ns;  // neighbour slots after compaction
    int popped, tested, pruned, visited, cuts;
};

// the mesh's bounding box as the fixed polygon of a cell
__device__ __forceinline__ Fixed domain_box(const CellArgs& A, const Owner& o)
{
    Fixed box;
    box.n = 4;
    set_fixed(box, 0, A.X0, A.Y0, o);
    set_fixed(box, 1, A.X1, A.Y0, o);
    set_fixed(box, 2, A.X1, A.Y1, o);
    set_fixed(box, 3, A.X0, A.Y1, o);
    return box;
}

// The cell of sorted site k clipped to the fixed polygon `box` (the mesh's bounding
// box, or a caller's polygon): P starts as the fixed polygon and is clipped by every
// site the walk cannot prove harmless.
template <int CAP, bool EXACT, class FX>
__device__ CellOut cell_stage(const CellArgs& A, int k, const SiteD& S, const Owner& o, const FX& box, Slot* slots,
                              int* map, Poly<CAP>*& P, Poly<CAP>*& Q)
{
    CellOut r{false, false, false, 0u, 0, 0, 0, 0, 0, 0};
    const int gi = A.perm[k];
    P->n = box.n;
    for (int e = 0; e < box.n; e++) {
        P->lab[e] = -1 - e;
        P->ux[e] = box.ux[e];
        P->uy[e] = box.uy[e];
        P->ur[e] = box.ur[e];
    }
    if (!(isfinite(S.x) && isfinite(S.y) && isfinite(S.w))) {
        r.st |= ST_BAD_INPUT;
        r.empty = true;
        P->n = 0;
        return r;
    }
    int ns = 0;
    const SiteTree& T = A.tree;
    const float ox = (float)S.x, oy = (float)S.y;
    const float owh = (float)(0.5 * S.w), oxa = fabsf(ox) + fabsf(oy);
    constexpr int kStack = 80;
    constexpr int kBucket = 4;
    constexpr int kWindow = 8;
    int stack[kStack];
    int sp = 0;
    if (T.n >= 2) stack[sp++] = 0;
    // Seeds, clipped first so that the walk below starts from a nearly final cell:
    // the previous evaluation's neighbours (same sites, nearby weights), or else the
    // Morton-order window around the site.  The walk skips the seeds.
    int nseed = 0;
    int seeds[kSeedCap];
    if (A.prev_valid && A.nb_cnt[k] > 0 && A.nb_cnt[k] <= kSeedCap) {
        nseed = A.nb_cnt[k];
        const int* pl = A.nb_lab + (size_t)k * kSeedCap;
        for (int s = 0; s < nseed; s++) seeds[s] = pl[s];
    }
    const bool windowed = nseed == 0;
    auto is_seed = [&](int q) -> bool {
        if (windowed) return q >= k - kWindow && q <= k + kWindow;
        for (int s = 0; s < nseed; s++)
            if (seeds[s] == q) return true;
        return false;
    };
    auto visit = [&](int q) -> bool {  // clip by sorted site q; false when the cell became empty
        if (q == k) return true;
        const SiteD C = A.sites[q];
        if (C.x == S.x && C.y == S.y) {
            // coincident sites: the larger weight, then the lower index, keeps the cell
            int gj = A.perm[q];
            if (C.w > S.w || (C.w == S.w && gj < gi)) return false;
            return true;
        }
        if (ns == CAP) {
            compact_slots(*P, slots, map, ns);
            if (ns == CAP) {
                r.overflow = true;
                return true;
            }
        }
        slots[ns] = make_slot(q, C, o);
        r.visited++;
        if (clip_poly<CAP, EXACT>(*P, *Q, ns, slots, box, o, A.sites, r.st, r.overflow)) {
            if (r.overflow) return true;
            r.cuts++;
            Poly<CAP>* t = P;
            P = Q;
            Q = t;
            ns++;
            if (P->n == 0) return false;
        }
        return true;
    };
    auto dist2 = [&](int c) -> float {
        if (c < 0) {
            float2 p = T.posf[c & 0x7fffffff];
            float dx = p.x - ox, dy = p.y - oy;
            return dx * dx + dy * dy;
        }
        float4 b = T.boxf[c];
        float dx = fmaxf(fmaxf(b.x - ox, ox - b.z), 0.0f), dy = fmaxf(fmaxf(b.y - oy, oy - b.w), 0.0f);
        return dx * dx + dy * dy;
    };
    if (windowed) {
        for (int q = max(k - kWindow, 0); q <= min(k + kWindow, A.n - 1) && !r.empty && !r.overflow; q++)
            if (!visit(q)) r.empty = true;
    } else {
        for (int s = 0; s < nseed && !r.empty && !r.overflow; s++)
            if (!visit(seeds[s])) r.empty = true;
    }
    // Two phases per round, so that the lanes of a warp clip together: every lane
    // walks until it reaches sites to clip against (a leaf or a small node: the range
    // [vlo, vhi]) or its stack runs out, and the lanes that found sites then clip
    // against them side by side.  Sites are met in the same depth-first order as in a
    // single loop, so the cell and its slots do not depend on the phases.
    for (;;) {
        int vlo = 0, vhi = -1;
        while (sp > 0 && !r.empty && !r.overflow) {
            if (A.abort_flag && (r.popped & 7) == 0 && *(volatile const int*)A.abort_flag) {
                r.aborted = true;
                break;
            }
            int nd = stack[--sp];
            r.popped++;
            if (nd < 0) {
                vlo = vhi = nd & 0x7fffffff;
                break;
            }
            // everything the node may need, loaded at once (one round trip, not three)
            const int2 rg = T.range[nd];
            const int2 ch = T.child[nd];
            const float4 nbf = T.boxf[nd];
            const float4 nnk = T.nk[nd];
            bool contains = rg.x <= k && k <= rg.y;
            if (!contains) {
                r.tested++;
                if (node_harmless(*P, ox, oy, owh, oxa, nbf, nnk)) {
                    r.pruned++;
                    continue;
                }
            }
            if (rg.y - rg.x < kBucket) {
                vlo = rg.x;
                vhi = rg.y;
                break;
            }
            if (sp > kStack - 2) {
                r.overflow = true;
                break;
            }
            // nearer child on top
            if (dist2(ch.x) <= dist2(ch.y)) {
                stack[sp++] = ch.y;
                stack[sp++] = ch.x;
            } else {
                stack[sp++] = ch.x;
                stack[sp++] = ch.y;
            }
        }
        if (vlo > vhi || r.aborted) break;
        for (int q = vlo; q <= vhi && !r.empty && !r.overflow; q++)
            if (!is_seed(q) && !visit(q)) r.empty = true;
    }
    if (r.empty) {
        P->n = 0;
        if (A.abort_flag) atomicExch(A.abort_flag, 1);
    }
    if (r.aborted) return r;
    if (!r.empty && !r.overflow && P->n > 0) compact_slots(*P, slots, map, ns);
    r.ns = ns;
    return r;
}

}  // namespace ma
