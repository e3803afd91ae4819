// ccd.cu — compute_collision_free_stepsize on the device.
//
// Restates src/ipc/ipc.cpp:42-106 -> candidates.cpp:128-222 (swept-box
// broad phase, inflation 0.5*min_distance) -> candidates.cpp:252-292
// (earliest time of impact over all candidates with tmax pruning) ->
// tight_inclusion_ccd.cpp:33-336 (the TightInclusionCCD strategy: initial
// distance check, effective minimum separation, small-ToI rerun without
// minimum separation and with no-zero-ToI, conservative rescaling).
//
// The root finder restates the published inclusion-based method of
// Tight-Inclusion (Wang et al., "A Large-Scale Benchmark and an
// Inclusion-Based Algorithm for Continuous Collision Detection", ACM TOG
// 2021; library version 1.0.6 is what the reference links): the vertex-face
// / edge-edge co-planarity function F(t,u,v) is multilinear, so the box of
// its image over a parameter box is the box of its 8 corner values; boxes
// whose image misses [-eps-ms, eps+ms]^3 are discarded and the rest are
// bisected (split_dim: a parameter whose halving discards a half, else time
// unless the straddling components barely change across it, else the
// parameter across which they change most).  A box is accepted when
// every component is either inside the separation box or narrower than the
// codomain tolerance (the union of Tight-Inclusion's two acceptance tests),
// or when the box is below the domain tolerances.  Boxes are totally ordered
// (lower corner, then levels) and increase along every path of the box tree,
// so the result -- the first accepted box in that order -- does not depend
// on the walk.  Each thread walks best first with a small heap and walks the
// subtree of any box the full heap cannot take depth first; the CPU oracle
// walks best first with an unbounded heap and returns the same box.  One
// thread per candidate; this file is compiled with -fmad=false so every
// value matches the CPU oracle bit for bit.
#include <algorithm>
#include <atomic>

#include "ccd_query.cuh"
#include "profile.cuh"

namespace ipcg {

std::atomic<int> g_ccd_stats { 0 };
// testing: the box budget of the one-thread pass (0: the default)
std::atomic<long long> g_ccd_thread_budget { 0 };

namespace {

// best-first heap per thread; a box the full heap cannot take has its
// subtree walked depth first on a stack that a 3 x 60-level tree cannot
// overflow (depth + 1 entries at most)
constexpr int CCD_HEAP = 64;
constexpr int CCD_STACK = 184;
constexpr int BLOCK = 128;
// The budgeted pass runs the queries (sorted by a lower bound on their time
// of impact) with a box budget, pruned by the earliest time found so far
// (re-read as it runs); a query that does not finish within the budget is
// deferred to the hard pass, which starts it again with the then earliest
// time as its horizon and runs it to completion.
constexpr long long CCD_PASS1_BUDGET = 128;
// The seed queries (each scene's likeliest earliest impacts) run first with a
// larger budget, so that a scene's earliest time is known before the bulk of
// its queries runs.
constexpr long long CCD_SEED_BUDGET = 2048;

// Order-preserving integer keys of finite doubles: signed 64-bit comparison
// of the keys orders the values (negative zero just below positive zero),
// so minima, maxima and comparisons run on the integer pipe, which GB300
// issues 32 times faster than FP64.  The results are the same doubles.
__device__ __forceinline__ long long okey(double x)
{
    const long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double ovalue(long long k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL)); }

struct CBox {
    double lo[3];
    int8_t lvl[3];
};

__device__ __forceinline__ double width_of(int lvl) { return ldexp(1.0, -lvl); }

// Total order of boxes: lower corner (t, u, v), then levels.  Children come
// after their parent.
// Lower corners are sums of non-negative powers of two starting from +0, so
// their bit patterns order like their values: the comparison runs on the
// integer pipe.
__device__ __forceinline__ bool box_before(const CBox& a, const CBox& b)
{
    for (int d = 0; d < 3; ++d) {
        const long long x = __double_as_longlong(a.lo[d]), y = __double_as_longlong(b.lo[d]);
        if (x != y) return x < y;
    }
    for (int d = 0; d < 3; ++d)
        if (a.lvl[d] != b.lvl[d]) return a.lvl[d] < b.lvl[d];
    return false;
}

__device__ __forceinline__ double F_comp(const Query& q, int c, double t, double u, double v)
{
    double x[4];
    for (int k = 0; k < 4; ++k) {
        const double a = comp(q.s[k], c), b = comp(q.e[k], c);
        x[k] = (b - a) * t + a;
    }
    if (q.vf) {
        const double pt = (x[2] - x[1]) * u + (x[3] - x[1]) * v + x[1];
        return x[0] - pt;
    }
    const double ea = (x[1] - x[0]) * u + x[0];
    const double eb = (x[3] - x[2]) * v + x[2];
    return ea - eb;
}

__device__ void domain_tol(const Query& q, double delta, double tol[3])
{
    for (int dim = 0; dim < 3; ++dim) {
        double L = 0;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) {
                double c0[3], c1[3];
                int o = 0;
                for (int k = 0; k < 3; ++k) {
                    if (k == dim) {
                        c0[k] = 0;
                        c1[k] = 1;
                    } else {
                        c0[k] = c1[k] = (o++ == 0) ? a : b;
                    }
                }
                double m = 0;
                for (int c = 0; c < 3; ++c)
                    m = fmax(m, fabs(F_comp(q, c, c1[0], c1[1], c1[2]) - F_comp(q, c, c0[0], c0[1], c0[2])));
                L = fmax(L, m);
            }
        L *= 3;
        tol[dim] = (L == 0) ? delta : delta / L;
    }
}

// Whether halving a box across parameter d leaves a half whose corner box
// misses [-r, r], for one component with corner values f[i][j][k] at
// (t_i, u_j, v_k): the halving face's values are taken as averages of the two
// opposite corners (exact for the multilinear F up to rounding; the average
// is the same for both halves because addition commutes).  Only used to pick
// a split, and only called for components that straddle [-r, r] (a half of
// a component inside it stays inside).
__device__ __forceinline__ bool halving_excludes(const double f[2][2][2], int d, double r)
{
    const long long big = 0x7fffffffffffffffLL;
    long long lo0 = big, hi0 = -big, lo1 = big, hi1 = -big, lom = big, him = -big;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
            double f0, f1;
            if (d == 0) {
                f0 = f[0][a][b];
                f1 = f[1][a][b];
            } else if (d == 1) {
                f0 = f[a][0][b];
                f1 = f[a][1][b];
            } else {
                f0 = f[a][b][0];
                f1 = f[a][b][1];
            }
            const long long k0 = okey(f0), k1 = okey(f1), km = okey((f1 + f0) * 0.5);
            lo0 = min(lo0, k0);
            hi0 = max(hi0, k0);
            lo1 = min(lo1, k1);
            hi1 = max(hi1, k1);
            lom = min(lom, km);
            him = max(him, km);
        }
    const long long kr = okey(r), knr = okey(-r);
    return min(lo0, lom) > kr || max(hi0, him) < knr || min(lo1, lom) > kr || max(hi1, him) < knr;
}

// Returns zero_in; sets box_in, the codomain widths cw[c], whether component
// c lies inside [-eps-ms, eps+ms] (inside[c]), for the components that do
// not the largest change of component c between the two faces of the box
// across parameter d, and in excl (bit d) whether halving across d leaves a
// half that some component excludes.  The vertex positions are interpolated
// once per time (the same expression as F_comp, so the same values), and the
// test stops at the first component that excludes the box.
__device__ bool inclusion(const Query& q, const CBox& b, const double err[3], double ms, bool& box_in, double cw[3],
    double var[3][3], bool inside[3], int& excl)
{
    const double ts[2] = { b.lo[0], b.lo[0] + width_of(b.lvl[0]) };
    const double us[2] = { b.lo[1], b.lo[1] + width_of(b.lvl[1]) };
    const double vs[2] = { b.lo[2], b.lo[2] + width_of(b.lvl[2]) };
    box_in = true;
    excl = 0;
    for (int c = 0; c < 3; ++c) {
        double f[2][2][2];
        for (int i = 0; i < 2; ++i) {
            double x[4];
            for (int k = 0; k < 4; ++k) x[k] = comp(q.d[k], c) * ts[i] + comp(q.s[k], c);
            if (q.vf) {
                const double d21 = x[2] - x[1], d31 = x[3] - x[1];
                for (int j = 0; j < 2; ++j)
                    for (int k = 0; k < 2; ++k) f[i][j][k] = x[0] - (d21 * us[j] + d31 * vs[k] + x[1]);
            } else {
                const double d10 = x[1] - x[0], d32 = x[3] - x[2];
                const double ea[2] = { d10 * us[0] + x[0], d10 * us[1] + x[0] };
                const double eb[2] = { d32 * vs[0] + x[2], d32 * vs[1] + x[2] };
                for (int j = 0; j < 2; ++j)
                    for (int k = 0; k < 2; ++k) f[i][j][k] = ea[j] - eb[k];
            }
        }
        long long kmn = okey(f[0][0][0]), kmx = kmn;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    const long long kf = okey(f[i][j][k]);
                    kmn = min(kmn, kf);
                    kmx = max(kmx, kf);
                }
        const double r = err[c] + ms;
        const long long kr = okey(r), knr = okey(-r);
        if (kmn > kr || kmx < knr) return false;
        inside[c] = (kmn >= knr && kmx <= kr);
        cw[c] = ovalue(kmx) - ovalue(kmn);
        var[c][0] = var[c][1] = var[c][2] = 0;
        if (!inside[c]) {
            box_in = false;
            for (int d = 0; d < 3; ++d)
                if (!(excl >> d & 1) && halving_excludes(f, d, r)) excl |= 1 << d;
            // non-negative doubles order like their bit patterns
            long long v0 = 0, v1 = 0, v2 = 0;
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    v0 = max(v0, __double_as_longlong(fabs(f[1][j][k] - f[0][j][k])));
                    v1 = max(v1, __double_as_longlong(fabs(f[j][1][k] - f[j][0][k])));
                    v2 = max(v2, __double_as_longlong(fabs(f[j][k][1] - f[j][k][0])));
                }
            var[c][0] = __longlong_as_double(v0);
            var[c][1] = __longlong_as_double(v1);
            var[c][2] = __longlong_as_double(v2);
        }
    }
    return true;
}

// Split parameter of a box that is neither discarded nor accepted:
// (1) a parameter whose halving discards a half at once (the one across
//     which the straddling components change most, if several);
// (2) else time, if the straddling components' change across time is at
//     least 1/16 of their largest change across any parameter: boxes are
//     visited in order of their earliest time, so a time split defers its
//     later half, while a u or v split leaves two boxes with the same
//     earliest time to resolve (this keeps near-parallel edge pairs, whose
//     root set is a whole segment, from being resolved point by point);
// (3) else the parameter across which the straddling components change
//     most.  Parameters at the depth limit are not split.
__device__ int split_dim(const CBox& b, const double var[3][3], const bool inside[3], int excl)
{
    double vmax[3] = { 0, 0, 0 };
    for (int c = 0; c < 3; ++c)
        if (!inside[c])
            for (int d = 0; d < 3; ++d) vmax[d] = fmax(vmax[d], var[c][d]);
    int sd = -1;
    double best = -1;
    for (int d = 0; d < 3; ++d)
        if (b.lvl[d] < 60 && vmax[d] > best && (excl >> d & 1)) {
            best = vmax[d];
            sd = d;
        }
    if (sd >= 0) return sd;
    if (b.lvl[0] < 60 && vmax[0] * 16.0 >= fmax(vmax[0], fmax(vmax[1], vmax[2]))) return 0;
    for (int d = 0; d < 3; ++d)
        if (b.lvl[d] < 60 && vmax[d] > best) {
            best = vmax[d];
            sd = d;
        }
    return sd;
}

// Search status: no root before tmax, a root box found, or the caller's box
// budget ran out before the search finished (result unknown).
enum : int { CCD_MISS = 0, CCD_HIT = 1, CCD_UNRESOLVED = 2 };

struct Budget {
    long long limit; // <= 0: unlimited
    long long spent;
};

struct BoxHeap {
    CBox a[CCD_HEAP];
    int n;
    __device__ void push(const CBox& b)
    {
        int i = n++;
        while (i > 0) {
            const int p = (i - 1) >> 1;
            if (!box_before(b, a[p])) break;
            a[i] = a[p];
            i = p;
        }
        a[i] = b;
    }
    __device__ CBox pop()
    {
        const CBox top = a[0];
        const CBox last = a[--n];
        int i = 0;
        for (;;) {
            int c = 2 * i + 1;
            if (c >= n) break;
            if (c + 1 < n && box_before(a[c + 1], a[c])) ++c;
            if (!box_before(a[c], last)) break;
            a[i] = a[c];
            i = c;
        }
        if (n > 0) a[i] = last;
        return top;
    }
};

// One step of the search on box b: returns 0 (discarded or accepted), or 1
// with the kept children in ch[0..nch).
struct Search {
    const Query& q;
    const double* err;
    double ms, delta;
    const double* tol;
    double tmax;    // boxes starting at or after it are skipped
    CBox best;      // first accepted box so far (in box order)
    bool found;
    double out_tol;
    long long itr, cap;
    Budget& bud;
    bool capped, unresolved;

    __device__ bool skip(const CBox& b) const { return b.lo[0] >= tmax || (found && !box_before(b, best)); }

    __device__ int step(const CBox& b, CBox ch[2], int& nch)
    {
        nch = 0;
        ++itr;
        if (++bud.spent > bud.limit && bud.limit > 0) {
            unresolved = true;
            return 0;
        }
        bool box_in, inside[3];
        double cw[3], var[3][3];
        int excl;
        if (!inclusion(q, b, err, ms, box_in, cw, var, inside, excl)) return 0;
        const double w[3] = { width_of(b.lvl[0]), width_of(b.lvl[1]), width_of(b.lvl[2]) };
        const bool small_co = (inside[0] || cw[0] <= delta) && (inside[1] || cw[1] <= delta)
            && (inside[2] || cw[2] <= delta);
        const bool small_dom = w[0] <= tol[0] && w[1] <= tol[1] && w[2] <= tol[2];
        const bool too_deep = b.lvl[0] >= 60 && b.lvl[1] >= 60 && b.lvl[2] >= 60;
        if (small_co || box_in || small_dom || too_deep) {
            best = b;
            found = true;
            out_tol = fmax(cw[0], fmax(cw[1], cw[2]));
            return 0;
        }
        if (itr > cap) {
            capped = true;
            out_tol = fmax(cw[0], fmax(cw[1], cw[2]));
            return 0;
        }
        const int sd = split_dim(b, var, inside, excl);
        CBox lo = b, hi = b;
        lo.lvl[sd] = hi.lvl[sd] = (int8_t)(b.lvl[sd] + 1);
        hi.lo[sd] = b.lo[sd] + width_of(lo.lvl[sd]);
        // VF: drop halves entirely outside u + v <= 1
        if (!(q.vf && sd != 0 && hi.lo[1] + hi.lo[2] > 1.0)) ch[nch++] = hi;
        if (!(q.vf && sd != 0 && lo.lo[1] + lo.lo[2] > 1.0)) ch[nch++] = lo;
        return 1;
    }
};

// `shared_best` (may be null) is the earliest time of impact found so far by
// any candidate; boxes starting at or after it cannot lower the final
// minimum, so it is re-read every 64 boxes to prune.
__device__ int root_finder(const Query& q, const double err[3], double ms, const double tol[3], double delta,
    double tmax, long long max_itr, double& toi, double& out_tol, const unsigned long long* shared_best, Budget& bud)
{
    // "unlimited" iterations are capped so that no query can run away; the
    // cap falls back to the conservative earliest unresolved time
    Search S { q, err, ms, delta, tol, tmax, CBox {}, false, 0.0, 0, max_itr > 0 ? max_itr : 100000000LL, bud, false,
        false };
    BoxHeap H;
    H.n = 0;
    CBox root;
    root.lo[0] = root.lo[1] = root.lo[2] = 0;
    root.lvl[0] = root.lvl[1] = root.lvl[2] = 0;
    H.push(root);
    CBox st[CCD_STACK];
    double capped_t = tmax;
    while (H.n > 0 && !S.capped && !S.unresolved) {
        if (shared_best && (S.itr & 63) == 0)
            S.tmax = fmin(S.tmax, __longlong_as_double((long long)*(volatile const unsigned long long*)shared_best));
        const CBox b = H.pop();
        if (S.skip(b)) break; // the heap's first box: every other one comes later
        CBox ch[2];
        int nch;
        if (!S.step(b, ch, nch)) {
            if (S.capped) capped_t = b.lo[0];
            continue;
        }
        for (int c = 0; c < nch; ++c) {
            if (H.n < CCD_HEAP) {
                H.push(ch[c]);
                continue;
            }
            // the heap is full: walk this child's subtree depth first
            int sp = 0;
            st[sp++] = ch[c];
            while (sp > 0 && !S.capped && !S.unresolved) {
                const CBox d = st[--sp];
                if (S.skip(d)) continue;
                CBox dc[2];
                int ndc;
                if (!S.step(d, dc, ndc)) {
                    if (S.capped) capped_t = d.lo[0];
                    continue;
                }
                for (int k = 0; k < ndc; ++k) st[sp++] = dc[k]; // the earlier (lower) half pops first
            }
            if (S.capped) {
                for (int k = 0; k < sp; ++k) capped_t = fmin(capped_t, st[k].lo[0]);
                break;
            }
        }
    }
    if (S.unresolved) return CCD_UNRESOLVED;
    if (S.capped) {
        // out of iterations: the earliest unresolved time bounds the root
        for (int k = 0; k < H.n; ++k) capped_t = fmin(capped_t, H.a[k].lo[0]);
        toi = S.found ? fmin(S.best.lo[0], capped_t) : capped_t;
        out_tol = S.out_tol;
        return CCD_HIT;
    }
    out_tol = S.found ? S.out_tol : 0;
    if (S.found) toi = S.best.lo[0];
    return S.found ? CCD_HIT : CCD_MISS;
}

// ---- the same search with a warp per query ----
// FP64 instructions cost the same pipe time however many lanes are active,
// so a long query's boxes are better examined 32 at a time: every round the
// warp takes the 32 first boxes (in box order) of a pool kept sorted in
// shared memory, examines them in parallel, keeps the first accepted box of
// the round if it comes before the best so far, and merges the kept children
// (sorted by a bitonic network) back into the pool.  The search ends when the
// pool's first box is skipped.  The result -- the first accepted box in box
// order -- is the same as the one-thread search's: every box before it is
// examined either way.  A pool that would overflow hands its last boxes to
// the lanes, which walk their subtrees depth first (as the one-thread search
// does with a full heap).  The box count for the iteration cap and the budget
// is the warp's total (checked per round).
constexpr int WPOOL = 256; // sorted pool per warp
constexpr int WCH = 64;    // children per round (2 per lane)
struct WarpPool {
    CBox* cur;  // WPOOL + WCH
    CBox* nxt;  // WPOOL + WCH
    CBox* ch;   // WCH
};
constexpr int CCD_WARP_SMEM = (2 * (WPOOL + WCH) + WCH) * (int)sizeof(CBox); // per warp

__device__ __forceinline__ CBox shfl_box(const CBox& b, int src_or_mask, bool xor_mode)
{
    CBox r;
    const unsigned FULL = 0xffffffffu;
    const int packed = (b.lvl[0] & 0xff) | ((b.lvl[1] & 0xff) << 8) | ((b.lvl[2] & 0xff) << 16);
    int pk;
    if (xor_mode) {
        for (int d = 0; d < 3; ++d) r.lo[d] = __shfl_xor_sync(FULL, b.lo[d], src_or_mask);
        pk = __shfl_xor_sync(FULL, packed, src_or_mask);
    } else {
        for (int d = 0; d < 3; ++d) r.lo[d] = __shfl_sync(FULL, b.lo[d], src_or_mask);
        pk = __shfl_sync(FULL, packed, src_or_mask);
    }
    for (int d = 0; d < 3; ++d) r.lvl[d] = (int8_t)((pk >> (8 * d)) & 0xff);
    return r;
}

__device__ __forceinline__ CBox end_box()
{
    CBox b;
    b.lo[0] = b.lo[1] = b.lo[2] = __longlong_as_double(0x7ff0000000000000LL);
    b.lvl[0] = b.lvl[1] = b.lvl[2] = 0;
    return b;
}

// Number of boxes in a[0, n) (sorted) that come before x (strict) or, with
// or_equal, not after it.
__device__ __forceinline__ int rank_in(const CBox* a, int n, const CBox& x, bool or_equal)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const bool left = or_equal ? !box_before(x, a[mid]) : box_before(a[mid], x);
        if (left) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ int root_finder_warp(const Query& q, const double err[3], double ms, const double tol[3], double delta,
    double tmax, long long max_itr, double& toi, double& out_tol, const unsigned long long* shared_best, Budget& bud,
    const WarpPool& w)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    Search S { q, err, ms, delta, tol, tmax, CBox {}, false, 0.0, 0, max_itr > 0 ? max_itr : 100000000LL, bud, false,
        false };
    CBox* cur = w.cur;
    CBox* nxt = w.nxt;
    if (lane == 0) {
        CBox root;
        root.lo[0] = root.lo[1] = root.lo[2] = 0;
        root.lvl[0] = root.lvl[1] = root.lvl[2] = 0;
        cur[0] = root;
    }
    __syncwarp();
    int n = 1;
    double capped_t = tmax;
    long long itr0 = 0, spent0 = bud.spent;
    CBox st[CCD_STACK];
    while (n > 0) {
        if (shared_best)
            S.tmax = fmin(S.tmax, __longlong_as_double((long long)*(volatile const unsigned long long*)shared_best));
        S.tmax = __shfl_sync(FULL, S.tmax, 0);
        if (S.skip(cur[0])) break; // the pool's first box: every other one comes later
        const int m = min(32, n);
        // examine the round's boxes
        S.itr = itr0;
        bud.spent = spent0;
        CBox ch[2];
        int nch = 0;
        bool acc = false;
        CBox accb = end_box();
        double acc_tol = 0;
        if (lane < m) {
            const CBox b = cur[lane];
            if (!S.skip(b)) {
                const bool had = S.found;
                const CBox prev = S.best;
                if (!S.step(b, ch, nch)) {
                    if (S.found && (!had || box_before(S.best, prev))) {
                        acc = true;
                        accb = S.best;
                        acc_tol = S.out_tol;
                    }
                    if (S.capped) capped_t = fmin(capped_t, b.lo[0]);
                }
            }
        }
        // the warp's totals and verdicts
        const int done = __popc(__ballot_sync(FULL, lane < m));
        itr0 += done;
        spent0 += done;
        const bool any_unres = __any_sync(FULL, S.unresolved);
        const bool any_cap = __any_sync(FULL, S.capped);
        if (any_unres) {
            bud.spent = spent0;
            return CCD_UNRESOLVED;
        }
        if (__any_sync(FULL, acc)) {
            // the first accepted box of the round
            CBox c = accb;
            double ct = acc_tol;
            for (int off = 16; off > 0; off >>= 1) {
                const CBox o = shfl_box(c, off, true);
                const double ot = __shfl_xor_sync(FULL, ct, off);
                if (box_before(o, c)) {
                    c = o;
                    ct = ot;
                }
            }
            S.best = c;
            S.out_tol = ct;
            S.found = true;
        } else {
            // every lane keeps the warp's best (lanes that examined nothing
            // may not have it)
            const int src = __ffs(__ballot_sync(FULL, S.found)) - 1;
            if (src >= 0) {
                S.best = shfl_box(S.best, src, false);
                S.out_tol = __shfl_sync(FULL, S.out_tol, src);
                S.found = true;
            }
        }
        if (any_cap) {
            S.capped = true;
            for (int off = 16; off > 0; off >>= 1) capped_t = fmin(capped_t, __shfl_xor_sync(FULL, capped_t, off));
            // the unexamined boxes bound the root from below
            for (int i = lane; i < n; i += 32) capped_t = fmin(capped_t, cur[i].lo[0]);
            for (int off = 16; off > 0; off >>= 1) capped_t = fmin(capped_t, __shfl_xor_sync(FULL, capped_t, off));
            break;
        }
        // the kept children, compacted into the round's buffer and sorted
        int keep = 0;
        CBox kc[2];
        for (int c = 0; c < nch; ++c)
            if (!S.skip(ch[c])) kc[keep++] = ch[c];
        int off = keep;
        for (int d = 1; d < 32; d <<= 1) {
            const int v = __shfl_up_sync(FULL, off, d);
            if (lane >= d) off += v;
        }
        const int C = __shfl_sync(FULL, off, 31);
        off -= keep;
        for (int c = 0; c < keep; ++c) w.ch[off + c] = kc[c];
        for (int i = C + lane; i < WCH; i += 32) w.ch[i] = end_box();
        __syncwarp();
        for (int k = 2; k <= WCH; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                // lane handles the pair (i, i ^ j) with i = its index with bit j clear
                const int i = ((lane & ~(j - 1)) << 1) | (lane & (j - 1));
                const int l = i ^ j;
                const bool up = (i & k) == 0;
                const CBox a = w.ch[i], b = w.ch[l];
                if (box_before(b, a) == up) {
                    w.ch[i] = b;
                    w.ch[l] = a;
                }
                __syncwarp();
            }
        // merge the pool's rest cur[m, n) with the children
        const int r = n - m;
        for (int i = lane; i < r; i += 32) {
            const CBox x = cur[m + i];
            nxt[i + rank_in(w.ch, C, x, false)] = x;
        }
        for (int k = lane; k < C; k += 32) {
            const CBox y = w.ch[k];
            nxt[k + rank_in(cur + m, r, y, true)] = y;
        }
        __syncwarp();
        n = r + C;
        CBox* t = cur;
        cur = nxt;
        nxt = t;
        if (n > WPOOL) {
            // overflow: the last boxes' subtrees are walked depth first, one
            // box per lane (at most 2 per lane)
            bool lane_acc = false;
            S.itr = itr0;
            bud.spent = spent0;
            for (int i = WPOOL + lane; i < n; i += 32) {
                int sp = 0;
                st[sp++] = cur[i];
                while (sp > 0 && !S.capped && !S.unresolved) {
                    const CBox d = st[--sp];
                    if (S.skip(d)) continue;
                    CBox dc[2];
                    int ndc;
                    const bool had = S.found;
                    const CBox prev = S.best;
                    if (!S.step(d, dc, ndc)) {
                        if (S.found && (!had || box_before(S.best, prev))) lane_acc = true;
                        if (S.capped) capped_t = fmin(capped_t, d.lo[0]);
                        continue;
                    }
                    for (int k = 0; k < ndc; ++k) st[sp++] = dc[k];
                }
                if (S.capped)
                    for (int k = 0; k < sp; ++k) capped_t = fmin(capped_t, st[k].lo[0]);
            }
            // totals again
            long long extra = S.itr - itr0;
            for (int o = 16; o > 0; o >>= 1) extra += __shfl_xor_sync(FULL, extra, o);
            itr0 += extra;
            spent0 += extra;
            if (__any_sync(FULL, S.unresolved)) {
                bud.spent = spent0;
                return CCD_UNRESOLVED;
            }
            CBox c = lane_acc || S.found ? S.best : end_box();
            double ct = S.out_tol;
            for (int o = 16; o > 0; o >>= 1) {
                const CBox ob = shfl_box(c, o, true);
                const double ot = __shfl_xor_sync(FULL, ct, o);
                if (box_before(ob, c)) {
                    c = ob;
                    ct = ot;
                }
            }
            if (__any_sync(FULL, S.found)) {
                S.best = c;
                S.out_tol = ct;
                S.found = true;
            }
            if (__any_sync(FULL, S.capped)) {
                S.capped = true;
                for (int o = 16; o > 0; o >>= 1) capped_t = fmin(capped_t, __shfl_xor_sync(FULL, capped_t, o));
                for (int i = lane; i < WPOOL; i += 32) capped_t = fmin(capped_t, cur[i].lo[0]);
                for (int o = 16; o > 0; o >>= 1) capped_t = fmin(capped_t, __shfl_xor_sync(FULL, capped_t, o));
                break;
            }
            n = WPOOL;
        }
    }
    bud.spent = spent0;
    if (S.capped) {
        toi = S.found ? fmin(S.best.lo[0], capped_t) : capped_t;
        out_tol = S.out_tol;
        return CCD_HIT;
    }
    out_tol = S.found ? S.out_tol : 0;
    if (S.found) toi = S.best.lo[0];
    return S.found ? CCD_HIT : CCD_MISS;
}

__device__ int ti_ccd(const Query& q, double ms_in, double& toi, double tol_in, double tmax_in, long long max_itr,
    double& out_tol, bool no_zero_toi, const unsigned long long* shared_best, Budget& bud, const WarpPool* wp)
{
    double err[3];
    numerical_error(q, ms_in > 0, err);
    double tmax = tmax_in, delta = tol_in, ms = ms_in;
    double tol[3];
    domain_tol(q, delta, tol);
    int hit = CCD_MISS;
    for (int it = 0; it < 256; ++it) {
        double t = 0;
        hit = wp ? root_finder_warp(q, err, ms, tol, delta, tmax, max_itr, t, out_tol, shared_best, bud, *wp)
                 : root_finder(q, err, ms, tol, delta, tmax, max_itr, t, out_tol, shared_best, bud);
        if (hit == CCD_UNRESOLVED) return hit;
        if (hit == CCD_HIT) toi = t;
        if (!(no_zero_toi && hit == CCD_HIT && toi == 0)) return hit;
        if (out_tol > delta) tmax *= 0.9;
        else if (10 * delta < ms) ms *= 0.5;
        else {
            delta *= 0.5;
            domain_tol(q, delta, tol);
        }
    }
    return hit;
}

__device__ int strategy(const Query& q, double min_distance, double d0, const CCDParams& P, double adj, double tmax,
    double& toi, const unsigned long long* shared_best, Budget& bud, const WarpPool* wp)
{
    if (d0 <= min_distance) {
        toi = 0;
        return CCD_HIT;
    }
    double mind = (1.0 - P.rescale) * (d0 - min_distance);
    mind = fmin(mind, 1e-4);
    mind += min_distance;
    double out_tol;
    int hit = ti_ccd(q, mind, toi, adj, tmax, P.max_iterations, out_tol, false, shared_best, bud, wp);
    if (hit == CCD_HIT && toi < 1e-6) {
        hit = ti_ccd(q, min_distance, toi, adj, tmax, -1, out_tol, true, shared_best, bud, wp);
        if (hit == CCD_HIT) toi *= P.rescale;
    }
    return hit;
}

__device__ int stencil_ccd(Query& q, double min_distance, const CCDParams& P, double tmax, double& toi,
    const unsigned long long* shared_best, Budget& bud, const WarpPool* wp = nullptr)
{
    double d2;
    if (q.vf) d2 = point_triangle_distance(q.s[0], q.s[1], q.s[2], q.s[3],
        point_triangle_distance_type(q.s[0], q.s[1], q.s[2], q.s[3]));
    else d2 = edge_edge_distance(q.s[0], q.s[1], q.s[2], q.s[3],
        edge_edge_distance_type(q.s[0], q.s[1], q.s[2], q.s[3]));
    const double d0 = sqrt(d2);
    if (v3eq(q.s[0], q.e[0]) && v3eq(q.s[1], q.e[1]) && v3eq(q.s[2], q.e[2]) && v3eq(q.s[3], q.e[3])) {
        if (d0 <= min_distance) {
            toi = 0;
            return CCD_HIT;
        }
        return CCD_MISS;
    }
    const double adj = fmin(0.5 * d0, P.tolerance);
    return strategy(q, min_distance, d0, P, adj, tmax, toi, shared_best, bud, wp);
}

// First sorted position of every scene that has queries.
__global__ void k_ccd_segments(const unsigned long long* __restrict__ keys, int n, int* __restrict__ seg)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int scene = (int)(keys[p] >> CCD_SCENE_SHIFT);
    if (p == 0 || (int)(keys[p - 1] >> CCD_SCENE_SHIFT) != scene) seg[scene] = p;
}

// The seed list: each scene's first CCD_SEEDS queries by estimate (thread
// k * CCD_SEEDS + j takes the j-th of scene k, if it has one).
constexpr int CCD_SEEDS = 32;
__global__ void k_ccd_seed_list(const unsigned long long* __restrict__ keys, const int* __restrict__ sorted, int n,
    const int* __restrict__ seg, int n_scenes, int* __restrict__ seeds, int* __restrict__ n_seeds)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_scenes * CCD_SEEDS) return;
    const int k = t / CCD_SEEDS, j = t % CCD_SEEDS;
    const int p = seg[k] + j;
    if (seg[k] < 0 || p >= n || (int)(keys[p] >> CCD_SCENE_SHIFT) != k) return;
    seeds[atomicAdd(n_seeds, 1)] = sorted[p];
}

// One thread per candidate (candidates.cpp:252-292).  With a box budget
// (pass 1) a query that does not finish within it is appended to `hard`
// instead; those are run to completion in pass 2 (hard != null selects the
// candidate list), by which time the earliest time of the easy queries
// prunes them.  Each query's result does not depend on the pass, so the
// minimum is the same as a single full pass.  In a batch each scene has its
// own minimum distance and its own earliest time (toi_bits[scene]).
__global__ void __launch_bounds__(BLOCK, 3) k_ccd(const int2* __restrict__ cand_ee, int n_ee,
    const int2* __restrict__ cand_fv, int n_fv, const double* __restrict__ V0, const double* __restrict__ V1,
    const int* __restrict__ E, const int* __restrict__ F, const double* __restrict__ min_distance, SceneView sv,
    CCDParams P, unsigned long long* toi_bits, long long budget, const int* __restrict__ list,
    const int* __restrict__ list_n, int list_len, int* __restrict__ hard, int* __restrict__ hard_n, int any_hit,
    const double* __restrict__ lb, const int* __restrict__ seg, long long* __restrict__ stats)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = list ? (list_n ? *list_n : list_len) : n_ee + n_fv;
    if (t >= n) return;
    const int i = list ? list[t] : t;
    Query q;
    const int scene = sv.of(load_query(i, cand_ee, n_ee, cand_fv, V0, V1, E, F, q));
    // the sorted list's first CCD_SEEDS queries of each scene ran as seeds
    if (seg && t - seg[scene] < CCD_SEEDS) return;
    unsigned long long* best = toi_bits + scene;
    const double tmax = __longlong_as_double((long long)*(volatile unsigned long long*)best);
    // a query whose time of impact cannot come before the scene's earliest
    // so far cannot change the result
    if (lb) {
        const double b = lb[i];
        if (b >= 1e-6 && b >= tmax) return;
    }
    double toi = __longlong_as_double(0x7ff0000000000000ULL);
    Budget bud { budget, 0 };
    const int st = stencil_ccd(q, __ldg(min_distance + scene), P, tmax, toi, best, bud);
    // any_hit (is_step_collision_free): a hit anywhere answers the question;
    // setting the scene's earliest time to 0 also stops every other query
    if (st == CCD_HIT && any_hit) atomicMin(best, 0ULL);
    else if (st == CCD_HIT && toi < tmax) atomicMin(best, (unsigned long long)__double_as_longlong(toi));
    else if (st == CCD_UNRESOLVED) hard[atomicAdd(hard_n, 1)] = i;
    if (stats) {
        // testing: queries run, boxes, the largest query, hits
        atomicAdd((unsigned long long*)stats, 1ull);
        atomicAdd((unsigned long long*)stats + 1, (unsigned long long)bud.spent);
        atomicMax(stats + 2, bud.spent);
        if (st == CCD_HIT) atomicAdd((unsigned long long*)stats + 3, 1ull);
    }
}

// The warp-per-query pass (the seeds, and the queries the budgeted pass left
// unfinished): like k_ccd, with every lane of a warp on the same query.
constexpr int WARPS_PER_BLOCK = 4;
__global__ void __launch_bounds__(32 * WARPS_PER_BLOCK) k_ccd_warp(const int2* __restrict__ cand_ee, int n_ee,
    const int2* __restrict__ cand_fv, int n_fv, const double* __restrict__ V0, const double* __restrict__ V1,
    const int* __restrict__ E, const int* __restrict__ F, const double* __restrict__ min_distance, SceneView sv,
    CCDParams P, unsigned long long* toi_bits, long long budget, const int* __restrict__ list,
    const int* __restrict__ list_n, int* __restrict__ hard, int* __restrict__ hard_n, int any_hit,
    const double* __restrict__ lb, long long* __restrict__ stats)
{
    extern __shared__ unsigned char smem[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    CBox* base = reinterpret_cast<CBox*>(smem + (size_t)wib * CCD_WARP_SMEM);
    const WarpPool wp { base, base + (WPOOL + WCH), base + 2 * (WPOOL + WCH) };
    const int n = *list_n;
    for (int t = blockIdx.x * WARPS_PER_BLOCK + wib; t < n; t += gridDim.x * WARPS_PER_BLOCK) {
        const int i = list[t];
        Query q;
        const int scene = sv.of(load_query(i, cand_ee, n_ee, cand_fv, V0, V1, E, F, q));
        unsigned long long* best = toi_bits + scene;
        double tmax = 0;
        if (lane == 0) tmax = __longlong_as_double((long long)*(volatile unsigned long long*)best);
        tmax = __shfl_sync(0xffffffffu, tmax, 0);
        if (lb) {
            const double b = lb[i];
            if (b >= 1e-6 && b >= tmax) continue;
        }
        double toi = __longlong_as_double(0x7ff0000000000000ULL);
        Budget bud { budget, 0 };
        const int st = stencil_ccd(q, __ldg(min_distance + scene), P, tmax, toi, best, bud, &wp);
        if (lane == 0) {
            if (st == CCD_HIT && any_hit) atomicMin(best, 0ULL);
            else if (st == CCD_HIT && toi < tmax) atomicMin(best, (unsigned long long)__double_as_longlong(toi));
            else if (st == CCD_UNRESOLVED) hard[atomicAdd(hard_n, 1)] = i;
            if (stats) {
                atomicAdd((unsigned long long*)stats, 1ull);
                atomicAdd((unsigned long long*)stats + 1, (unsigned long long)bud.spent);
                atomicMax(stats + 2, bud.spent);
                if (st == CCD_HIT) atomicAdd((unsigned long long*)stats + 3, 1ull);
            }
        }
        __syncwarp();
    }
}

__global__ void k_ccd_stencils(int is_ee, int n, const double* __restrict__ x0, const double* __restrict__ x1,
    double min_distance, double tmax, CCDParams P, int8_t* __restrict__ hit, double* __restrict__ toi)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Query q;
    q.vf = !is_ee;
    for (int k = 0; k < 4; ++k) {
        q.s[k] = load_v3(x0 + 12 * (int64_t)i, k);
        q.e[k] = load_v3(x1 + 12 * (int64_t)i, k);
    }
    q.set_deltas();
    double t = __longlong_as_double(0x7ff0000000000000ULL);
    Budget bud { 0, 0 };
    const int h = stencil_ccd(q, min_distance, P, tmax, t, nullptr, bud);
    hit[i] = h == CCD_HIT ? 1 : 0;
    toi[i] = t;
}

__global__ void k_distance_stencils(int kind, int n, const double* __restrict__ x, int8_t* __restrict__ dtype,
    double* __restrict__ dist)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (kind == 0) {
        const double* p = x + 9 * (int64_t)i;
        const V3 a = load_v3(p, 0), b = load_v3(p, 1), c = load_v3(p, 2);
        const int t = point_edge_distance_type(a, b, c);
        dtype[i] = (int8_t)t;
        dist[i] = point_edge_distance(a, b, c, t);
    } else {
        const double* p = x + 12 * (int64_t)i;
        const V3 a = load_v3(p, 0), b = load_v3(p, 1), c = load_v3(p, 2), d = load_v3(p, 3);
        if (kind == 1) {
            const int t = point_triangle_distance_type(a, b, c, d);
            dtype[i] = (int8_t)t;
            dist[i] = point_triangle_distance(a, b, c, d, t);
        } else {
            const int t = edge_edge_distance_type(a, b, c, d);
            dtype[i] = (int8_t)t;
            dist[i] = edge_edge_distance(a, b, c, d, t);
        }
    }
}

} // namespace

// The CCD passes over candidate lists (EE pairs, then FV (face, vertex)
// pairs).  Every query first gets a lower bound on its time of impact and an
// estimate of it; the queries are sorted by scene and estimate, each scene's
// likeliest earliest impacts run first (the seeds) and set its earliest
// time, which then skips every query whose bound is not below it.  The sorted list runs with a box budget, then the
// unfinished queries to completion.  toi_bits (one per scene, set by the
// caller) is the scene's earliest time so far; with any_hit a hit sets it to
// 0 instead.
void ccd_passes(ipcg_mesh* m, const int2* cee, int64_t n_ee, const int2* cfv, int64_t n_fv, const double* V0,
    const double* V1, const double* md, const CCDParams& P, int any_hit)
{
    cudaStream_t s = m->stream;
    const SceneView sv = scene_view(m);
    if (n_ee + n_fv >= (int64_t)INT32_MAX) throw Error(IPCG_ERR_INVALID, "too many CCD candidates");
    if (m->n_scenes >= (1 << (64 - CCD_SCENE_SHIFT))) throw Error(IPCG_ERR_INVALID, "too many scenes for the CCD");
    const int nc = (int)(n_ee + n_fv);
    if (nc == 0) return;
    const int ns = (int)m->n_scenes;
    m->ivals_a.reserve((int64_t)nc + 1 + ns + (int64_t)ns * CCD_SEEDS + 1);
    m->ivals_b.reserve(2 * (nc + 1));
    m->keys_a.reserve(nc + 1);
    m->keys_b.reserve(nc + 1);
    m->ccd_lb.reserve(nc + 1);
    int* hard = m->ivals_a.p;                       // left by the budgeted passes
    int* seg = m->ivals_a.p + nc + 1;               // per scene: its first sorted position
    int* seeds = m->ivals_a.p + nc + 1 + ns;        // each scene's first queries by bound
    int* ids = m->ivals_b.p;
    int* sorted = m->ivals_b.p + nc + 1;
    m->counters.reserve(32);
    int* seeds_n = m->counters.p + 30;
    int* hard_n = m->counters.p + 31;
    IPCG_CUDA(cudaMemsetAsync(seeds_n, 0, 2 * sizeof(int), s));
    // testing: per pass (seeds, budgeted, hard) queries run, boxes, the
    // largest query, hits, accumulated until read
    long long* st = nullptr;
    if (g_ccd_stats.load()) {
        m->ccd_stats.reserve(12);
        if (!m->ccd_stats_live) {
            IPCG_CUDA(cudaMemsetAsync(m->ccd_stats.p, 0, sizeof(long long) * 12, s));
            m->ccd_stats_live = true;
        }
        st = m->ccd_stats.p;
    }
    IPCG_CUDA(cudaMemsetAsync(seg, 0xff, sizeof(int) * ns, s));
    ccd_bound_launch(s, cee, (int)n_ee, cfv, (int)n_fv, V0, V1, m->E.p, m->F.p, md, sv, P.tolerance, P.rescale,
        m->ccd_lb.p, m->keys_a.p, ids);
    sort_pairs_u64(m, s, m->keys_a.p, m->keys_b.p, ids, sorted, nc, 64);
    IPCG_LAUNCH("k_ccd_segments", s, k_ccd_segments<<<grid_for(nc, 256), 256, 0, s>>>(m->keys_b.p, nc, seg));
    IPCG_LAUNCH("k_ccd_seed_list", s, k_ccd_seed_list<<<grid_for((int64_t)ns * CCD_SEEDS, 256), 256, 0, s>>>(
        m->keys_b.p, sorted, nc, seg, ns, seeds, seeds_n));
    const long long tb = g_ccd_thread_budget.load() > 0 ? g_ccd_thread_budget.load() : CCD_PASS1_BUDGET;
    // seeds first: each scene's likeliest earliest impacts set its earliest
    // time before the bulk of its queries runs (in the same order)
    const int wsmem = WARPS_PER_BLOCK * CCD_WARP_SMEM;
    static bool smem_set[64] = {};
    if (m->device >= 0 && m->device < 64 && !smem_set[m->device]) {
        IPCG_CUDA(cudaFuncSetAttribute(k_ccd_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, wsmem));
        smem_set[m->device] = true;
    }
    const int wblocks = std::max(1, std::min(ns * CCD_SEEDS / WARPS_PER_BLOCK + 1, 152 * 8));
    IPCG_LAUNCH("k_ccd_seeds", s, k_ccd_warp<<<wblocks, 32 * WARPS_PER_BLOCK, wsmem, s>>>(cee, (int)n_ee, cfv,
        (int)n_fv, V0, V1, m->E.p, m->F.p, md, sv, P, m->toi_bits.p, CCD_SEED_BUDGET, seeds, seeds_n, hard, hard_n,
        any_hit, m->ccd_lb.p, st ? st : nullptr));
    IPCG_LAUNCH("k_ccd", s, k_ccd<<<grid_for(nc, BLOCK), BLOCK, 0, s>>>(cee, (int)n_ee, cfv, (int)n_fv, V0, V1,
        m->E.p, m->F.p, md, sv, P, m->toi_bits.p, tb, sorted, nullptr, nc, hard, hard_n, any_hit,
        m->ccd_lb.p, seg, st ? st + 4 : nullptr));
    IPCG_LAUNCH("k_ccd_hard", s, k_ccd_warp<<<152 * 8, 32 * WARPS_PER_BLOCK, wsmem, s>>>(cee, (int)n_ee, cfv,
        (int)n_fv, V0, V1, m->E.p, m->F.p, md, sv, P, m->toi_bits.p, 0, hard, hard_n, nullptr, nullptr, any_hit,
        m->ccd_lb.p, st ? st + 8 : nullptr));
}

void collision_free_stepsize(ipcg_mesh* m, const double* V0, const double* V1, const double* min_distance,
    double tolerance, int64_t max_iterations, double rescale, double* steps, int64_t* n_candidates)
{
    cudaStream_t s = m->stream;
    const int ns = (int)m->n_scenes;
    // per scene: broad-phase inflation 0.5 * min_distance, then min_distance
    std::vector<double> h(2 * ns);
    for (int k = 0; k < ns; ++k) {
        h[k] = 0.5 * min_distance[k];
        h[ns + k] = min_distance[k];
    }
    m->scene_md.reserve(2 * ns);
    IPCG_CUDA(cudaMemcpyAsync(m->scene_md.p, h.data(), sizeof(double) * 2 * ns, cudaMemcpyHostToDevice, s));
    int64_t n_ee = 0, n_fv = 0;
    detect_candidates(m, V0, V1, m->scene_md.p, n_ee, n_fv);
    if (n_candidates) *n_candidates = n_ee + n_fv;
    if (n_ee + n_fv == 0) {
        for (int k = 0; k < ns; ++k) steps[k] = 1.0;
        return;
    }
    m->toi_bits.reserve(ns);
    std::vector<unsigned long long> ones(ns, 0x3ff0000000000000ULL); // 1.0
    IPCG_CUDA(cudaMemcpyAsync(m->toi_bits.p, ones.data(), sizeof(unsigned long long) * ns, cudaMemcpyHostToDevice,
        s));
    const CCDParams P { tolerance, (long long)max_iterations, rescale };
    ccd_passes(m, m->cand.p, n_ee, m->cand.p + m->cand_cap, n_fv, V0, V1, m->scene_md.p + ns, P, 0);
    std::vector<unsigned long long> bits(ns);
    IPCG_CUDA(cudaMemcpyAsync(bits.data(), m->toi_bits.p, sizeof(unsigned long long) * ns, cudaMemcpyDeviceToHost,
        s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < ns; ++k) memcpy(steps + k, &bits[k], sizeof(double));
}

bool step_collision_free(ipcg_mesh* m, const double* V0, const double* V1, double min_distance, double tolerance,
    int64_t max_iterations, double rescale)
{
    if (m->n_scenes != 1) throw Error(IPCG_ERR_INVALID, "is_step_collision_free takes a single-scene mesh");
    cudaStream_t s = m->stream;
    const double h[2] = { 0.5 * min_distance, min_distance };
    m->scene_md.reserve(2);
    IPCG_CUDA(cudaMemcpyAsync(m->scene_md.p, h, sizeof(h), cudaMemcpyHostToDevice, s));
    int64_t n_ee = 0, n_fv = 0;
    detect_candidates(m, V0, V1, m->scene_md.p, n_ee, n_fv);
    if (n_ee + n_fv == 0) return true;
    m->toi_bits.reserve(1);
    const unsigned long long one = 0x3ff0000000000000ULL; // 1.0
    IPCG_CUDA(cudaMemcpyAsync(m->toi_bits.p, &one, sizeof(one), cudaMemcpyHostToDevice, s));
    const CCDParams P { tolerance, (long long)max_iterations, rescale };
    ccd_passes(m, m->cand.p, n_ee, m->cand.p + m->cand_cap, n_fv, V0, V1, m->scene_md.p + 1, P, 1);
    unsigned long long bits = 1;
    IPCG_CUDA(cudaMemcpyAsync(&bits, m->toi_bits.p, sizeof(bits), cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    return bits != 0;
}

double candidates_collision_free_stepsize(ipcg_mesh* m, const int2* cee, int64_t n_ee, const int2* cfv,
    int64_t n_fv, const double* V0, const double* V1, double min_distance, double tolerance, int64_t max_iterations,
    double rescale)
{
    if (m->n_scenes != 1) throw Error(IPCG_ERR_INVALID, "candidate sets are built on single-scene meshes");
    if (n_ee + n_fv == 0) return 1.0;
    cudaStream_t s = m->stream;
    m->scene_md.reserve(2);
    const double h[2] = { 0.5 * min_distance, min_distance };
    IPCG_CUDA(cudaMemcpyAsync(m->scene_md.p, h, sizeof(h), cudaMemcpyHostToDevice, s));
    m->toi_bits.reserve(1);
    m->counters.reserve(16);
    const unsigned long long one = 0x3ff0000000000000ULL; // 1.0
    IPCG_CUDA(cudaMemcpyAsync(m->toi_bits.p, &one, sizeof(one), cudaMemcpyHostToDevice, s));
    const CCDParams P { tolerance, (long long)max_iterations, rescale };
    ccd_passes(m, cee, n_ee, cfv, n_fv, V0, V1, m->scene_md.p + 1, P, 0);
    unsigned long long bits = 0;
    IPCG_CUDA(cudaMemcpyAsync(&bits, m->toi_bits.p, sizeof(bits), cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    double t;
    memcpy(&t, &bits, sizeof(t));
    return t;
}

void ccd_stencils(cudaStream_t s, int is_ee, int64_t n, const double* x0, const double* x1, double min_distance,
    double tmax, double tolerance, int64_t max_iterations, double rescale, int8_t* hit, double* toi)
{
    if (n <= 0) return;
    const CCDParams P { tolerance, (long long)max_iterations, rescale };
    IPCG_LAUNCH("k_ccd_stencils", s, k_ccd_stencils<<<grid_for(n, BLOCK), BLOCK, 0, s>>>(is_ee, (int)n, x0, x1, min_distance, tmax, P, hit, toi));
    IPCG_CHECK_LAUNCH();
}

void distance_stencils(cudaStream_t s, int kind, int64_t n, const double* x, int8_t* dtype, double* dist)
{
    if (n <= 0) return;
    IPCG_LAUNCH("k_distance_stencils", s, k_distance_stencils<<<grid_for(n, 256), 256, 0, s>>>(kind, (int)n, x, dtype, dist));
    IPCG_CHECK_LAUNCH();
}

} // namespace ipcg
