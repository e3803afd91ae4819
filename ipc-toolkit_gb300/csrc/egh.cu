// egh.cu — barrier energy, gradient and PSD-projected Hessian in one pass,
// with a cached sparsity pattern and the whole step replayed as a CUDA graph.
//
// Restates src/ipc/potentials/potential.cpp:36-222 (sum over contacts, dense
// gradient, sparse Hessian from local 3n x 3n blocks with duplicates summed),
// normal_potential.cpp:127-232 (per-contact energy, gradient and Hessian) and
// eigen_ext.tpp:64-108 (PSD projection), the way SparseMatrixCache
// (matrix_cache.cpp:80-214) reuses a pattern between Newton iterations.
//
// Per collision set (rebuilt only when the set, the mesh or the chunk bound
// changes) the pattern is built once: every contact's n^2 vertex blocks are
// keyed (row << 32 | col), radix-sorted and run-length encoded, which gives
// the CSR pattern, and for every contribution its slot in block-sorted order
// (perm).  The gradient's contributions (a contact's diagonal blocks) get
// slots grouped by vertex the same way.  A step is then, per chunk,
//   k_local (persistent): warps take 32-contact tiles from a work queue; each
//     lane computes one contact's energy, gradient and local Hessian and
//     writes the energy to its own slot, the gradient to its vertex-grouped
//     slots and the Hessian to an element-major local slab;
//   k_psd_scatter (persistent, same queue scheme): each lane projects one
//     local Hessian to PSD (its negative eigenpairs in FP64, or in df64 on
//     the FP32 pipes) and writes each 3x3 block to its block-sorted slot;
//   k_hess_reduce / k_grad_reduce / k_energy_parts: streaming sums of
//     contiguous runs of slots into the CSR values, the gradient and partial
//     energies, each value written once;
// and k_energy_scenes sums each scene's partial energies at the end.
// Everything is in fixed order (deterministic: no launch shape changes a
// bit) and every size is known from the pattern, so no step needs the host:
// from a pattern's second step on, the launches of a step are captured once
// into a CUDA graph and replayed, reading the call's pointers (positions,
// outputs, scratch) from a small device-side argument block that is updated
// before each replay (a pattern's first step runs as plain launches).
//
// The two per-contact stages are split because they want different
// residency: the local Hessian code is long and register-heavy, the
// projection short of registers but heavy on per-thread scratch.  Each
// stage's grid shape (threads per block, blocks per SM) and work-queue grab
// size are chosen by a small autotuner per device.
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "contact.cuh"
#include "profile.cuh"

namespace ipcg {

// CSR row pointers and columns of a cached pattern; matrices built on it
// share them (and keep them alive after the set is rebuilt).
struct EghPattern {
    DBuf<int64_t> row_ptr;
    DBuf<int> col;
};

namespace {

// Pointers of one call, read by the graph's kernels from device memory: the
// positions, the outputs, and the step's scratch (taken from the library's
// stream-ordered pool for the call, so sets on many meshes share it).
struct EghDev {
    const double* V;
    double* grad;
    double* val;
    double *slab, *gslab, *eslab;
    double* lh;             // local Hessians, element-major
    unsigned char* pflag;   // per contact: its Hessian is to be projected
    double* epart;          // energy partial sums
    int64_t* fixlist;       // contacts the df64 projection left to FP64
};

// A run of consecutive scenes whose contacts are processed together (one
// chunk for a single scene or a small batch).  Contacts of type t in the
// chunk are [lo[t], hi[t]) of that type's list; the chunk-local contact
// index runs VV | EV | EE | FV.
struct EChunk {
    int64_t lo[4], hi[4];
    int64_t r0, r1;        // vertex rows
    int64_t k0, k1;        // scenes
    int64_t n, ncontrib;   // contacts, Hessian contributions (sum of n^2)
    int64_t B0, nb;        // first CSR block, blocks
    int64_t perm_off;      // offset of the chunk in perm (contributions)
    int64_t rs_off;        // offset in run_start (nb + 1 entries per chunk)
    int64_t gs_off;        // offset in gstart (r1 - r0 + 1 entries per chunk)
    int64_t gslot_off;     // offset in gslot (4 per contact)
    int64_t ep0, nep;      // energy parts
};

} // namespace

struct EghCache {
    // key
    uint64_t version = 0, mesh_serial = 0;
    int64_t budget = 0;
    bool valid = false;
    std::vector<EChunk> chunks;
    int64_t n = 0, nb = 0, max_contrib = 0, max_n = 0, max_gs = 0;
    std::shared_ptr<EghPattern> pattern;
    DBuf<unsigned> perm, run_start, gstart, gslot;
    DBuf<int64_t> vbase;   // per block: CSR position of its entry (0, 0)
    DBuf<int> vnbr;        // per block: blocks in its block row
    DBuf<int64_t> eparts;  // energy parts: chunk-local [begin, end) of eslab
    DBuf<int64_t> epstart; // per scene: its first energy part (ns + 1)
    int64_t nparts = 0;
    DBuf<double> energy;   // per-scene energies of the last step
    DBuf<unsigned long long> queue;    // per chunk: local F64, local F32, projection, fix-up count
    // a chunk's contacts ordered by arithmetic path and kind: keys (path),
    // sorted keys (pkey), contact indices (iota -> list), FP64 count (nsel)
    DBuf<int> iota, list, nsel;
    DBuf<unsigned char> path, pkey, part_tmp;
    size_t part_bytes = 0;
    DBuf<long long> fail;  // [failed, chunk-local contact, chunk, non-finite entries]
    HBuf<long long> hfail;
    DBuf<EghDev> dev;
    HBuf<EghDev> hdev;
    // captured step
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::string graph_key;
    int graph_kernels = 0;
    int64_t steps = 0; // steps run on this pattern
    ~EghCache()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

namespace {

constexpr int WANT_E = 1, WANT_G = 2, WANT_H = 4;

std::atomic<int> g_defer_df64 { 0 };
std::mutex g_tune_mu;
EghTuning g_tune[64][3];
bool g_tune_set[64][3] = {};

ContactsView full_view(const ipcg_collisions* cs)
{
    return ContactsView { cs->nvv, cs->nev, cs->nee, cs->nfv, cs->vv.p, cs->ev.p, cs->ee.p, cs->fv.p, cs->vv_w.p,
        cs->ev_w.p, cs->ee_w.p, cs->fv_w.p, cs->ee_eps.p, cs->ee_dtype.p };
}

ContactsView chunk_view(const ContactsView& cv, const EChunk& c)
{
    ContactsView v = cv;
    v.nvv = c.hi[0] - c.lo[0];
    v.nev = c.hi[1] - c.lo[1];
    v.nee = c.hi[2] - c.lo[2];
    v.nfv = c.hi[3] - c.lo[3];
    v.vv = cv.vv + c.lo[0];
    v.vv_w = cv.vv_w + c.lo[0];
    v.ev = cv.ev + c.lo[1];
    v.ev_w = cv.ev_w + c.lo[1];
    v.ee = cv.ee + c.lo[2];
    v.ee_w = cv.ee_w + c.lo[2];
    v.ee_eps = cv.ee_eps + c.lo[2];
    v.ee_dt = cv.ee_dt + c.lo[2];
    v.fv = cv.fv + c.lo[3];
    v.fv_w = cv.fv_w + c.lo[3];
    return v;
}

// First contribution of chunk-local contact i (VV: 4, EV: 9, EE / FV: 16 each).
__device__ __forceinline__ int64_t contrib_offset(const ContactsView& cv, int64_t i)
{
    if (i < cv.nvv) return 4 * i;
    if (i < cv.nvv + cv.nev) return 4 * cv.nvv + 9 * (i - cv.nvv);
    return 4 * cv.nvv + 9 * cv.nev + 16 * (i - cv.nvv - cv.nev);
}

// ---- pattern build (once per collision set) ----

__global__ void k_p_scene_ranges(ContactsView cv, const int64_t* __restrict__ offs, int S, int64_t* __restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * S) return;
    const int type = t / S;
    const int2* list = type == 0 ? cv.vv : (type == 1 ? cv.ev : (type == 2 ? cv.ee : cv.fv));
    const int64_t n = type == 0 ? cv.nvv : (type == 1 ? cv.nev : (type == 2 ? cv.nee : cv.nfv));
    const int64_t key = offs[t];
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (list[mid].x < key) lo = mid + 1;
        else hi = mid;
    }
    out[t] = lo;
}

__global__ void k_p_keys(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F,
    unsigned long long* __restrict__ keys, int* __restrict__ ids)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    const int64_t off = contrib_offset(cv, i);
    for (int a = 0; a < c.n; ++a)
        for (int b = 0; b < c.n; ++b) {
            keys[off + a * c.n + b] = ((unsigned long long)c.vid[a] << 32) | (unsigned)c.vid[b];
            ids[off + a * c.n + b] = (int)(off + a * c.n + b);
        }
}

__global__ void k_p_perm(const int* __restrict__ sorted_ids, int64_t n, unsigned* __restrict__ perm)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) perm[sorted_ids[s]] = (unsigned)s;
}

__global__ void k_p_runs(const int* __restrict__ start, int nb, unsigned total, unsigned* __restrict__ run_start)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nb) run_start[q] = (unsigned)start[q];
    if (q == nb) run_start[q] = total;
}

// Block row pointers (chunk-local) of rows r0 .. r0 + nr from the sorted keys.
__global__ void k_p_bptr(const unsigned long long* __restrict__ ukeys, int nb, int64_t r0, int nr, int* __restrict__ bptr)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > nr) return;
    const unsigned long long key = (unsigned long long)(r0 + j) << 32;
    int lo = 0, hi = nb;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ukeys[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    bptr[j] = lo;
}

// CSR rows 3 r0 .. 3 r1 of the chunk (B0 blocks of earlier chunks first).
__global__ void k_p_rows(const int* __restrict__ bptr, int64_t r0, int nr, int64_t B0, int64_t* __restrict__ row_ptr)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > nr) return;
    const int64_t b0 = B0 + bptr[j];
    const int64_t r = r0 + j;
    if (j == nr) {
        row_ptr[3 * r] = 9 * b0;
        return;
    }
    const int64_t nbr = bptr[j + 1] - bptr[j];
    for (int k = 0; k < 3; ++k) row_ptr[3 * r + k] = 9 * b0 + 3 * k * nbr;
}

// Per block: CSR columns, the position of entry (0, 0) and the row's block
// count; diagonal blocks record their run for the gradient slots.
__global__ void k_p_blocks(const unsigned long long* __restrict__ ukeys, int nb, const int* __restrict__ bptr,
    int64_t r0, int64_t B0, const int* __restrict__ run_len, int* __restrict__ col, int64_t* __restrict__ vbase,
    int* __restrict__ vnbr, int* __restrict__ diag_len, int* __restrict__ diag_q)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nb) return;
    const unsigned long long key = ukeys[q];
    const int64_t row = (int64_t)(key >> 32);
    const int cc = (int)(key & 0xffffffffu);
    const int j = (int)(row - r0);
    const int b0 = bptr[j];
    const int nbr = bptr[j + 1] - b0;
    const int64_t base = 9 * (B0 + b0) + 3 * (int64_t)(q - b0);
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) col[base + 3 * (int64_t)k * nbr + l] = 3 * cc + l;
    vbase[q] = base;
    vnbr[q] = nbr;
    if (row == cc) {
        diag_len[j] = run_len[q];
        diag_q[j] = q;
    }
}

// Gradient slot of (contact i, local vertex a): the rank of its diagonal
// contribution within the vertex's diagonal block, after the vertex's start.
__global__ void k_p_gslot(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F, int64_t r0,
    const unsigned* __restrict__ perm, const unsigned* __restrict__ run_start, const int* __restrict__ diag_q,
    const int* __restrict__ gstart, unsigned* __restrict__ gslot)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Local c;
    load_contact(cv, E, F, i, c);
    const int64_t off = contrib_offset(cv, i);
    for (int a = 0; a < c.n; ++a) {
        const int v = (int)(c.vid[a] - r0);
        const unsigned s = perm[off + a * c.n + a];
        gslot[4 * i + a] = (unsigned)gstart[v] + (s - run_start[diag_q[v]]);
    }
}

// ---- the step ----

// Local Hessians, element-major per stencil size: the VV contacts' 6x6
// matrices, then the EV contacts' 9x9, then the EE and FV contacts' 12x12
// (EE first), element k of the r-th matrix of a group at k * stride + r.
struct LhLayout {
    int64_t off[3], stride[3], first[3]; // per group: offset, contacts, first chunk-local contact
    __device__ __forceinline__ LhLayout(const ContactsView& cv)
    {
        first[0] = 0;
        first[1] = cv.nvv;
        first[2] = cv.nvv + cv.nev;
        stride[0] = cv.nvv;
        stride[1] = cv.nev;
        stride[2] = cv.nee + cv.nfv;
        off[0] = 0;
        off[1] = 36 * cv.nvv;
        off[2] = 36 * cv.nvv + 81 * cv.nev;
    }
};

// Contact j of type CT (j counts within the type's list).
template <int CT>
__device__ __forceinline__ void load_typed(const ContactsView& cv, const int* __restrict__ E, const int* __restrict__ F,
    int64_t j, Local& c)
{
    c.type = CT;
    if constexpr (CT == CT_VV) {
        const int2 p = cv.vv[j];
        c.n = 2;
        c.vid[0] = p.x;
        c.vid[1] = p.y;
        c.w = cv.vv_w[j];
    } else if constexpr (CT == CT_EV) {
        const int2 p = cv.ev[j];
        c.n = 3;
        c.vid[0] = p.y;
        c.vid[1] = E[2 * p.x];
        c.vid[2] = E[2 * p.x + 1];
        c.w = cv.ev_w[j];
    } else if constexpr (CT == CT_EE) {
        const int2 p = cv.ee[j];
        c.n = 4;
        c.vid[0] = E[2 * p.x];
        c.vid[1] = E[2 * p.x + 1];
        c.vid[2] = E[2 * p.y];
        c.vid[3] = E[2 * p.y + 1];
        c.w = cv.ee_w[j];
        c.eps = cv.ee_eps[j];
        c.dtype = cv.ee_dt[j];
    } else {
        const int2 p = cv.fv[j];
        c.n = 4;
        c.vid[0] = p.y;
        c.vid[1] = F[3 * p.x];
        c.vid[2] = F[3 * p.x + 1];
        c.vid[3] = F[3 * p.x + 2];
        c.w = cv.fv_w[j];
    }
}

// Energy, gradient and local Hessian of contact j of type CT (chunk-local
// index i): the energy to its own slot, the gradient to its vertex-grouped
// slots, the Hessian to the element-major local slab, whether it is to be
// projected to pflag.
// Which arithmetic a local-stage launch runs: it takes only contacts of the
// FP32 or only contacts of the FP64 path.
enum : int { PATH_F32 = 1, PATH_F64 = 2 };

template <int CT, int PATH>
__device__ __forceinline__ void local_one(const ContactsView& cv, const int* __restrict__ E, const int* __restrict__ F,
    const EghDev& d, const Params* __restrict__ sp, const SceneView& sv, const unsigned* __restrict__ gslot,
    const LhLayout& L, int64_t i, int64_t j, int want)
{
    constexpr int NS = CT == CT_VV ? 2 : (CT == CT_EV ? 3 : 4), N = 3 * NS, G = CT == CT_VV ? 0 : (CT == CT_EV ? 1 : 2);
    Local c;
    load_typed<CT>(cv, E, F, j, c);
    const Params P = sp[sv.of(c.vid[0])];
    V3 x[4];
#pragma unroll
    for (int a = 0; a < NS; ++a) x[a] = load_v3(d.V, c.vid[a]);
    double e, g[12], H[144];
    bool pr;
    if constexpr (PATH == PATH_F32) pr = contact_egh_f32(c, x, P, e, g, H);
    else pr = contact_egh_f64(c, x, P, e, g, H);
    if (want & WANT_E) d.eslab[i] = e;
    if (want & WANT_G)
#pragma unroll
        for (int a = 0; a < NS; ++a) {
            const int64_t s = gslot[4 * i + a];
            d.gslab[3 * s] = g[3 * a];
            d.gslab[3 * s + 1] = g[3 * a + 1];
            d.gslab[3 * s + 2] = g[3 * a + 2];
        }
    double* __restrict__ lh = d.lh + L.off[G] + (i - L.first[G]);
    const int64_t st = L.stride[G];
#pragma unroll 4
    for (int k = 0; k < N * N; ++k) lh[k * st] = H[k];
    d.pflag[i] = pr ? 1 : 0;
}

// Persistent work-queue loop: warps take `grab` 32-contact tiles at a time,
// the last tiles (the edge-edge and face-vertex contacts, the costly ones)
// first; body(i) runs for every chunk-local contact i < n.
template <class Body>
__device__ __forceinline__ void tile_queue(int64_t n, unsigned long long* __restrict__ queue, int grab, const Body& body)
{
    const int64_t ntiles = (n + 31) / 32;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long t0 = 0;
        if (lane == 0) t0 = atomicAdd(queue, (unsigned long long)grab);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if ((int64_t)t0 >= ntiles) break;
        const int64_t t1 = min((int64_t)t0 + grab, ntiles);
        for (int64_t tt = (int64_t)t0; tt < t1; ++tt) {
            const int64_t i = (ntiles - 1 - tt) * 32 + lane;
            if (i < n) body(i);
        }
    }
}

// Stage 1: per contact, energy, gradient and local Hessian (one lane each).
// The launch takes the contacts list[0, *nsel) (FP64 path) or list[*nsel, n)
// (FP32 path) of the chunk's order by path and kind (k_path_keys).
template <int PATH>
__global__ void __launch_bounds__(128) k_local(ContactsView cv, const int* __restrict__ E, const int* __restrict__ F,
    const EghDev* __restrict__ dev, const Params* __restrict__ sp, SceneView sv, const unsigned* __restrict__ gslot,
    unsigned long long* __restrict__ queue, int want, int grab, const int* __restrict__ list,
    const int* __restrict__ nsel)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const EghDev d = *dev;
    const LhLayout L(cv);
    const int64_t k = *nsel;
    const int64_t first = PATH == PATH_F64 ? 0 : k, count = PATH == PATH_F64 ? k : n - k;
    tile_queue(count, queue, grab, [&](int64_t t) {
        const int64_t i = list[first + t];
        if (i < L.first[1]) local_one<CT_VV, PATH>(cv, E, F, d, sp, sv, gslot, L, i, i, want);
        else if (i < L.first[2]) local_one<CT_EV, PATH>(cv, E, F, d, sp, sv, gslot, L, i, i - L.first[1], want);
        else if (i < L.first[2] + cv.nee)
            local_one<CT_EE, PATH>(cv, E, F, d, sp, sv, gslot, L, i, i - L.first[2], want);
        else local_one<CT_FV, PATH>(cv, E, F, d, sp, sv, gslot, L, i, i - L.first[2] - cv.nee, want);
    });
}

// Stage 1's order (every mode).  Per contact of the chunk a 4-bit key: its
// kind on the FP64 path (VV, EV, each edge-edge distance type, FV) or
// KEY_F32; nsel counts the FP64 contacts.  A radix sort on the keys puts the
// FP64 contacts first, grouped by kind, so that the FP64 distance code's
// branches (one inlined copy per distance type) agree across a warp's lanes.
constexpr unsigned char KEY_F32 = 15;
__global__ void __launch_bounds__(256) k_path_keys(ContactsView cv, const int* __restrict__ E,
    const int* __restrict__ F, const EghDev* __restrict__ dev, const Params* __restrict__ sp, SceneView sv,
    unsigned char* __restrict__ key, int* __restrict__ nsel)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool f64 = false;
    if (i < n) {
        Local c;
        load_contact(cv, E, F, i, c);
        const Params P = sp[sv.of(c.vid[0])];
        V3 x[4];
        gather(dev->V, c, x);
        f64 = !fp32_local_contact(P, c, x);
        key[i] = !f64 ? KEY_F32
                      : (unsigned char)(c.type == CT_VV ? 0 : c.type == CT_EV ? 1 : c.type == CT_EE ? 2 + c.dtype : 11);
    }
    const unsigned b = __ballot_sync(0xffffffffu, f64);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(nsel, __popc(b));
}

__global__ void k_iota(int* __restrict__ a, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (int)i;
}

// Flag on the projection method: the df64 pass leaves every projection to
// the FP64 fix-up pass (a testing switch, ipcg_testing_defer_df64_psd).
constexpr int PSD_DEFER = 16;

// A 3x3-block scatter of one projected local Hessian: entry (r, c), r <= c,
// and its mirror to the block-sorted slots of the contact's contributions.
template <int NS> struct BlockScatter {
    double* __restrict__ slab;
    unsigned slot[NS * NS];
    __device__ __forceinline__ BlockScatter(double* s, const unsigned* __restrict__ pm) : slab(s)
    {
#pragma unroll
        for (int q = 0; q < NS * NS; ++q) slot[q] = pm[q];
    }
    __device__ __forceinline__ void operator()(int rr, int cc, double v) const
    {
        const int a = rr / 3, k = rr % 3, b = cc / 3, l = cc % 3;
        slab[9 * (int64_t)slot[a * NS + b] + 3 * k + l] = v;
        if (cc != rr) slab[9 * (int64_t)slot[b * NS + a] + 3 * l + k] = v;
    }
};

__device__ __forceinline__ void record_failure(long long* __restrict__ fail, const SlabAcc& acc, int N, int64_t i,
    int chunk)
{
    // the first failure records which contact and whether its matrix had
    // non-finite entries
    if (atomicCAS((unsigned long long*)fail, 0ull, 1ull) == 0ull) {
        int bad = 0;
        for (int k = 0; k < N * N; ++k) bad += isfinite(acc(k)) ? 0 : 1;
        fail[1] = i;
        fail[2] = chunk;
        fail[3] = bad;
    }
}

// Stage 2 for one contact with an NS-vertex stencil: the PSD projection of
// its local Hessian (its negative eigenpairs in arithmetic T), applied while
// each 3x3 block is written to its block-sorted slot.  If the eigensolver
// does not converge, FP64 records the failure (and writes the unprojected
// matrix); df64 writes nothing and appends the contact to the list that the
// FP64 fix-up pass (k_psd_fixup) projects after it.
template <int NS, class T>
__device__ __forceinline__ void psd_one(const EghDev& d, const unsigned* __restrict__ pm, int64_t i, int64_t r,
    int64_t off, int64_t stride, int psd, int chunk, unsigned long long* __restrict__ nfix,
    long long* __restrict__ fail)
{
    const Slab hs { d.lh + off, stride };
    const SlabAcc acc { hs, r };
    double wv[MAXPAIRS * 12], sl[MAXPAIRS], sigma = 1.0;
    int np = 0;
    const int method = psd & 15;
    const bool defer = PsdReal<T>::rescale && (psd & PSD_DEFER); // testing: every projection to the fix-up
    const bool project = method != IPCG_PSD_NONE && d.pflag[i];
    // The lanes that arrive here together solve in step (wm) and all of them
    // meet again before the scatter (all): each makes the same __syncwarp
    // calls, and none returns before the last of them.
    const unsigned all = __activemask();
    const unsigned wm = __ballot_sync(all, project && !defer);
    bool unsolved = project && defer;
    if (project && !defer && !psd_pairs<T>(NS, acc, method, wv, sl, np, sigma, wm)) unsolved = true;
    // the lanes that go on to the scatter (df64 hands unsolved contacts to the
    // fix-up pass instead)
    const unsigned keep = all & ~__ballot_sync(all, unsolved && PsdReal<T>::rescale);
    if (unsolved) {
        if constexpr (PsdReal<T>::rescale) {
            d.fixlist[atomicAdd(nfix, 1ull)] = i; // at most one entry per contact
            return;
        } else {
            record_failure(fail, acc, 3 * NS, i, chunk);
            np = 0;
            sigma = 1.0;
        }
    }
    psd_apply(NS, acc, wv, sl, np, sigma, BlockScatter<NS>(d.slab, pm), keep);
}

// Stage 2: PSD projection and scatter of every local Hessian to the
// block-sorted slots (T = double: FP64; T = dd: df64 eigenpairs).
template <class T>
__global__ void __launch_bounds__(128) k_psd_scatter(ContactsView cv, const EghDev* __restrict__ dev,
    const unsigned* __restrict__ perm, unsigned long long* __restrict__ queue, int psd, int grab, int chunk,
    long long* __restrict__ fail)
{
    const int64_t n = cv.nvv + cv.nev + cv.nee + cv.nfv;
    const EghDev d = *dev;
    const LhLayout L(cv);
    unsigned long long* nfix = queue + 1;
    tile_queue(n, queue, grab, [&](int64_t i) {
        const int64_t off = contrib_offset(cv, i);
        if (i < L.first[1]) psd_one<2, T>(d, perm + off, i, i, L.off[0], L.stride[0], psd, chunk, nfix, fail);
        else if (i < L.first[2])
            psd_one<3, T>(d, perm + off, i, i - L.first[1], L.off[1], L.stride[1], psd, chunk, nfix, fail);
        else psd_one<4, T>(d, perm + off, i, i - L.first[2], L.off[2], L.stride[2], psd, chunk, nfix, fail);
    });
}

// The df64 pass's fix-up: the contacts it listed, projected in FP64 (a fixed
// grid striding over the list, whose length is read on the device).
constexpr int FIX_BLOCKS = 152, FIX_THREADS = 32;
__global__ void __launch_bounds__(FIX_THREADS) k_psd_fixup(ContactsView cv, const EghDev* __restrict__ dev,
    const unsigned* __restrict__ perm, const unsigned long long* __restrict__ nfix, int psd, int chunk,
    long long* __restrict__ fail)
{
    const EghDev d = *dev;
    const LhLayout L(cv);
    const int64_t cnt = (int64_t)*nfix;
    psd &= 15;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = d.fixlist[j];
        const int64_t off = contrib_offset(cv, i);
        if (i < L.first[1]) psd_one<2, double>(d, perm + off, i, i, L.off[0], L.stride[0], psd, chunk, nullptr, fail);
        else if (i < L.first[2])
            psd_one<3, double>(d, perm + off, i, i - L.first[1], L.off[1], L.stride[1], psd, chunk, nullptr, fail);
        else psd_one<4, double>(d, perm + off, i, i - L.first[2], L.off[2], L.stride[2], psd, chunk, nullptr, fail);
    }
}

// CSR values: each stored value sums its block's contiguous run of slots.
__global__ void k_hess_reduce(int64_t nb, const unsigned* __restrict__ run_start, const int64_t* __restrict__ vbase,
    const int* __restrict__ vnbr, const EghDev* __restrict__ dev)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 9 * nb) return;
    const double* __restrict__ slab = dev->slab;
    const int64_t q = t / 9;
    const int kl = (int)(t % 9), k = kl / 3, l = kl % 3;
    double sum = 0;
    const unsigned s1 = run_start[q + 1];
    unsigned s = run_start[q];
    // four loads in flight, summed in slot order
    for (; s + 4 <= s1; s += 4) {
        const double a = slab[9 * (int64_t)s + kl], b = slab[9 * (int64_t)(s + 1) + kl];
        const double c = slab[9 * (int64_t)(s + 2) + kl], e = slab[9 * (int64_t)(s + 3) + kl];
        sum += a;
        sum += b;
        sum += c;
        sum += e;
    }
    for (; s < s1; ++s) sum += slab[9 * (int64_t)s + kl];
    dev->val[vbase[q] + 3 * (int64_t)k * vnbr[q] + l] = sum;
}

// Gradient entries of vertex rows [r0, r0 + nr): contiguous runs of slots.
__global__ void k_grad_reduce(int64_t r0, int64_t nr, const unsigned* __restrict__ gstart,
    const EghDev* __restrict__ dev)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * nr) return;
    const double* __restrict__ gslab = dev->gslab;
    const int64_t v = t / 3;
    const int k = (int)(t % 3);
    double sum = 0;
    for (unsigned s = gstart[v]; s < gstart[v + 1]; ++s) sum += gslab[3 * (int64_t)s + k];
    dev->grad[3 * (r0 + v) + k] = sum;
}

// Per-scene energies in two fixed-order stages (deterministic): parts of at
// most EPART contacts, each inside one scene's range of one contact type,
// summed by one block each (a fixed reduction tree); then each scene's parts
// in order.  Parts are numbered across the chunks, scene by scene.
constexpr int ER_BLOCK = 256;
constexpr int64_t EPART = 8192;
__global__ void __launch_bounds__(ER_BLOCK) k_energy_parts(const int64_t* __restrict__ parts, int64_t p0,
    const EghDev* __restrict__ dev)
{
    const int64_t p = p0 + blockIdx.x;
    const int64_t b = parts[2 * p], e = parts[2 * p + 1];
    const double* __restrict__ eslab = dev->eslab;
    double s = 0;
    for (int64_t i = b + threadIdx.x; i < e; i += ER_BLOCK) s += eslab[i];
    typedef cub::BlockReduce<double, ER_BLOCK> BR;
    __shared__ typename BR::TempStorage tmp;
    const double tot = BR(tmp).Sum(s);
    if (threadIdx.x == 0) dev->epart[p] = tot;
}
__global__ void k_energy_scenes(const int64_t* __restrict__ pstart, int64_t ns, const EghDev* __restrict__ dev,
    double* __restrict__ energy)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    const double* __restrict__ ep = dev->epart;
    double s = 0;
    for (int64_t p = pstart[k]; p < pstart[k + 1]; ++p) s += ep[p];
    energy[k] = s;
}

int device_index()
{
    int d = 0;
    IPCG_CUDA(cudaGetDevice(&d));
    return d < 0 || d >= 64 ? 0 : d;
}

// Work per chunk: runs of whole scenes with at most `budget` contacts.
std::vector<EChunk> plan(const ipcg_collisions* cs, ipcg_mesh* m, const ContactsView& cv, int64_t budget,
    std::vector<int64_t>& ranges /* 4 x (ns + 1) */)
{
    const int64_t ns = m->n_scenes;
    const int S = (int)(ns + 1);
    ranges.assign(4 * S, 0);
    const int64_t counts[4] = { cs->nvv, cs->nev, cs->nee, cs->nfv };
    if (ns == 1) {
        for (int t = 0; t < 4; ++t) ranges[t * S + 1] = counts[t];
    } else {
        DBuf<int64_t> d_out;
        d_out.reserve(4 * S);
        IPCG_LAUNCH("k_p_scene_ranges", m->stream, k_p_scene_ranges<<<grid_for(4 * S, 256), 256, 0, m->stream>>>(cv,
            m->scene_offs.p, S, d_out.p));
        IPCG_CUDA(cudaMemcpyAsync(ranges.data(), d_out.p, sizeof(int64_t) * 4 * S, cudaMemcpyDeviceToHost, m->stream));
        IPCG_CUDA(cudaStreamSynchronize(m->stream));
    }
    auto count = [&](int64_t a, int64_t b) {
        int64_t c = 0;
        for (int t = 0; t < 4; ++t) c += ranges[t * S + b] - ranges[t * S + a];
        return c;
    };
    std::vector<EChunk> out;
    int64_t k0 = 0;
    while (k0 < ns) {
        int64_t k1 = k0 + 1;
        while (k1 < ns && count(k0, k1 + 1) <= budget) ++k1;
        EChunk c {};
        for (int t = 0; t < 4; ++t) {
            c.lo[t] = ranges[t * S + k0];
            c.hi[t] = ranges[t * S + k1];
        }
        c.r0 = m->h_voff[k0];
        c.r1 = m->h_voff[k1];
        c.k0 = k0;
        c.k1 = k1;
        c.n = count(k0, k1);
        c.ncontrib = 4 * (c.hi[0] - c.lo[0]) + 9 * (c.hi[1] - c.lo[1]) + 16 * ((c.hi[2] - c.lo[2]) + (c.hi[3] - c.lo[3]));
        out.push_back(c);
        k0 = k1;
    }
    return out;
}

void build_pattern(const ipcg_collisions* cs, ipcg_mesh* m, EghCache& C)
{
    cudaStream_t s = m->stream;
    const ContactsView cv = full_view(cs);
    const int64_t budget = g_hess_chunk_contacts.load();
    std::vector<int64_t> ranges;
    C.chunks = plan(cs, m, cv, budget, ranges);
    const int64_t ns = m->n_scenes, S = ns + 1, nV = m->nV;
    int64_t tot_contrib = 0, tot_n = 0;
    C.max_contrib = C.max_n = 0;
    for (EChunk& c : C.chunks) {
        if (c.ncontrib >= (int64_t)INT32_MAX) throw Error(IPCG_ERR_INVALID, "too many Hessian contributions in one chunk");
        c.perm_off = tot_contrib;
        c.gslot_off = 4 * tot_n;
        tot_contrib += c.ncontrib;
        tot_n += c.n;
        C.max_contrib = std::max(C.max_contrib, c.ncontrib);
        C.max_n = std::max(C.max_n, c.n);
    }
    C.n = tot_n;
    // energy parts: each scene's chunk-local range of each type in pieces of
    // at most EPART contacts
    std::vector<int64_t> parts, pstart(ns + 1, 0);
    for (EChunk& c : C.chunks) {
        const int64_t base[4] = { 0, c.hi[0] - c.lo[0], (c.hi[0] - c.lo[0]) + (c.hi[1] - c.lo[1]),
            (c.hi[0] - c.lo[0]) + (c.hi[1] - c.lo[1]) + (c.hi[2] - c.lo[2]) };
        c.ep0 = (int64_t)parts.size() / 2;
        for (int64_t k = c.k0; k < c.k1; ++k) {
            pstart[k] = (int64_t)parts.size() / 2;
            for (int t = 0; t < 4; ++t) {
                const int64_t b = base[t] + ranges[t * S + k] - c.lo[t];
                const int64_t e = base[t] + ranges[t * S + k + 1] - c.lo[t];
                for (int64_t q = b; q < e; q += EPART) {
                    parts.push_back(q);
                    parts.push_back(std::min(e, q + EPART));
                }
            }
        }
        c.nep = (int64_t)parts.size() / 2 - c.ep0;
    }
    pstart[ns] = (int64_t)parts.size() / 2;
    C.nparts = pstart[ns];
    C.eparts.reserve(parts.size() + 2);
    C.epstart.reserve(ns + 1);
    if (!parts.empty())
        IPCG_CUDA(cudaMemcpyAsync(C.eparts.p, parts.data(), sizeof(int64_t) * parts.size(), cudaMemcpyHostToDevice, s));
    IPCG_CUDA(cudaMemcpyAsync(C.epstart.p, pstart.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice, s));
    C.perm.reserve(tot_contrib + 1);
    C.gslot.reserve(4 * tot_n + 1);
    // work space of the sort
    const int64_t mk = C.max_contrib + 1;
    m->keys_a.reserve(mk);
    m->keys_b.reserve(mk);
    m->ivals_a.reserve(nV + 2);
    m->ivals_b.reserve(3 * mk + 3);
    m->counters.reserve(16);
    int* d_nb = m->counters.p + 13;
    auto pat = std::make_shared<EghPattern>();
    pat->row_ptr.reserve(3 * nV + 1);
    // the chunks' block counts are only known after their sorts: columns and
    // block arrays grow as chunks finish (the row pointers are sized already)
    int64_t B0 = 0, rs_tot = 0, gs_tot = 0;
    DBuf<int> tmp_start, diag_len, diag_q, gstart_i;
    C.max_gs = 0;
    for (size_t ci = 0; ci < C.chunks.size(); ++ci) {
        EChunk& ch = C.chunks[ci];
        const ContactsView cc = chunk_view(cv, ch);
        const int64_t nk = ch.ncontrib;
        const int64_t nr = ch.r1 - ch.r0;
        ch.B0 = B0;
        ch.rs_off = rs_tot;
        ch.gs_off = gs_tot;
        int nb = 0;
        int* ids_in = m->ivals_b.p;
        int* sorted_ids = m->ivals_b.p + (nk + 1);
        int* run_len = m->ivals_b.p + 2 * (nk + 1);
        if (ch.n > 0) {
            IPCG_LAUNCH("k_p_keys", s, k_p_keys<<<grid_for(ch.n, 128), 128, 0, s>>>(cc, m->E.p, m->F.p, m->keys_a.p,
                ids_in));
            sort_pairs_u64(m, s, m->keys_a.p, m->keys_b.p, ids_in, sorted_ids, (int)nk, 32 + bits_for(nV + 1));
            rle_u64(m, s, m->keys_b.p, m->keys_a.p, run_len, d_nb, (int)nk);
            IPCG_CUDA(cudaMemcpyAsync(m->h_counters.p, d_nb, sizeof(int), cudaMemcpyDeviceToHost, s));
            IPCG_CUDA(cudaStreamSynchronize(s));
            nb = m->h_counters.p[0];
        }
        ch.nb = nb;
        // blocks of this chunk: run starts, CSR columns, positions
        C.run_start.grow_keep(rs_tot + nb + 2, rs_tot, s);
        C.vbase.grow_keep(B0 + nb + 1, B0, s);
        C.vnbr.grow_keep(B0 + nb + 1, B0, s);
        pat->col.grow_keep(9 * (B0 + nb) + 1, 9 * B0, s);
        tmp_start.reserve(nb + 1);
        diag_len.reserve(nr + 2);
        diag_q.reserve(nr + 2);
        gstart_i.reserve(nr + 2);
        int* bptr = m->ivals_a.p;
        IPCG_CUDA(cudaMemsetAsync(diag_len.p, 0, sizeof(int) * (nr + 1), s));
        if (nb > 0) {
            exclusive_sum_i32(m, s, run_len, tmp_start.p, nb);
            IPCG_LAUNCH("k_p_runs", s, k_p_runs<<<grid_for(nb + 1, 256), 256, 0, s>>>(tmp_start.p, nb, (unsigned)nk,
                C.run_start.p + rs_tot));
            IPCG_LAUNCH("k_p_perm", s, k_p_perm<<<grid_for(nk, 256), 256, 0, s>>>(sorted_ids, nk,
                C.perm.p + ch.perm_off));
        }
        IPCG_LAUNCH("k_p_bptr", s, k_p_bptr<<<grid_for(nr + 1, 256), 256, 0, s>>>(m->keys_a.p, nb, ch.r0, (int)nr,
            bptr));
        IPCG_LAUNCH("k_p_rows", s, k_p_rows<<<grid_for(nr + 1, 256), 256, 0, s>>>(bptr, ch.r0, (int)nr, B0,
            pat->row_ptr.p));
        if (nb > 0)
            IPCG_LAUNCH("k_p_blocks", s, k_p_blocks<<<grid_for(nb, 256), 256, 0, s>>>(m->keys_a.p, nb, bptr, ch.r0, B0,
                run_len, pat->col.p, C.vbase.p + B0, C.vnbr.p + B0, diag_len.p, diag_q.p));
        // gradient slots: vertex starts from the diagonal runs
        exclusive_sum_i32(m, s, diag_len.p, gstart_i.p, (int)(nr + 1));
        C.gstart.grow_keep(gs_tot + nr + 2, gs_tot, s);
        IPCG_CUDA(cudaMemcpyAsync(C.gstart.p + gs_tot, gstart_i.p, sizeof(int) * (nr + 1), cudaMemcpyDeviceToDevice, s));
        if (ch.n > 0)
            IPCG_LAUNCH("k_p_gslot", s, k_p_gslot<<<grid_for(ch.n, 128), 128, 0, s>>>(cc, m->E.p, m->F.p, ch.r0,
                C.perm.p + ch.perm_off, C.run_start.p + rs_tot, diag_q.p, gstart_i.p, C.gslot.p + ch.gslot_off));
        int gtot = 0;
        IPCG_CUDA(cudaMemcpyAsync(&gtot, gstart_i.p + nr, sizeof(int), cudaMemcpyDeviceToHost, s));
        IPCG_CUDA(cudaStreamSynchronize(s));
        C.max_gs = std::max<int64_t>(C.max_gs, gtot);
        rs_tot += nb + 1;
        gs_tot += nr + 1;
        B0 += nb;
    }
    C.nb = B0;
    C.pattern = pat;
    C.energy.reserve(ns + 1);
    C.queue.reserve(4 * C.chunks.size() + 1);
    C.iota.reserve(C.max_n + 1);
    C.list.reserve(C.max_n + 1);
    C.path.reserve(C.max_n + 1);
    C.pkey.reserve(C.max_n + 1);
    C.nsel.reserve(1);
    if (C.max_n > 0) {
        IPCG_LAUNCH("k_iota", s, k_iota<<<grid_for(C.max_n, 256), 256, 0, s>>>(C.iota.p, C.max_n));
        C.part_bytes = 0;
        IPCG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, C.part_bytes, C.path.p, C.pkey.p, C.iota.p, C.list.p,
            (int)C.max_n, 0, 4, s));
        C.part_tmp.reserve(C.part_bytes + 16);
    }
    C.fail.reserve(4);
    C.hfail.reserve(4);
    C.dev.reserve(1);
    C.hdev.reserve(1);
    IPCG_CUDA(cudaStreamSynchronize(s));
    C.version = cs->version;
    C.mesh_serial = m->serial;
    C.budget = budget;
    C.valid = true;
    if (C.exec) {
        cudaGraphExecDestroy(C.exec);
        C.exec = nullptr;
    }
    if (C.graph) {
        cudaGraphDestroy(C.graph);
        C.graph = nullptr;
    }
    C.graph_key.clear();
    C.steps = 0;
}

// Launch geometry of a stage for a tuning: a persistent grid of
// blocks_per_sm blocks per SM (at most what fits), never more warps than
// tiles.
// Resident blocks per SM of a kernel at a block size, per device (cached, so
// that launches enqueued while capturing a graph query nothing).
std::mutex g_occ_mu;
std::map<std::tuple<int, const void*, int>, int> g_occ;
template <class K> int occupancy(int dev, K kernel, int threads)
{
    const auto key = std::make_tuple(dev, (const void*)kernel, threads);
    {
        std::lock_guard<std::mutex> lk(g_occ_mu);
        auto it = g_occ.find(key);
        if (it != g_occ.end()) return it->second;
    }
    int occ = 0;
    IPCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, 0));
    std::lock_guard<std::mutex> lk(g_occ_mu);
    g_occ[key] = occ;
    return occ;
}

template <class K> void egh_grid(const EghTuning& t, int64_t n, K kernel, int& blocks, int& threads)
{
    int dev = 0, sms = 1;
    IPCG_CUDA(cudaGetDevice(&dev));
    IPCG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    threads = t.threads;
    const int occ = occupancy(dev, kernel, threads);
    const int64_t need = (n + 31) / 32 * 32 / threads + 1;
    const int64_t per_sm = std::max(1, std::min(t.blocks_per_sm, occ));
    blocks = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * per_sm, need));
}

// Stage 1 of one chunk; q[0], q[1] are its work queues.  The chunk's
// contacts are first ordered by arithmetic path (FP64 first, grouped by kind:
// k_path_keys), so that no warp runs both paths, each path has its own
// register budget and the FP64 path's warps take one distance branch (in the
// all-FP64 mode every contact is on the FP64 path and the order is by kind).
// Returns the kernels launched.
int launch_local(const ContactsView& cc, const ipcg_mesh* m, EghCache& C, const EChunk& ch, const Params* sp,
    const SceneView& sv, unsigned long long* q, int want, const EghTuning& t, cudaStream_t s)
{
    int blocks, threads;
    const unsigned* gs = C.gslot.p + ch.gslot_off;
    IPCG_CUDA(cudaMemsetAsync(C.nsel.p, 0, sizeof(int), s));
    IPCG_LAUNCH("k_path_keys", s, k_path_keys<<<grid_for(ch.n, 256), 256, 0, s>>>(cc, m->E.p, m->F.p, C.dev.p, sp,
        sv, C.path.p, C.nsel.p));
    size_t bytes = C.part_bytes;
    IPCG_LAUNCH("cub_path_sort", s, IPCG_CUDA(cub::DeviceRadixSort::SortPairs(C.part_tmp.p, bytes, C.path.p, C.pkey.p,
        C.iota.p, C.list.p, (int)ch.n, 0, 4, s)));
    egh_grid(t, ch.n, k_local<PATH_F64>, blocks, threads);
    IPCG_LAUNCH("k_local", s, k_local<PATH_F64><<<blocks, threads, 0, s>>>(cc, m->E.p, m->F.p, C.dev.p, sp, sv, gs,
        q, want, t.tiles_per_grab, C.list.p, C.nsel.p));
    egh_grid(t, ch.n, k_local<PATH_F32>, blocks, threads);
    IPCG_LAUNCH("k_local_f32", s, k_local<PATH_F32><<<blocks, threads, 0, s>>>(cc, m->E.p, m->F.p, C.dev.p, sp, sv,
        gs, q + 1, want, t.tiles_per_grab, C.list.p, C.nsel.p));
    return 4;
}

// Stage 2 of one chunk; q[0] is its work queue, q[1] the fix-up count.
// Returns the kernels launched.
int launch_psd(const ContactsView& cc, EghCache& C, const EChunk& ch, int ci, unsigned long long* q, int psd,
    bool df64, const EghTuning& t, cudaStream_t s)
{
    int blocks, threads;
    if (df64) {
        egh_grid(t, ch.n, k_psd_scatter<dd>, blocks, threads);
        const int pm = psd | (g_defer_df64.load() ? PSD_DEFER : 0);
        IPCG_LAUNCH("k_psd_scatter", s, k_psd_scatter<dd><<<blocks, threads, 0, s>>>(cc, C.dev.p,
            C.perm.p + ch.perm_off, q, pm, t.tiles_per_grab, ci, C.fail.p));
        if (psd == IPCG_PSD_NONE) return 1;
        IPCG_LAUNCH("k_psd_fixup", s, k_psd_fixup<<<FIX_BLOCKS, FIX_THREADS, 0, s>>>(cc, C.dev.p,
            C.perm.p + ch.perm_off, q + 1, psd, ci, C.fail.p));
        return 2;
    }
    egh_grid(t, ch.n, k_psd_scatter<double>, blocks, threads);
    IPCG_LAUNCH("k_psd_scatter", s, k_psd_scatter<double><<<blocks, threads, 0, s>>>(cc, C.dev.p,
        C.perm.p + ch.perm_off, q, psd, t.tiles_per_grab, ci, C.fail.p));
    return 1;
}

// Enqueue the launches of one step on the mesh stream (also while capturing).
int enqueue_step(const ipcg_collisions* cs, ipcg_mesh* m, EghCache& C, const Params* sp, int psd, bool df64, int want,
    const EghTuning* tune)
{
    cudaStream_t s = m->stream;
    const ContactsView cv = full_view(cs);
    const SceneView sv = scene_view(m);
    int kernels = 0;
    IPCG_CUDA(cudaMemsetAsync(C.queue.p, 0, sizeof(unsigned long long) * 4 * C.chunks.size(), s));
    for (size_t ci = 0; ci < C.chunks.size(); ++ci) {
        const EChunk& ch = C.chunks[ci];
        const ContactsView cc = chunk_view(cv, ch);
        if (ch.n > 0) {
            kernels += launch_local(cc, m, C, ch, sp, sv, C.queue.p + 4 * ci, want, tune[0], s);
            kernels += launch_psd(cc, C, ch, (int)ci, C.queue.p + 4 * ci + 2, psd, df64, tune[1], s);
        }
        if (ch.nb > 0) {
            IPCG_LAUNCH("k_hess_reduce", s, k_hess_reduce<<<grid_for(9 * ch.nb, 256), 256, 0, s>>>(ch.nb,
                C.run_start.p + ch.rs_off, C.vbase.p + ch.B0, C.vnbr.p + ch.B0, C.dev.p));
            ++kernels;
        }
        const int64_t nr = ch.r1 - ch.r0;
        if ((want & WANT_G) && nr > 0) {
            IPCG_LAUNCH("k_grad_reduce", s, k_grad_reduce<<<grid_for(3 * nr, 256), 256, 0, s>>>(ch.r0, nr,
                C.gstart.p + ch.gs_off, C.dev.p));
            ++kernels;
        }
        if ((want & WANT_E) && ch.nep > 0) {
            IPCG_LAUNCH("k_energy_parts", s, k_energy_parts<<<(int)ch.nep, ER_BLOCK, 0, s>>>(C.eparts.p, ch.ep0,
                C.dev.p));
            ++kernels;
        }
    }
    if (want & WANT_E) {
        const int64_t ns = m->n_scenes;
        IPCG_LAUNCH("k_energy_scenes", s, k_energy_scenes<<<grid_for(ns, 256), 256, 0, s>>>(C.epstart.p, ns, C.dev.p,
            C.energy.p));
        ++kernels;
    }
    return kernels;
}

Params* upload_params_egh(const ipcg_collisions* cs, ipcg_mesh* m, const BarrierArgs& a)
{
    const int ns = (int)m->n_scenes;
    std::vector<Params> hp(ns);
    for (int k = 0; k < ns; ++k) {
        const double dh = a.scene_dhat ? a.scene_dhat[k] : a.dhat;
        const double kap = a.scene_kappa ? a.scene_kappa[k] : a.kappa;
        const double dm = (k < (int)cs->scene_dmin.size()) ? cs->scene_dmin[k] : cs->dmin;
        const double xh = (2 * dm + dh) * dh;
        hp[k] = Params { kap, dm * dm, xh, a.physical ? dh / barrier_units(a.kind, xh) : 1.0, a.psd, a.mixed, a.kind,
            a.fp32_local };
    }
    const size_t pbytes = sizeof(Params) * ns;
    const unsigned char* hb = reinterpret_cast<const unsigned char*>(hp.data());
    if (m->params_host.size() != pbytes || memcmp(m->params_host.data(), hb, pbytes) != 0) {
        m->params_buf.reserve(pbytes);
        IPCG_CUDA(cudaMemcpyAsync(m->params_buf.p, hb, pbytes, cudaMemcpyHostToDevice, m->stream));
        m->params_host.assign(hb, hb + pbytes);
    }
    return reinterpret_cast<Params*>(m->params_buf.p);
}

// The step's scratch for the largest chunk from the library's pool (freed in
// stream order after the step): local Hessians and their block-sorted
// copies, projection flags, gradient slots, energies and energy parts.
struct Scratch {
    double *slab = nullptr, *gslab = nullptr, *eslab = nullptr, *lh = nullptr, *epart = nullptr;
    unsigned char* pflag = nullptr;
    int64_t* fixlist = nullptr;
    cudaStream_t s = nullptr;
    template <class P> void take(P*& p, size_t count)
    {
        IPCG_CUDA(cudaMallocFromPoolAsync((void**)&p, sizeof(P) * count, device_pool(), s));
    }
    void alloc(const EghCache& C, cudaStream_t st)
    {
        s = st;
        take(slab, 9 * C.max_contrib + 9);
        take(lh, 9 * C.max_contrib + 9);
        take(gslab, 3 * C.max_gs + 3);
        take(eslab, C.max_n + 1);
        take(pflag, C.max_n + 1);
        take(epart, C.nparts + 1);
        take(fixlist, C.max_n + 1);
    }
    EghDev dev(const double* V, double* grad, double* val) const
    {
        return EghDev { V, grad, val, slab, gslab, eslab, lh, pflag, epart, fixlist };
    }
    ~Scratch()
    {
        for (void* p : { (void*)slab, (void*)gslab, (void*)eslab, (void*)lh, (void*)epart, (void*)pflag,
                 (void*)fixlist })
            if (p) cudaFreeAsync(p, s);
    }
};

EghCache& cache_for(const ipcg_collisions* cs, ipcg_mesh* m)
{
    auto* c = const_cast<ipcg_collisions*>(cs);
    if (!c->egh) c->egh = std::make_shared<EghCache>();
    EghCache& C = *c->egh;
    if (!C.valid || C.version != cs->version || C.mesh_serial != m->serial
        || C.budget != g_hess_chunk_contacts.load())
        build_pattern(cs, m, C);
    return C;
}

} // namespace

// The message of a projection failure: which contact, from the record.
static std::string psd_failure(const EghCache& C)
{
    const long long* r = C.hfail.p;
    std::string msg = "unable to project matrix onto positive semi-definite cone";
    if (r[2] < 0 || r[2] >= (long long)C.chunks.size()) return msg;
    const EChunk& ch = C.chunks[r[2]];
    int64_t i = r[1];
    static const char* names[4] = { "vertex-vertex", "edge-vertex", "edge-edge", "face-vertex" };
    for (int t = 0; t < 4; ++t) {
        const int64_t cnt = ch.hi[t] - ch.lo[t];
        if (i < cnt) {
            msg += " (the eigensolver did not converge on " + std::string(names[t]) + " collision "
                + std::to_string(ch.lo[t] + i) + "; its local Hessian has " + std::to_string(r[3])
                + " non-finite entries)";
            break;
        }
        i -= cnt;
    }
    return msg;
}

void egh_defer_df64(bool on) { g_defer_df64.store(on ? 1 : 0); }

// ---- the device's FP64 FMA rate ----
// Each thread runs FP64_CHAINS independent chains of fused multiply-adds
// (independent so that the pipe, not the latency, is the limit), on a grid
// of 64 warps per SM; the sum of the chains is written so that nothing is
// removed as dead code.
constexpr int FP64_CHAINS = 8, FP64_ITERS = 4096;
__global__ void __launch_bounds__(256) k_fp64_rate(double a, double b, double* __restrict__ out)
{
    double x[FP64_CHAINS];
#pragma unroll
    for (int k = 0; k < FP64_CHAINS; ++k) x[k] = threadIdx.x + k;
    for (int it = 0; it < FP64_ITERS; ++it)
#pragma unroll
        for (int k = 0; k < FP64_CHAINS; ++k) x[k] = fma(x[k], a, b);
    double sum = 0;
#pragma unroll
    for (int k = 0; k < FP64_CHAINS; ++k) sum += x[k];
    if (sum == 12345.678) out[0] = sum;
}

double fp64_fma_rate()
{
    int dev = 0, sms = 1;
    IPCG_CUDA(cudaGetDevice(&dev));
    IPCG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DBuf<double> out;
    out.reserve(1);
    cudaEvent_t e0, e1;
    IPCG_CUDA(cudaEventCreate(&e0));
    IPCG_CUDA(cudaEventCreate(&e1));
    const int blocks = sms * 8, threads = 256;
    float best = 1e30f;
    for (int r = 0; r < 4; ++r) {
        IPCG_CUDA(cudaEventRecord(e0, 0));
        k_fp64_rate<<<blocks, threads>>>(0.999999, 1e-7, out.p);
        IPCG_CHECK_LAUNCH();
        IPCG_CUDA(cudaEventRecord(e1, 0));
        IPCG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        IPCG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (r > 0) best = std::min(best, ms); // the first run warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * FP64_CHAINS * FP64_ITERS * (double)blocks * threads;
    return flops / (best * 1e-3) / 1e12;
}

EghTuning egh_tuning(int stage)
{
    const int d = device_index();
    if (stage < 0 || stage > 2) stage = 1;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tune_set[d][stage] ? g_tune[d][stage] : EghTuning {};
}

void egh_set_tuning(int stage, const EghTuning& t)
{
    if (stage < 0 || stage > 2)
        throw Error(IPCG_ERR_INVALID, "tuning stage is 0 (local Hessians), 1 (FP64 projection) or 2 (df64 projection)");
    if (!(t.threads == 32 || t.threads == 64 || t.threads == 128) || t.blocks_per_sm < 1 || t.blocks_per_sm > 64
        || t.tiles_per_grab < 1 || t.tiles_per_grab > 64)
        throw Error(IPCG_ERR_INVALID, "tuning out of range: threads 32/64/128, blocks_per_sm 1-64, tiles_per_grab 1-64");
    const int d = device_index();
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[d][stage] = t;
    g_tune_set[d][stage] = true;
}

bool barrier_egh(const ipcg_collisions* cs, ipcg_mesh* m, const double* V, const BarrierArgs& a, double* energy_host,
    double* grad_dev, ipcg_csr* hess)
{
    if (!hess || a.shape) return false;
    if (m->n_scenes > 1 && !cs->sorted) return false;
    cudaStream_t s = m->stream;
    const int64_t n = cs->size();
    const int ns = (int)m->n_scenes;
    hess->rows = 3 * m->nV;
    hess->stream = s;
    if (n == 0) {
        // nothing to evaluate: zero energies and gradient, an empty matrix
        if (energy_host) std::fill(energy_host, energy_host + ns, 0.0);
        if (grad_dev) IPCG_CUDA(cudaMemsetAsync(grad_dev, 0, sizeof(double) * 3 * m->nV, s));
        hess->row_ptr.reserve(3 * m->nV + 1, s);
        IPCG_CUDA(cudaMemsetAsync(hess->row_ptr.p, 0, sizeof(int64_t) * (3 * m->nV + 1), s));
        hess->nnz = 0;
        IPCG_CUDA(cudaStreamSynchronize(s));
        return true;
    }
    EghCache& C = cache_for(cs, m);
    const Params* sp = upload_params_egh(cs, m, a);
    const int want = WANT_H | (energy_host ? WANT_E : 0) | (grad_dev ? WANT_G : 0);
    // outputs: the values are the call's own; the pattern is shared
    const int64_t nnz = 9 * C.nb;
    hess->val.reserve(nnz + 1, s);
    hess->nnz = nnz;
    hess->pattern = C.pattern;
    hess->row_ptr_shared = C.pattern->row_ptr.p;
    hess->col_shared = C.pattern->col.p;
    Scratch scr;
    scr.alloc(C, s);
    C.hdev.p[0] = scr.dev(V, grad_dev, hess->val.p);
    IPCG_CUDA(cudaMemcpyAsync(C.dev.p, C.hdev.p, sizeof(EghDev), cudaMemcpyHostToDevice, s));
    IPCG_CUDA(cudaMemsetAsync(C.fail.p, 0, sizeof(long long) * 4, s));
    const bool df64 = a.df64_psd != 0;
    const EghTuning tune[2] = { egh_tuning(0), egh_tuning(df64 ? 2 : 1) };
    // A pattern's first step runs as plain launches: a set that is rebuilt
    // before its next Hessian (a Newton loop whose collision set changes,
    // a served request) would pay the capture and instantiation for nothing.
    // From its second step on, the step is captured once and replayed.
    const bool direct = prof::enabled() || C.steps == 0;
    ++C.steps;
    if (direct) {
        // (per-kernel timing also needs the launches themselves)
        enqueue_step(cs, m, C, sp, a.psd, df64, want, tune);
    } else {
        char key[200];
        snprintf(key, sizeof(key), "%p|%d|%d%d|%d|%d,%d,%d|%d,%d,%d", (const void*)sp, a.psd, (int)df64,
            g_defer_df64.load(), want,
            tune[0].threads, tune[0].blocks_per_sm, tune[0].tiles_per_grab, tune[1].threads, tune[1].blocks_per_sm,
            tune[1].tiles_per_grab);
        if (!C.exec || C.graph_key != key) {
            if (C.exec) cudaGraphExecDestroy(C.exec);
            if (C.graph) cudaGraphDestroy(C.graph);
            C.exec = nullptr;
            C.graph = nullptr;
            {
                // launch shapes (and their occupancy queries) before capturing
                int b, t;
                egh_grid(tune[0], C.max_n, k_local<PATH_F64>, b, t);
                egh_grid(tune[0], C.max_n, k_local<PATH_F32>, b, t);
                if (df64) egh_grid(tune[1], C.max_n, k_psd_scatter<dd>, b, t);
                else egh_grid(tune[1], C.max_n, k_psd_scatter<double>, b, t);
            }
            IPCG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            int kernels = 0;
            try {
                kernels = enqueue_step(cs, m, C, sp, a.psd, df64, want, tune);
            } catch (...) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(s, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            IPCG_CUDA(cudaStreamEndCapture(s, &C.graph));
            IPCG_CUDA(cudaGraphInstantiate(&C.exec, C.graph, 0));
            C.graph_key = key;
            C.graph_kernels = kernels;
        }
        IPCG_CUDA(cudaGraphLaunch(C.exec, s));
        prof::count_graph(C.graph_kernels);
    }
    if (energy_host)
        IPCG_CUDA(cudaMemcpyAsync(energy_host, C.energy.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaMemcpyAsync(C.hfail.p, C.fail.p, sizeof(long long) * 4, cudaMemcpyDeviceToHost, s));
    IPCG_CUDA(cudaStreamSynchronize(s));
    if (C.hfail.p[0]) throw Error(IPCG_ERR_CUDA, psd_failure(C));
    return true;
}


std::string egh_autotune(const ipcg_collisions* cs, ipcg_mesh* m, const double* V, const BarrierArgs& a)
{
    cudaStream_t s = m->stream;
    if (cs->size() == 0) throw Error(IPCG_ERR_INVALID, "autotuning needs a non-empty collision set");
    if (m->n_scenes > 1 && !cs->sorted) throw Error(IPCG_ERR_INVALID, "autotuning needs a built collision set");
    EghCache& C = cache_for(cs, m);
    const Params* sp = upload_params_egh(cs, m, a);
    const bool df64 = a.df64_psd != 0;
    // the largest chunk is the workload
    size_t big = 0;
    for (size_t i = 0; i < C.chunks.size(); ++i)
        if (C.chunks[i].n > C.chunks[big].n) big = i;
    const EChunk& ch = C.chunks[big];
    const ContactsView cc = chunk_view(full_view(cs), ch);
    const SceneView sv = scene_view(m);
    Scratch scr;
    scr.alloc(C, s);
    C.hdev.p[0] = scr.dev(V, nullptr, nullptr);
    IPCG_CUDA(cudaMemcpyAsync(C.dev.p, C.hdev.p, sizeof(EghDev), cudaMemcpyHostToDevice, s));
    IPCG_CUDA(cudaMemsetAsync(C.fail.p, 0, sizeof(long long) * 4, s));
    int dev = 0;
    IPCG_CUDA(cudaGetDevice(&dev));
    cudaEvent_t e0, e1;
    IPCG_CUDA(cudaEventCreate(&e0));
    IPCG_CUDA(cudaEventCreate(&e1));
    const int want = WANT_H | WANT_G | WANT_E;
    // one stage, one tuning: a warm-up run and a timed one
    auto time_stage = [&](int stage, const EghTuning& t) {
        float ms = 0;
        for (int r = 0; r < 2; ++r) {
            IPCG_CUDA(cudaMemsetAsync(C.queue.p, 0, sizeof(unsigned long long) * 4, s));
            IPCG_CUDA(cudaEventRecord(e0, s));
            if (stage == 0) launch_local(cc, m, C, ch, sp, sv, C.queue.p, want, t, s);
            else launch_psd(cc, C, ch, (int)big, C.queue.p + 2, a.psd, df64, t, s);
            prof::count();
            IPCG_CUDA(cudaEventRecord(e1, s));
            IPCG_CUDA(cudaEventSynchronize(e1));
            IPCG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        }
        return ms;
    };
    std::string rep = "{\"workload_contacts\": " + std::to_string(ch.n) + ", \"device\": " + std::to_string(dev);
    const char* names[2] = { "local", "psd" };
    for (int stage = 0; stage < 2; ++stage) {
        const int slot = stage == 0 ? 0 : (df64 ? 2 : 1);
        // stage 1 projects the local Hessians stage 0 left in the scratch
        EghTuning best {};
        float best_ms = 1e30f;
        rep += std::string(", \"") + names[stage] + "\": {\"candidates\": [";
        bool first = true;
        auto consider = [&](const EghTuning& t) {
            const float ms = time_stage(stage, t);
            char buf[160];
            snprintf(buf, sizeof(buf), "%s{\"threads\": %d, \"blocks_per_sm\": %d, \"tiles_per_grab\": %d, \"ms\": %.4f}",
                first ? "" : ", ", t.threads, t.blocks_per_sm, t.tiles_per_grab, ms);
            rep += buf;
            first = false;
            if (ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        };
        for (int threads : { 32, 64, 128 }) {
            const int occ = stage == 0 ? occupancy(dev, k_local<PATH_F64>, threads)
                : (df64 ? occupancy(dev, k_psd_scatter<dd>, threads) : occupancy(dev, k_psd_scatter<double>, threads));
            for (int bps : { 1, 2, 4, 8, 16, 32 }) {
                if (bps > occ) break;
                consider(EghTuning { threads, bps, 1 });
            }
            if (occ > 0 && occ < 32 && (occ & (occ - 1)) != 0) consider(EghTuning { threads, occ, 1 });
        }
        consider(EghTuning { best.threads, best.blocks_per_sm, 4 });
        egh_set_tuning(slot, best);
        char buf[220];
        snprintf(buf, sizeof(buf), "], \"stage\": %d, \"chosen\": {\"threads\": %d, \"blocks_per_sm\": %d, "
            "\"tiles_per_grab\": %d, \"ms\": %.4f}}", slot, best.threads, best.blocks_per_sm, best.tiles_per_grab,
            best_ms);
        rep += buf;
        if (stage == 0) time_stage(0, best); // leave stage 0's output for stage 1
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    rep += "}";
    return rep;
}

} // namespace ipcg
