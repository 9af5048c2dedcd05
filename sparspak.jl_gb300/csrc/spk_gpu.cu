// C-ABI of the GB300 supernodal LU engine: structure analysis, the level
// schedule and the entry points of include/spk_gpu.h.  The kernels live in
// spk_kernels.cuh; their storage layout is described there.

#include "../../include/spk_gpu.h"
#include "spk_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <new>
#include <type_traits>
#include <string>
#include <vector>

using spk::ll;
typedef int64_t i64;

namespace {

struct LaunchRec {
    i64 off = 0;      // into sched_ids
    i64 poff = 0;     // into sched_prefix
    int count = 0;
    int tiles = 0;
    double flops = 0.0;   // algorithmic flops of the launch (solves: per right-hand side)
    double words = 0.0;   // algorithmic factor entries read or written (times sizeof(T) = bytes)
    int bw = 1;           // widest block in the launch (sizes dynamic shared memory)
};

// A captured launch sequence and the accounting of one replay.
struct GraphRec {
    cudaGraphExec_t exec = nullptr;
    double flops[SPK_K_COUNT] = {};
    double bytes[SPK_K_COUNT] = {};
    int64_t launches[SPK_K_COUNT] = {};
};

// One CUDA event pair per timed launch.
struct Timed {
    cudaEvent_t a, b;
    int kind;
};

// Launches of one elimination-tree level: per block step t the block LU,
// panel and trailing kernels; then the Schur complements; for the solves
// the forward block steps, and backward the U12 product and block steps.
struct LevelPlan {
    LaunchRec schur, schur_tc, bwdu;
    // schur_tc in two parts: the tiles whose targets the next level factors
    // (near) and the others (far, beside the next level's factorisation)
    LaunchRec schur_tc_near, schur_tc_far;
    // btrail_tc0: tile 0 of each packed front's trailing update (it holds the
    // next block's diagonal block); btrail_tc: its tiles 1..
    std::vector<LaunchRec> blu, bpanel, btrail, btrail_tc0, btrail_tc, fwd, bwd;
    // bpanel split in two parts: the near tiles (the first 128 rows below the
    // block and columns right of it, which tile 0 reads) and the far ones
    std::vector<LaunchRec> bpanel_near, bpanel_far;
    std::vector<char> blu_pc;   // every piece of the step's blocks is at most 32 columns (k_block_lu_pc)
    // Solves: fronts with many blocks by one cluster launch each direction
    // (front_big, one tile per front), the others by block steps
    // (fwd_small / bwd_small); the transposed solves use fwd / bwd.
    // fronts factored whole by k_leaf_factor (a warp each), by width class;
    // leaf_q: the leaf queue's fronts of this level, for when the queue is off
    LaunchRec leaf_factor[spk::LF_CLASSES], leaf_q[spk::LF_CLASSES];
    LaunchRec front_big, front_l21;   // front_l21: tiles of k_fwd_l21 for the front_big fronts
    // Root fronts of more than spk::FC_CHUNK blocks: solved in chunks of
    // consecutive blocks (a cluster launch each, on a pseudo front - the
    // front's storage, the chunk's blocks), linked by k_front_gemv.
    struct SolveChunk {
        int front, lo, hi;   // front-local columns [lo, hi)
        LaunchRec rec;       // the cluster launch on the pseudo front
    };
    std::vector<SolveChunk> chunks;
    // Small fronts (one block of at most 32 columns, m <= spk::LEAF_M) by
    // k_solve_leaf, a warp per front; bwdu_small: U12 products of the others.
    LaunchRec front_leaf[spk::LF_CLASSES], bwdu_small;   // front_leaf by width class (k_solve_leaf<W>)
    std::vector<LaunchRec> fwd_small, bwd_small;
};

// FP32 fronts whose rank updates go to the tensor cores (k_tc_update,
// 128 x 128 tiles from packed panels): a Schur complement of at least
// tc_schur_m rows, or more than one block with at least tc_trail_rows rows
// below the first (spk_handle; defaults below, SPK_OPT_TC_* to change).
constexpr int TC_SCHUR_M = 96, TC_TRAIL_ROWS = 128;
// Polls of a bounded device wait (the leaf queue's dependency waits) before
// it gives up and records a timeout.
constexpr long long WAIT_BUDGET = 1 << 20;

// Block partition and schedule for one precision (block width BlockMax<T>).
struct Plan {
    bool built = false;
    bool sym = false;                     // the symmetric (SPD) form's tiles
    int schur_nh = 1;                     // 128-column tiles per tensor-core Schur tile (wide: 2)
    int bmax = 0, bwmax = 1;
    std::vector<int> blk_c0, blk_c1, blk_p0, blk_np;
    std::vector<ll> blk_inv2;
    std::vector<ll> blk_lpack, blk_upack;  // byte offsets of the packed panels (-1: front not packed)
    ll pack_size = 0;
    std::vector<int> blk_front;
    std::vector<int> inv_ids;             // k_block_inv entries grouped by level group, then line width (32, 64, 128)
    int inv_off[2][4] = {};               // group g, class c: inv_ids[inv_off[g][c] .. inv_off[g][c+1])
    int inv_sub[2][spk::LF_CLASSES + 1] = {};   // class 0 split by width class (k_block_inv_small<W>)
    int inv_split = 0;                    // group 0: blocks of fronts below this level (final before it starts)
    ll inv2_size = 0;
    std::vector<int> block0, nblocks;     // per front
    // per front: update-row tiles holding the rows that fronts of the next
    // level own (spk::schur_part_tile; DFront::sq)
    std::vector<int> schur_q;
    // pseudo fronts of the chunked solves (LevelPlan::SolveChunk): front,
    // first block, blocks; device front ids from the number of fronts on
    std::vector<int> pf_front, pf_b0, pf_nb;
    std::vector<LevelPlan> levels;
    std::vector<int> sched_ids, sched_prefix;
    // The leaf queue (k_leaf_queue): the fronts factored whole (by a warp)
    // whose descendants all are, in level order.  Per queue position: the
    // front, and its parent when that is in the queue (else -1); per front:
    // the number of its children in the queue.
    std::vector<int> q_order, q_parent, q_deps;
    int nq = 0, q_grid = 1;
    double q_flops = 0.0, q_words = 0.0;
    int *d_q_order = nullptr, *d_q_parent = nullptr, *d_q_deps0 = nullptr, *d_q_deps = nullptr, *d_q_next = nullptr;
    spk::DFront* d_fronts = nullptr;
    int *d_blk_c0 = nullptr, *d_blk_c1 = nullptr, *d_blk_p0 = nullptr, *d_blk_np = nullptr;
    ll* d_blk_inv2 = nullptr;
    ll *d_blk_lpack = nullptr, *d_blk_upack = nullptr;
    int* d_blk_front = nullptr;
    int* d_inv_ids = nullptr;
    int *d_sched_ids = nullptr, *d_sched_prefix = nullptr;
    spk::Sched sched{};
};

struct HFront {
    i64 f;
    int nf, m, piece0, npieces, parent, level;
    i64 loff, uoff, rows_off, runid_off;
    int run0, nruns;
};

template <typename T>
struct Storage {
    T* d = nullptr;
    T* inv2 = nullptr;      // whole-block forward / backward operators
    unsigned char* pack = nullptr;   // packed panels of the tensor-core fronts (FP32)
    bool loaded = false;    // values assembled since the last factor
    bool factored = false;
};

}  // namespace

struct spk_handle {
    i64 n = 0, nsuper = 0;
    std::vector<int> xs;            // 0-based first column per supernode [nsuper+1]
    std::vector<int> lindx0;        // 0-based rows
    std::vector<i64> xlindx0;       // 0-based offsets [nsuper+1]
    std::vector<i64> xlnz0, xunz0;  // reference layout, 0-based offsets [n+1]
    std::vector<HFront> fronts;
    std::vector<int> col_front;     // column -> front
    std::vector<int> col_snode;     // column -> supernode (0-based)
    std::vector<int> rows;          // concatenated R_F
    std::vector<int> runid, run_tgt, run_start;
    std::vector<ll> run_rel;
    std::vector<int> rel;
    Plan plan[4];                   // [0] FP64, [1] FP32, [2] FP64 SPD form, [3] FP32 SPD form
    int nlevels = 0;
    i64 fsize = 0;
    int wmax = 1;             // widest supernode
    double amalgamation = 0.1;  // allowed relative padding of a front
    double lu_flops = 0.0;

    // device structure shared by both plans
    int *d_xs = nullptr, *d_rows = nullptr, *d_runid = nullptr, *d_run_tgt = nullptr, *d_run_start = nullptr,
        *d_rel = nullptr;
    ll* d_run_rel = nullptr;
    int* d_ipiv = nullptr;
    int* d_bmap = nullptr;     // row sources of each block's interchanges (k_block_lu -> panels)
    int* d_info = nullptr;

    // pattern and values
    bool have_pattern = false, have_values = false;
    i64 nnz = 0;
    std::vector<int> rperm0, rinvp0;
    ll* d_slot = nullptr;
    double* d_aval = nullptr;
    double* d_acsr = nullptr;   // A's values in CSR order (the residuals)
    int *d_rowptr = nullptr, *d_col = nullptr;
    ll* d_src = nullptr;
    int *d_ccolptr = nullptr, *d_crow = nullptr, *d_ccol = nullptr;   // A's pattern in CSC order (0-based)
    int *d_rperm = nullptr, *d_rinvp = nullptr;

    // factor storage per precision, [0] LU form, [1] SPD (symmetric) form
    Storage<double> s64[2];
    Storage<float> s32[2];
    Storage<float> s16[2];   // SPK_BF16S: float factor, BF16 packed panels
    int fmode = 0;        // which float form the float paths use: 0 SPK_FP32, 1 SPK_BF16S
    int sym = 0;          // which factorisation the paths use: 0 LU, 1 SPD form (SPK_SPD)

    // solve work space (sized for MAXRHS right-hand sides)
    void *d_wb = nullptr, *d_wy = nullptr, *d_wx = nullptr;   // factor precision
    double *d_rhs = nullptr, *d_x = nullptr, *d_r = nullptr;  // FP64, n*cap
    double* d_sums = nullptr;
    i64 rhs_cap = 0;
    // GMRES-IR work space (spk_refine_ex): bases V (GM_M + 1 blocks) and
    // Z = M^-1 V (GM_M blocks) of n x GM_MAXRHS, w, and the small coefficients
    double *gm_V = nullptr, *gm_Z = nullptr, *gm_w = nullptr, *gm_c = nullptr;

    cudaStream_t own = nullptr, stream = nullptr;
    // Look-ahead of the factorisation: the bulk of a block step's tensor-core
    // trailing update runs on `side` while the next block LU runs on the
    // launch stream (evP: panels done; evB: trailing update done).
    cudaStream_t side = nullptr;
    // The solve operators of the lower levels' blocks (k_block_inv) run on
    // side2 while the last levels are factored (evP2: those levels done; evI:
    // the operators done).
    cudaStream_t side2 = nullptr;
    cudaEvent_t evP2 = nullptr, evI = nullptr;
    // The far tiles of a level's tensor-core Schur complements run on side3
    // beside the next level (evS: the level done; evF[l % 2]: level l's far
    // tiles done, awaited before level l + 2 starts).
    cudaStream_t side3 = nullptr;
    cudaEvent_t evS = nullptr, evF[2] = {nullptr, nullptr};
    bool fc16 = false;   // front solves by clusters of 16 CTAs
    cudaEvent_t evP = nullptr, evB = nullptr;
    int device = -1;
    int nsm = 1;                 // SMs of the device (grid of the persistent kernels)
    // options (spk_set_option)
    int leaf_queue = 0;                    // SPK_OPT_LEAF_QUEUE (off: slower on the measured workloads)
    long long wait_budget = WAIT_BUDGET;   // SPK_OPT_WAIT_BUDGET
    int stall_test = -1;                   // SPK_OPT_STALL_TEST
    int tc_schur_m = TC_SCHUR_M, tc_trail_rows = TC_TRAIL_ROWS;
    int tc_wide = 1;                       // SPK_OPT_TC_WIDE: Schur tiles of 128 x 256
    int lu_pieces = 0;                     // SPK_OPT_LU_PIECES: block LU by pieces (slower on GB300, see header)
    int fc_minb = spk::FC_MINB;            // SPK_OPT_SOLVE_CLUSTER_MINB: blocks of a front for the cluster solve
    int panel_split = 1;                   // SPK_OPT_PANEL_SPLIT: near / far panel tiles on two streams
    int schur_split = 1;                   // SPK_OPT_SCHUR_SPLIT: far Schur tiles beside the next level
    int schur_far_sms = 0;                 // SPK_OPT_SCHUR_FAR_SMS: their CTAs (0: seven eighths of the SMs)
    int solve_chunk = 1;                   // SPK_OPT_SOLVE_CHUNK: root fronts solved in chunks of blocks
    std::string err;

    // launch accounting and optional per-class event timing
    unsigned prof_mask = 0;
    std::vector<Timed> pending;
    std::vector<cudaEvent_t> event_pool;
    double prof_ms[SPK_K_COUNT] = {};
    double prof_flops[SPK_K_COUNT] = {};
    double prof_bytes[SPK_K_COUNT] = {};
    int64_t prof_launches[SPK_K_COUNT] = {};

    // captured sequences: factor per precision, solve per precision x right-hand sides
    bool use_graphs = true;
    // [0] FP64, [1] FP32, [2] BF16S; + 3 for the SPD form
    GraphRec g_factor[6];
    // fused factorisation + first solve (spk_factor_refine), per right-hand
    // sides: the factorisation with the lower levels' forward substitution,
    // and the rest of that solve
    GraphRec g_factor_fs[6][spk::MAXRHS + 1];
    GraphRec g_fs_tail[6][spk::MAXRHS + 1];
    GraphRec g_solve[6][spk::MAXRHS + 1];
    GraphRec g_tsolve[6][spk::MAXRHS + 1];   // transposed solves
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
static thread_local std::string g_create_err;

static int set_err(spk_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

#define CU(h, call)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return set_err(h, e_ == cudaErrorMemoryAllocation ? SPK_ENOMEM : SPK_ECUDA,               \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                       \
    } while (0)

template <typename T>
static int upload(spk_handle* h, T** dst, const std::vector<T>& src) {
    size_t bytes = sizeof(T) * std::max<size_t>(src.size(), 1);
    CU(h, cudaMalloc((void**)dst, bytes));
    if (!src.empty()) CU(h, cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
    return SPK_OK;
}

static spk::Launch launch_of(const Plan& P, const LaunchRec& r) {
    spk::Launch L;
    L.front_ids = P.d_sched_ids + r.off;
    L.prefix = P.d_sched_prefix + r.poff;
    L.count = r.count;
    return L;
}

template <typename T>
static constexpr int prec_index() { return std::is_same<T, float>::value ? 1 : 0; }

// Slot of the captured graphs: FP64, FP32 or BF16S (the float form
// selected), LU or SPD form.
template <typename T>
static int graph_index(const spk_handle* h) { return (std::is_same<T, float>::value ? 1 + h->fmode : 0) + 3 * h->sym; }

// Plan of the selected form: block partition of precision T, LU or SPD tiles.
template <typename T>
static int plan_index(const spk_handle* h) { return prec_index<T>() + 2 * h->sym; }

static cudaEvent_t take_event(spk_handle* h) {
    if (!h->event_pool.empty()) {
        cudaEvent_t e = h->event_pool.back();
        h->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Bracket one kernel launch: count it, add its algorithmic work, and when
// its class is selected by spk_profile record an event pair around it.
struct LaunchScope {
    spk_handle* h;
    int kind;
    Timed t{};
    bool timed;
    LaunchScope(spk_handle* h_, int kind_, double flops, double bytes) : h(h_), kind(kind_) {
        h->prof_launches[kind] += 1;
        h->prof_flops[kind] += flops;
        h->prof_bytes[kind] += bytes;
        timed = (h->prof_mask >> kind) & 1u;
        if (timed) {
            t.a = take_event(h);
            t.b = take_event(h);
            t.kind = kind;
            cudaEventRecord(t.a, h->stream);
        }
    }
    ~LaunchScope() {
        if (timed) {
            cudaEventRecord(t.b, h->stream);
            h->pending.push_back(t);
        }
    }
};

static void collect_events(spk_handle* h) {
    for (Timed& t : h->pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(t.b) == cudaSuccess && cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess)
            h->prof_ms[t.kind] += ms;
        h->event_pool.push_back(t.a);
        h->event_pool.push_back(t.b);
    }
    h->pending.clear();
}

static void drop_graph(GraphRec& g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = GraphRec();
}

static void drop_solve_graphs(spk_handle* h) {
    for (int p = 0; p < 6; ++p)
        for (int r = 0; r <= spk::MAXRHS; ++r) {
            drop_graph(h->g_solve[p][r]);
            drop_graph(h->g_tsolve[p][r]);
            drop_graph(h->g_factor_fs[p][r]);
            drop_graph(h->g_fs_tail[p][r]);
        }
}

// Every captured factorisation (plain and fused with a solve).
static void drop_factor_graphs(spk_handle* h) {
    for (GraphRec& g : h->g_factor) drop_graph(g);
    for (int p = 0; p < 6; ++p)
        for (int r = 0; r <= spk::MAXRHS; ++r) {
            drop_graph(h->g_factor_fs[p][r]);
            drop_graph(h->g_fs_tail[p][r]);
        }
}

// Run `body` (which issues launches on h->stream) through a CUDA graph: the
// first call captures it on the handle's own stream, every call replays it
// on h->stream.  With event timing requested the launches go out eagerly.
template <typename Body>
static int via_graph(spk_handle* h, GraphRec& g, Body body) {
    if (h->prof_mask != 0 || !h->use_graphs) return body();
    if (!g.exec) {
        double f0[SPK_K_COUNT], b0[SPK_K_COUNT];
        int64_t l0[SPK_K_COUNT];
        for (int k = 0; k < SPK_K_COUNT; ++k) { f0[k] = h->prof_flops[k]; b0[k] = h->prof_bytes[k]; l0[k] = h->prof_launches[k]; }
        cudaStream_t user = h->stream;
        h->stream = h->own;
        cudaError_t e = cudaStreamBeginCapture(h->own, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            h->stream = user;
            return set_err(h, SPK_ECUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
        }
        int rc = body();
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(h->own, &graph);
        h->stream = user;
        if (rc != SPK_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return set_err(h, SPK_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            g.exec = nullptr;
            return set_err(h, SPK_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
        for (int k = 0; k < SPK_K_COUNT; ++k) {
            g.flops[k] = h->prof_flops[k] - f0[k];
            g.bytes[k] = h->prof_bytes[k] - b0[k];
            g.launches[k] = h->prof_launches[k] - l0[k];
            h->prof_flops[k] = f0[k];
            h->prof_bytes[k] = b0[k];
            h->prof_launches[k] = l0[k];
        }
    }
    CU(h, cudaGraphLaunch(g.exec, h->stream));
    for (int k = 0; k < SPK_K_COUNT; ++k) {
        h->prof_flops[k] += g.flops[k];
        h->prof_bytes[k] += g.bytes[k];
        h->prof_launches[k] += g.launches[k];
    }
    return SPK_OK;
}

// ---------------------------------------------------------------------------
// structure analysis
// ---------------------------------------------------------------------------
static int analyse(spk_handle* h, const int64_t* xsuper, const int64_t* snode, const int64_t* xlindx,
                   const int64_t* lindx, const int64_t* xlnz, const int64_t* xunz, int base) {
    const i64 n = h->n, ns = h->nsuper;
    h->xs.resize(ns + 1);
    for (i64 s = 0; s <= ns; ++s) h->xs[s] = (int)(xsuper[s] - base);
    if (h->xs[0] != 0 || h->xs[ns] != n) return set_err(h, SPK_ESTRUCT, "xsuper does not span 1..n");
    for (i64 s = 0; s < ns; ++s) {
        int w = h->xs[s + 1] - h->xs[s];
        if (w <= 0) return set_err(h, SPK_ESTRUCT, "xsuper is not increasing");
        if (w > spk::MAXW) return set_err(h, SPK_EARG, "supernodes wider than 64 columns are not supported");
        h->wmax = std::max(h->wmax, w);
    }
    h->col_snode.resize(n);
    for (i64 j = 0; j < n; ++j) {
        i64 s = snode[j] - base;
        if (s < 0 || s >= ns || j < h->xs[s] || j >= h->xs[s + 1]) return set_err(h, SPK_ESTRUCT, "snode inconsistent with xsuper");
        h->col_snode[j] = (int)s;
    }
    h->xlindx0.resize(ns + 1);
    for (i64 s = 0; s <= ns; ++s) h->xlindx0[s] = xlindx[s] - base;
    const i64 nsub = h->xlindx0[ns];
    h->lindx0.resize(nsub);
    for (i64 k = 0; k < nsub; ++k) {
        i64 r = lindx[k] - base;
        if (r < 0 || r >= n) return set_err(h, SPK_ESTRUCT, "lindx entry out of range");
        h->lindx0[k] = (int)r;
    }
    h->xlnz0.resize(n + 1);
    h->xunz0.resize(n + 1);
    for (i64 j = 0; j <= n; ++j) { h->xlnz0[j] = xlnz[j] - base; h->xunz0[j] = xunz[j] - base; }
    // each supernode: rows start with its own columns, ascending; rectangular storage
    for (i64 s = 0; s < ns; ++s) {
        int f = h->xs[s], w = h->xs[s + 1] - f;
        i64 a = h->xlindx0[s], len = h->xlindx0[s + 1] - a;
        if (len < w) return set_err(h, SPK_ESTRUCT, "supernode has fewer rows than columns");
        for (int k = 0; k < w; ++k)
            if (h->lindx0[a + k] != f + k) return set_err(h, SPK_ESTRUCT, "lindx does not start with the supernode's columns");
        for (i64 k = 1; k < len; ++k)
            if (h->lindx0[a + k] <= h->lindx0[a + k - 1]) return set_err(h, SPK_ESTRUCT, "lindx not ascending");
        for (int k = 0; k < w; ++k) {
            if (h->xlnz0[f + k + 1] - h->xlnz0[f + k] != len) return set_err(h, SPK_ESTRUCT, "xlnz inconsistent with lindx");
            if (h->xunz0[f + k + 1] - h->xunz0[f + k] != len - w) return set_err(h, SPK_ESTRUCT, "xunz inconsistent with lindx");
        }
    }
    // LU flop count from column counts (every column of a supernode of length
    // len at offset k has c = len - k nonzeros in L)
    double fl = 0.0;
    for (i64 s = 0; s < ns; ++s) {
        int w = h->xs[s + 1] - h->xs[s];
        i64 len = h->xlindx0[s + 1] - h->xlindx0[s];
        for (int k = 0; k < w; ++k) {
            double c1 = (double)(len - k - 1);
            fl += c1 + 2.0 * c1 * c1;
        }
    }
    h->lu_flops = fl;

    // Fronts: maximal paths s, s+1, ..., e of the supernodal elimination tree
    // (each supernode's parent is the next one) whose dense front storage
    // (nf^2 + 2 nf m entries) exceeds the pieces' exact lnz+unz storage by at
    // most the amalgamation allowance.  Exact fundamental chains need no
    // padding; padded positions are structural zeros and stay exactly zero
    // (every product that reaches them has a structurally zero factor).
    h->col_front.assign(n, -1);
    h->fronts.clear();
    auto exact_entries = [&](i64 t) {
        double w = h->xs[t + 1] - h->xs[t], len = (double)(h->xlindx0[t + 1] - h->xlindx0[t]);
        return 2.0 * len * w - w * w;
    };
    for (i64 s = 0; s < ns;) {
        i64 e = s;
        double exact = exact_entries(s);
        while (e + 1 < ns) {
            int w = h->xs[e + 1] - h->xs[e];
            i64 a = h->xlindx0[e], len = h->xlindx0[e + 1] - a;
            if (len == w || h->lindx0[a + w] != h->xs[e + 1]) break;   // parent is not the next supernode
            double ex2 = exact + exact_entries(e + 1);
            double nf = h->xs[e + 2] - h->xs[s];
            double m = (double)(h->xlindx0[e + 2] - h->xlindx0[e + 1]) - (h->xs[e + 2] - h->xs[e + 1]);
            if (nf * nf + 2.0 * nf * m > (1.0 + h->amalgamation) * ex2) break;
            exact = ex2;
            ++e;
        }
        HFront F{};
        F.f = h->xs[s];
        F.nf = h->xs[e + 1] - h->xs[s];
        i64 a = h->xlindx0[e], len = h->xlindx0[e + 1] - a;
        int we = h->xs[e + 1] - h->xs[e];
        F.m = (int)(len - we);
        F.piece0 = (int)s;
        F.npieces = (int)(e - s + 1);
        F.rows_off = (i64)h->rows.size();
        for (i64 k = 0; k < F.m; ++k) h->rows.push_back(h->lindx0[a + we + k]);
        F.parent = -1;
        F.level = 0;
        int id = (int)h->fronts.size();
        for (i64 j = F.f; j < F.f + F.nf; ++j) h->col_front[j] = id;
        h->fronts.push_back(F);
        s = e + 1;
    }
    const int nfr = (int)h->fronts.size();
    i64 off = 0;
    for (int i = 0; i < nfr; ++i) {
        HFront& F = h->fronts[i];
        if (F.m > 0) {
            int r0 = h->rows[F.rows_off];
            if (r0 < F.f + F.nf) return set_err(h, SPK_ESTRUCT, "off-diagonal row inside its own front");
            F.parent = h->col_front[r0];
        }
        F.loff = off;
        off += (i64)(F.nf + F.m) * F.nf;
        F.uoff = off;
        off += (i64)F.m * F.nf;
    }
    h->fsize = off;
    for (int i = 0; i < nfr; ++i)
        if (h->fronts[i].parent >= 0)
            h->fronts[h->fronts[i].parent].level =
                std::max(h->fronts[h->fronts[i].parent].level, h->fronts[i].level + 1);
    h->nlevels = 0;
    for (int i = 0; i < nfr; ++i) h->nlevels = std::max(h->nlevels, h->fronts[i].level + 1);
    // runs and relative positions
    h->runid.clear();
    h->run_tgt.clear();
    h->run_start.clear();
    h->run_rel.clear();
    h->rel.clear();
    for (int i = 0; i < nfr; ++i) {
        HFront& F = h->fronts[i];
        F.runid_off = (i64)h->runid.size();
        F.run0 = (int)h->run_tgt.size();
        F.nruns = 0;
        const int* R = h->rows.data() + F.rows_off;
        int x = 0;
        while (x < F.m) {
            int g = h->col_front[R[x]];
            const HFront& G = h->fronts[g];
            int run = (int)h->run_tgt.size();
            h->run_tgt.push_back(g);
            h->run_start.push_back(x);
            h->run_rel.push_back((ll)h->rel.size());
            ++F.nruns;
            const int* RG = h->rows.data() + G.rows_off;
            int q = 0;
            for (int y = x; y < F.m; ++y) {
                int row = R[y];
                int pos;
                if (row < G.f) return set_err(h, SPK_ESTRUCT, "update row precedes its target front");
                if (row < G.f + G.nf) pos = (int)(row - G.f);
                else {
                    while (q < G.m && RG[q] < row) ++q;
                    // absent: the update there is an exact zero (padding of F), skipped
                    pos = (q < G.m && RG[q] == row) ? G.nf + q : -1;
                }
                h->rel.push_back(pos);
            }
            int y = x;
            while (y < F.m && R[y] < G.f + G.nf) { h->runid.push_back(run); ++y; }
            x = y;
        }
    }
    return SPK_OK;
}

static void add_launch(Plan* h, LaunchRec& rec, const std::vector<int>& ids, const std::vector<int>& tiles,
                       const std::vector<double>& flops, const std::vector<double>& words) {
    rec.off = (i64)h->sched_ids.size();
    rec.poff = (i64)h->sched_prefix.size();
    rec.count = 0;
    rec.flops = rec.words = 0.0;
    int acc = 0;
    for (size_t k = 0; k < ids.size(); ++k) {
        if (tiles[k] <= 0) continue;
        h->sched_ids.push_back(ids[k]);
        h->sched_prefix.push_back(acc);
        acc += tiles[k];
        ++rec.count;
        rec.flops += flops[k];
        rec.words += words[k];
    }
    h->sched_prefix.push_back(acc);
    rec.tiles = acc;
}

// Lines per panel tile: the 128-wide FP32 form (a launch with a block wider
// than 64 columns) takes spk::PT_LINES, the others 64.
static int panel_lines(bool fp32, bool wide) { return fp32 && wide ? spk::PT_LINES : 64; }

// Group each front's pieces into blocks of at most `bmax` columns and lay
// out the launches of every level.
static void build_plan(const spk_handle* h, Plan& P, int bmax, bool tc, bool sym) {
    using spk::cdiv;
    P = Plan();
    P.bmax = bmax;
    P.sym = sym;
    P.schur_nh = h->tc_wide ? 2 : 1;
    const int nfr = (int)h->fronts.size();
    P.block0.resize(nfr);
    P.nblocks.resize(nfr);
    for (int i = 0; i < nfr; ++i) {
        const HFront& F = h->fronts[i];
        P.block0[i] = (int)P.blk_c0.size();
        int s = F.piece0;
        const int e = F.piece0 + F.npieces;
        while (s < e) {
            int t = s + 1;
            while (t < e && h->xs[t + 1] - h->xs[s] <= bmax) ++t;
            const int c0 = h->xs[s] - (int)F.f, c1 = h->xs[t] - (int)F.f, bw = c1 - c0;
            P.blk_c0.push_back(c0);
            P.blk_c1.push_back(c1);
            P.blk_p0.push_back(s);
            P.blk_np.push_back(t - s);
            P.blk_inv2.push_back(P.inv2_size);
            P.inv2_size += 2 * (ll)bw * bw;
            P.blk_front.push_back(i);
            P.bwmax = std::max(P.bwmax, bw);
            s = t;
        }
        P.nblocks[i] = (int)P.blk_c0.size() - P.block0[i];
    }
    P.blk_lpack.assign(P.blk_c0.size(), -1);
    P.blk_upack.assign(P.blk_c0.size(), -1);
    if (tc) {
        const ll chunk = spk::umma::PCHUNK;
        for (int i = 0; i < nfr; ++i) {
            const HFront& F = h->fronts[i];
            const int b0 = P.block0[i], nb = P.nblocks[i];
            const bool packed = F.m >= h->tc_schur_m || (nb > 1 && F.nf + F.m - P.blk_c1[b0] >= h->tc_trail_rows);
            if (!packed) continue;
            const int n2 = cdiv(F.m, spk::umma::TM);
            for (int b = b0; b < b0 + nb; ++b) {
                const int n1 = cdiv(F.nf - P.blk_c1[b], spk::umma::TM);
                const ll bytes = (ll)(n1 + n2) * cdiv(P.blk_c1[b] - P.blk_c0[b], spk::umma::KCH) * chunk;
                P.blk_lpack[b] = P.pack_size;
                P.blk_upack[b] = P.pack_size + bytes;
                P.pack_size += 2 * bytes;
            }
        }
    }
    {
        // Solve-operator work: blocks up to 32 wide, one entry per block
        // (k_block_inv_small, by width class); wider ones by line width
        // 64 / 128 (k_block_inv), entries blk * 4 + kind * 2 + tile.
        // Group 0 (fronts below the last two levels) can run beside the top
        // of the factorisation, group 1 after it.
        const int lim[3] = {32, 64, 128};
        P.inv_split = std::max(0, h->nlevels - 2);
        for (int g = 0; g < 2; ++g) {
            for (int c = 0; c < 3; ++c) {
                P.inv_off[g][c] = (int)P.inv_ids.size();
                if (c == 0)
                    for (int wc = 0; wc < spk::LF_CLASSES; ++wc) {
                        P.inv_sub[g][wc] = (int)P.inv_ids.size();
                        for (int b = 0; b < (int)P.blk_c0.size(); ++b) {
                            const int bw = P.blk_c1[b] - P.blk_c0[b];
                            if (bw > 32 || spk::leaf_class(bw) != wc) continue;
                            if ((h->fronts[P.blk_front[b]].level < P.inv_split) != (g == 0)) continue;
                            P.inv_ids.push_back(b);
                        }
                    }
                if (c == 0) P.inv_sub[g][spk::LF_CLASSES] = (int)P.inv_ids.size();
                for (int b = 0; b < (int)P.blk_c0.size(); ++b) {
                    const int bw = P.blk_c1[b] - P.blk_c0[b];
                    if (!(bw <= lim[c] && (c == 0 || bw > lim[c - 1]))) continue;
                    if ((h->fronts[P.blk_front[b]].level < P.inv_split) != (g == 0)) continue;
                    if (c == 0) {
                        continue;   // below, by width class
                    } else {
                        for (int kind = 0; kind < 2; ++kind)
                            for (int tile = 0; tile < spk::cdiv(bw, 64); ++tile)
                                P.inv_ids.push_back(b * 4 + kind * 2 + tile);
                    }
                }
            }
            P.inv_off[g][3] = (int)P.inv_ids.size();
        }
    }
    P.schur_q.assign(nfr, 0);
    for (int i = 0; i < nfr; ++i) {   // the last row a front of the next level owns
        const HFront& F = h->fronts[i];
        int p = 0;
        for (int k = 0; k < F.m; ++k)
            if (h->fronts[h->col_front[h->rows[F.rows_off + k]]].level <= F.level + 1) p = k + 1;
        P.schur_q[i] = cdiv(p, spk::umma::TM);
    }
    const int nlev = h->nlevels;
    std::vector<std::vector<int>> at(nlev);
    for (int i = 0; i < nfr; ++i) at[h->fronts[i].level].push_back(i);
    // the leaf queue: a front factored whole (one block of at most 32
    // columns, m <= LF_M) whose children all are in the queue
    std::vector<char> inq(nfr, 0);
    for (int i = 0; i < nfr; ++i) {
        const HFront& F = h->fronts[i];
        inq[i] = P.nblocks[i] == 1 && F.nf <= 32 && F.m <= spk::LF_M;
    }
    for (int l = 0; l < nlev; ++l)   // children before parents
        for (int i : at[l])
            if (!inq[i] && h->fronts[i].parent >= 0) inq[h->fronts[i].parent] = 0;
    P.q_deps.assign(nfr, 0);
    for (int l = 0; l < nlev; ++l)
        for (int i : at[l])
            if (inq[i]) {
                const int par = h->fronts[i].parent;
                P.q_order.push_back(i);
                P.q_parent.push_back(par >= 0 && inq[par] ? par : -1);
                if (par >= 0 && inq[par]) ++P.q_deps[par];
            }
    P.nq = (int)P.q_order.size();
    P.levels.assign(nlev, LevelPlan());
    for (int l = 0; l < nlev; ++l) {
        LevelPlan& L = P.levels[l];
        const std::vector<int>& ids = at[l];
        const size_t nid = ids.size();
        int maxb = 0;
        for (int id : ids) maxb = std::max(maxb, P.nblocks[id]);
        L.blu.resize(maxb);
        L.blu_pc.assign(maxb, 1);
        L.bpanel.resize(maxb);
        L.bpanel_near.resize(maxb);
        L.bpanel_far.resize(maxb);
        L.btrail.resize(maxb);
        L.btrail_tc0.resize(maxb);
        L.btrail_tc.resize(maxb);
        L.fwd.resize(maxb);
        L.bwd.resize(maxb);
        L.fwd_small.resize(maxb);
        L.bwd_small.resize(maxb);
        std::vector<char> big(nid, 0), leaf(nid, 0);
        {
            std::vector<int> tl1(nid);
            std::vector<double> fl1(nid), wl1(nid);
            for (size_t k = 0; k < nid; ++k) {
                const HFront& F = h->fronts[ids[k]];
                leaf[k] = P.nblocks[ids[k]] == 1 && F.nf <= 32 && F.m <= spk::LEAF_M;
                tl1[k] = leaf[k] ? 1 : 0;
                fl1[k] = 2.0 * F.nf * (double)F.nf + 2.0 * F.nf * (double)F.m;   // per right-hand side and direction
                wl1[k] = F.nf * (double)F.nf + F.nf * (double)F.m;
            }
            for (int c = 0; c < spk::LF_CLASSES; ++c) {
                std::vector<int> tc(nid);
                for (size_t k = 0; k < nid; ++k) tc[k] = tl1[k] && spk::leaf_class(h->fronts[ids[k]].nf) == c ? 1 : 0;
                add_launch(&P, L.front_leaf[c], ids, tc, fl1, wl1);
            }
        }
        {
            std::vector<int> tbig(nid);
            std::vector<double> fbig(nid), wbig(nid);
            for (size_t k = 0; k < nid; ++k) {
                const HFront& F = h->fronts[ids[k]];
                const int nb = P.nblocks[ids[k]];
                big[k] = nb >= h->fc_minb && nb <= spk::FC * spk::FC_OWN;
                const bool chunked = big[k] && h->solve_chunk && F.m == 0 && nb > spk::FC_CHUNK;
                tbig[k] = big[k] && !chunked ? 1 : 0;
                const double nf = F.nf;
                fbig[k] = 2.0 * nf * nf;   // per right-hand side, both directions alike
                wbig[k] = nf * nf;
                if (chunked) {   // equal chunks of at most FC_CHUNK blocks
                    const int nch = cdiv(nb, spk::FC_CHUNK);
                    for (int c = 0, b = 0; c < nch; ++c) {
                        const int len = (nb - b) / (nch - c);
                        LevelPlan::SolveChunk ch;
                        ch.front = ids[k];
                        ch.lo = P.blk_c0[P.block0[ids[k]] + b];
                        ch.hi = P.blk_c1[P.block0[ids[k]] + b + len - 1];
                        const int pid = nfr + (int)P.pf_front.size();
                        P.pf_front.push_back(ids[k]);
                        P.pf_b0.push_back(P.block0[ids[k]] + b);
                        P.pf_nb.push_back(len);
                        const double w = ch.hi - ch.lo;
                        add_launch(&P, ch.rec, std::vector<int>{pid}, std::vector<int>{1},
                                   std::vector<double>{2.0 * w * w}, std::vector<double>{w * w});
                        L.chunks.push_back(ch);
                        b += len;
                    }
                }
            }
            add_launch(&P, L.front_big, ids, tbig, fbig, wbig);
            for (size_t k = 0; k < nid; ++k) {
                const HFront& F = h->fronts[ids[k]];
                tbig[k] = big[k] && F.m > 0 ? cdiv(F.m, spk::L21_ROWS) * cdiv(F.nf, spk::L21_COLS) : 0;
                fbig[k] = 2.0 * F.nf * (double)F.m;
                wbig[k] = F.nf * (double)F.m;
            }
            add_launch(&P, L.front_l21, ids, tbig, fbig, wbig);
        }
        std::vector<char> leafF(nid, 0);   // factored whole by k_leaf_factor or k_leaf_queue
        {
            std::vector<int> tlf(nid), tlq(nid);
            std::vector<double> flf(nid), wlf(nid);
            for (size_t k = 0; k < nid; ++k) {
                const HFront& F = h->fronts[ids[k]];
                leafF[k] = P.nblocks[ids[k]] == 1 && F.nf <= 32 && F.m <= spk::LF_M;
                const double nf = F.nf, m = F.m;
                flf[k] = sym ? 2.0 * nf * nf * nf + nf * nf * m + m * (m + 1.0) * nf
                             : 2.0 * nf * nf * nf + 3.0 * nf * nf * m + 2.0 * m * m * nf;
                wlf[k] = nf * nf + 2.0 * nf * m + m * m;
            }
            for (int c = 0; c < spk::LF_CLASSES; ++c) {
                for (size_t k = 0; k < nid; ++k) {
                    const bool in_class = leafF[k] && spk::leaf_class(h->fronts[ids[k]].nf) == c;
                    tlf[k] = in_class && !inq[ids[k]] ? 1 : 0;
                    tlq[k] = in_class && inq[ids[k]] ? 1 : 0;
                }
                add_launch(&P, L.leaf_factor[c], ids, tlf, flf, wlf);
                add_launch(&P, L.leaf_q[c], ids, tlq, flf, wlf);
                P.q_flops += L.leaf_q[c].flops;
                P.q_words += L.leaf_q[c].words;
            }
        }
        std::vector<char> wide(maxb, 0);   // a block of the step is wider than 64 columns
        for (int id : ids)
            for (int t = 0; t < P.nblocks[id]; ++t)
                if (P.blk_c1[P.block0[id] + t] - P.blk_c0[P.block0[id] + t] > 64) wide[t] = 1;
        for (int t = 0; t < maxb; ++t) {
            std::vector<int> tl(nid), tp(nid), tt(nid), ttc(nid), ttc0(nid), tf(nid), tb(nid);
            std::vector<double> fl(nid), wl(nid), fp(nid), wp(nid), ft(nid), wt(nid), ff(nid), wf(nid), fb(nid), wb(nid);
            for (size_t k = 0; k < nid; ++k) {
                const HFront& F = h->fronts[ids[k]];
                const int nb = P.nblocks[ids[k]];
                if (t >= nb) { tl[k] = tp[k] = tt[k] = ttc[k] = ttc0[k] = tf[k] = tb[k] = 0; continue; }
                const int blk = P.block0[ids[k]] + t;
                const int c0 = P.blk_c0[blk], c1 = P.blk_c1[blk];
                const double bw = c1 - c0;
                const int ld = F.nf + F.m;
                tl[k] = leafF[k] ? 0 : 1;
                fl[k] = 2.0 * bw * bw * bw;
                wl[k] = 2.0 * bw * bw + 2.0 * bw;   // the block read and written once, its pivots and row sources
                const int lpt = panel_lines(tc, wide[t]);
                // the SPD form launches the L-panel tiles only (they also write the U side)
                tp[k] = leafF[k] ? 0 : cdiv(ld - c1, lpt) + (sym ? 0 : cdiv(F.nf - c1, lpt) + cdiv(F.m, lpt));
                const double rowsL = ld - c1, colsU = (double)(F.nf - c1) + F.m;
                fp[k] = bw * bw * rowsL + (sym ? 0.0 : 2.0 * bw * bw * colsU);
                wp[k] = 2.0 * bw * (rowsL + colsU) + 2.0 * bw * bw;
                tt[k] = sym ? spk::lower_tiles(cdiv(ld - c1, spk::TT), cdiv(F.nf - c1, spk::TT))
                            : cdiv(ld - c1, spk::TT) * cdiv(F.nf - c1, spk::TT) + cdiv(F.nf - c1, spk::TT) * cdiv(F.m, spk::TT);
                ttc[k] = ttc0[k] = 0;
                if (P.blk_lpack[blk] >= 0) {   // packed front: 128-tiles, row / column regions split at nf
                    const int n1 = cdiv(F.nf - c1, spk::umma::TM), n2 = cdiv(F.m, spk::umma::TM);
                    const int all = sym ? spk::lower_tiles(n1 + n2, n1) : (n1 + n2) * n1 + n1 * n2;
                    ttc0[k] = all > 0 ? 1 : 0;
                    ttc[k] = all - ttc0[k];
                    tt[k] = 0;
                }
                // SPD form: only the lower part of the front columns (and none of U12)
                const double nfc = F.nf - c1;
                const double area = sym ? nfc * (ld - c1) - 0.5 * nfc * (nfc - 1.0)
                                        : (double)(ld - c1) * (F.nf - c1) + (double)(F.nf - c1) * F.m;
                ft[k] = 2.0 * bw * area;
                wt[k] = 2.0 * area + bw * (rowsL + colsU);
                tf[k] = std::max(1, cdiv(ld - c1, spk::TS)) * cdiv(c1 - c0, spk::SC);
                ff[k] = 2.0 * bw * bw + 2.0 * bw * rowsL;
                wf[k] = bw * bw + bw * rowsL;
                const int rb = P.block0[ids[k]] + nb - 1 - t;
                const int r0 = P.blk_c0[rb];
                const double rbw = P.blk_c1[rb] - r0;
                tb[k] = std::max(1, cdiv(r0, spk::TS)) * cdiv((int)rbw, spk::SC);
                fb[k] = rbw * rbw + 2.0 * rbw * r0;
                wb[k] = 0.5 * rbw * rbw + rbw * r0;
            }
            add_launch(&P, L.blu[t], ids, tl, fl, wl);
            for (size_t k = 0; k < nid; ++k)
                if (tl[k] > 0) {
                    const int blk = P.block0[ids[k]] + t;
                    for (int q = P.blk_p0[blk]; q < P.blk_p0[blk] + P.blk_np[blk]; ++q)
                        if (h->xs[q + 1] - h->xs[q] > 32) L.blu_pc[t] = 0;
                }
            add_launch(&P, L.bpanel[t], ids, tp, fp, wp);
            {   // the near and far parts (spk::panel_tile): two line tiles each side
                std::vector<int> tn(nid), tfar(nid);
                std::vector<double> fn(nid), wn(nid), ffar(nid), wfar(nid);
                for (size_t k = 0; k < nid; ++k) {
                    tn[k] = tfar[k] = 0;
                    fn[k] = wn[k] = ffar[k] = wfar[k] = 0.0;
                    if (tp[k] <= 0) continue;
                    const HFront& F = h->fronts[ids[k]];
                    const int c1 = P.blk_c1[P.block0[ids[k]] + t], lpt = panel_lines(tc, wide[t]);
                    tn[k] = std::min(2, cdiv(F.nf + F.m - c1, lpt)) + (sym ? 0 : std::min(2, cdiv(F.nf - c1, lpt)));
                    tfar[k] = tp[k] - tn[k];
                    const double a = (double)tn[k] / tp[k];
                    fn[k] = fp[k] * a;
                    wn[k] = wp[k] * a;
                    ffar[k] = fp[k] - fn[k];
                    wfar[k] = wp[k] - wn[k];
                }
                add_launch(&P, L.bpanel_near[t], ids, tn, fn, wn);
                add_launch(&P, L.bpanel_far[t], ids, tfar, ffar, wfar);
            }
            int bwl = 1;
            for (size_t k = 0; k < nid; ++k)
                if (t < P.nblocks[ids[k]]) {
                    const int blk = P.block0[ids[k]] + t;
                    bwl = std::max(bwl, P.blk_c1[blk] - P.blk_c0[blk]);
                }
            L.blu[t].bw = L.bpanel[t].bw = bwl;
            add_launch(&P, L.btrail[t], ids, tt, ft, wt);
            {   // flops and words of the tensor-core update split by tiles
                std::vector<double> f0(nid), w0(nid), f1(nid), w1(nid);
                for (size_t k = 0; k < nid; ++k) {
                    const double all = ttc0[k] + ttc[k], a = all > 0 ? ttc0[k] / all : 0.0;
                    f0[k] = ft[k] * a;
                    w0[k] = wt[k] * a;
                    f1[k] = ft[k] - f0[k];
                    w1[k] = wt[k] - w0[k];
                }
                add_launch(&P, L.btrail_tc0[t], ids, ttc0, f0, w0);
                add_launch(&P, L.btrail_tc[t], ids, ttc, f1, w1);
            }
            add_launch(&P, L.fwd[t], ids, tf, ff, wf);
            add_launch(&P, L.bwd[t], ids, tb, fb, wb);
            for (size_t k = 0; k < nid; ++k)
                if (big[k] || leaf[k]) tf[k] = tb[k] = 0;
            add_launch(&P, L.fwd_small[t], ids, tf, ff, wf);
            add_launch(&P, L.bwd_small[t], ids, tb, fb, wb);
        }
        std::vector<int> tsch(nid), tsch_tc(nid), tbu(nid);
        std::vector<double> fs(nid), ws(nid), fu(nid), wu(nid);
        for (size_t k = 0; k < nid; ++k) {
            const HFront& F = h->fronts[ids[k]];
            const int nts = cdiv(F.m, spk::TT), ntc = cdiv(F.m, spk::umma::TM);
            tsch[k] = F.m > 0 && !leafF[k] ? (sym ? spk::lower_tiles(nts, nts) : nts * nts) : 0;
            tsch_tc[k] = 0;
            if (F.m > 0 && P.blk_lpack[P.block0[ids[k]]] >= 0) {
                tsch_tc[k] = sym ? spk::lower_tiles_w(ntc, P.schur_nh) : ntc * cdiv(ntc, P.schur_nh);
                tsch[k] = 0;
            }
            tbu[k] = F.m > 0 ? cdiv(F.nf, spk::U12_ROWS) * cdiv(F.m, spk::U12_COLS) : 0;
            // SPD form: the lower part with the diagonal, m (m + 1) / 2 entries
            fs[k] = (sym ? (double)F.m * (F.m + 1.0) : 2.0 * (double)F.m * F.m) * F.nf;
            ws[k] = 2.0 * (double)F.m * F.nf + 2.0 * (double)F.m * F.m;
            fu[k] = 2.0 * (double)F.m * F.nf;
            wu[k] = (double)F.m * F.nf;
        }
        add_launch(&P, L.schur, ids, tsch, fs, ws);
        add_launch(&P, L.schur_tc, ids, tsch_tc, fs, ws);
        {   // its near and far parts, flops and words by tile share
            std::vector<int> tn(nid), tfar(nid);
            std::vector<double> fn(nid), wn(nid), ffar(nid), wfar(nid);
            for (size_t k = 0; k < nid; ++k) {
                tn[k] = tfar[k] = 0;
                fn[k] = wn[k] = ffar[k] = wfar[k] = 0.0;
                if (tsch_tc[k] <= 0) continue;
                const int ntc = cdiv(h->fronts[ids[k]].m, spk::umma::TM), q = P.schur_q[ids[k]];
                tn[k] = spk::schur_part_count(1, ntc, P.schur_nh, q, sym);
                tfar[k] = spk::schur_part_count(2, ntc, P.schur_nh, q, sym);
                const double a = (double)tn[k] / tsch_tc[k];
                fn[k] = fs[k] * a;
                wn[k] = ws[k] * a;
                ffar[k] = fs[k] - fn[k];
                wfar[k] = ws[k] - wn[k];
            }
            add_launch(&P, L.schur_tc_near, ids, tn, fn, wn);
            add_launch(&P, L.schur_tc_far, ids, tfar, ffar, wfar);
        }
        add_launch(&P, L.bwdu, ids, tbu, fu, wu);
        for (size_t k = 0; k < nid; ++k)
            if (leaf[k]) tbu[k] = 0;
        add_launch(&P, L.bwdu_small, ids, tbu, fu, wu);
    }
}

static int upload_structure(spk_handle* h) {
    int rc;
    if ((rc = upload(h, &h->d_xs, h->xs))) return rc;
    if ((rc = upload(h, &h->d_rows, h->rows))) return rc;
    if ((rc = upload(h, &h->d_runid, h->runid))) return rc;
    if ((rc = upload(h, &h->d_run_tgt, h->run_tgt))) return rc;
    if ((rc = upload(h, &h->d_run_start, h->run_start))) return rc;
    if ((rc = upload(h, &h->d_run_rel, h->run_rel))) return rc;
    if ((rc = upload(h, &h->d_rel, h->rel))) return rc;
    CU(h, cudaMalloc((void**)&h->d_ipiv, sizeof(int) * std::max<i64>(h->n, 1)));
    CU(h, cudaMalloc((void**)&h->d_bmap, sizeof(int) * std::max<i64>(h->n, 1)));
    // first singular piece, tensor-core wait timeout, leaf-queue wait timeout
    CU(h, cudaMalloc((void**)&h->d_info, 3 * sizeof(int)));
    return SPK_OK;
}

// Build (once) and upload the plan of precision T.
// Dynamic shared memory of the panel sweeps: `n` staged triangles of W lines.
template <typename T, int W>
static size_t sweep_smem(int n) { return sizeof(T) * (size_t)n * W * spk::SLD<T, W>::value; }
// Dynamic shared memory of k_block_panel<T, W>: the staged triangle, plus the
// line tile of the 128-wide FP32 form.
template <typename T, int W>
static int panel_threads() {
    return (std::is_same<T, float>::value && W == 128) ? 4 * spk::PT_LINES : 256;
}
template <typename T, int W>
static size_t panel_smem() {
    return sweep_smem<T, W>(1) + ((std::is_same<T, float>::value && W == 128) ? (size_t)spk::PT_SMEM : 0);
}

template <typename T>
static int ensure_plan(spk_handle* h) {
    Plan& P = h->plan[plan_index<T>(h)];
    if (P.built) return SPK_OK;
    try {
        build_plan(h, P, spk::BlockMax<T>::value, std::is_same<T, float>::value, h->sym != 0);
    } catch (const std::bad_alloc&) {
        return set_err(h, SPK_ENOMEM, "host allocation failed while planning");
    }
    std::vector<spk::DFront> df(h->fronts.size());
    for (size_t i = 0; i < h->fronts.size(); ++i) {
        const HFront& F = h->fronts[i];
        spk::DFront& d = df[i];
        d.loff = F.loff;
        d.uoff = F.uoff;
        d.rows_off = F.rows_off;
        d.runid_off = F.runid_off;
        d.f = (int)F.f;
        d.nf = F.nf;
        d.m = F.m;
        d.ld = F.nf + F.m;
        d.piece0 = F.piece0;
        d.npieces = F.npieces;
        d.run0 = F.run0;
        d.block0 = P.block0[i];
        d.nblocks = P.nblocks[i];
        d.sq = P.schur_q[i];
    }
    for (size_t k = 0; k < P.pf_front.size(); ++k) {   // pseudo fronts of the chunked solves
        spk::DFront d = df[P.pf_front[k]];
        d.block0 = P.pf_b0[k];
        d.nblocks = P.pf_nb[k];
        df.push_back(d);
    }
    int rc;
    if ((rc = upload(h, &P.d_fronts, df))) return rc;
    if ((rc = upload(h, &P.d_blk_c0, P.blk_c0))) return rc;
    if ((rc = upload(h, &P.d_blk_c1, P.blk_c1))) return rc;
    if ((rc = upload(h, &P.d_blk_p0, P.blk_p0))) return rc;
    if ((rc = upload(h, &P.d_blk_np, P.blk_np))) return rc;
    if ((rc = upload(h, &P.d_blk_inv2, P.blk_inv2))) return rc;
    if ((rc = upload(h, &P.d_blk_lpack, P.blk_lpack))) return rc;
    if ((rc = upload(h, &P.d_blk_upack, P.blk_upack))) return rc;
    if ((rc = upload(h, &P.d_blk_front, P.blk_front))) return rc;
    if ((rc = upload(h, &P.d_inv_ids, P.inv_ids))) return rc;
    if ((rc = upload(h, &P.d_sched_ids, P.sched_ids))) return rc;
    if ((rc = upload(h, &P.d_sched_prefix, P.sched_prefix))) return rc;
    if ((rc = upload(h, &P.d_q_order, P.q_order))) return rc;
    if ((rc = upload(h, &P.d_q_parent, P.q_parent))) return rc;
    if ((rc = upload(h, &P.d_q_deps0, P.q_deps))) return rc;
    if ((rc = upload(h, &P.d_q_deps, P.q_deps))) return rc;
    CU(h, cudaMalloc((void**)&P.d_q_next, sizeof(int)));
    spk::Sched& S = P.sched;
    S.fronts = P.d_fronts;
    S.xsuper = h->d_xs;
    S.rows = h->d_rows;
    S.runid = h->d_runid;
    S.run_tgt = h->d_run_tgt;
    S.run_start = h->d_run_start;
    S.run_rel = h->d_run_rel;
    S.rel = h->d_rel;
    S.blk_c0 = P.d_blk_c0;
    S.blk_c1 = P.d_blk_c1;
    S.blk_p0 = P.d_blk_p0;
    S.blk_np = P.d_blk_np;
    S.blk_inv2 = P.d_blk_inv2;
    S.blk_lpack = P.d_blk_lpack;
    S.blk_upack = P.d_blk_upack;
    S.sym = P.sym ? 1 : 0;
    constexpr int BM = spk::BlockMax<T>::value;
    CU(h, cudaFuncSetAttribute(spk::k_block_panel<T, BM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)panel_smem<T, BM>()));
    CU(h, cudaFuncSetAttribute(spk::k_block_lu_pc<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)spk::PcLu<T>::smem));
    CU(h, cudaFuncSetAttribute(spk::k_block_inv<T, BM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)sweep_smem<T, BM>(1)));
    CU(h, cudaFuncSetAttribute(spk::k_leaf_factor<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)spk::LeafSmem<T, 4>::bytes));
    CU(h, cudaFuncSetAttribute(spk::k_leaf_factor<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)spk::LeafSmem<T, 8>::bytes));
    CU(h, cudaFuncSetAttribute(spk::k_leaf_factor<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)spk::LeafSmem<T, 16>::bytes));
    CU(h, cudaFuncSetAttribute(spk::k_leaf_factor<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)spk::LeafSmem<T, 32>::bytes));
    CU(h, cudaFuncSetAttribute(spk::k_leaf_queue<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)spk::LeafSmem<T, 32>::bytes));
    {   // the queue's persistent grid: every CTA the SMs hold at once
        int per_sm = 0;
        CU(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spk::k_leaf_queue<T>, 32 * spk::LF_WARPS,
                                                            spk::LeafSmem<T, 32>::bytes));
        P.q_grid = std::max(1, std::min(h->nsm * std::max(per_sm, 1), spk::cdiv(std::max(P.nq, 1), spk::LF_WARPS)));
    }
    CU(h, cudaFuncSetAttribute(spk::k_front_solve<T, true, spk::FC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)spk::FcSmem<T>::bytes));
    CU(h, cudaFuncSetAttribute(spk::k_front_solve<T, false, spk::FC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)spk::FcSmem<T>::bytes));
    {   // clusters of 16 (a non-portable size) where the GPU can hold one
        h->fc16 = false;
        auto k16f = spk::k_front_solve<T, true, 16>;
        auto k16b = spk::k_front_solve<T, false, 16>;
        if (cudaFuncSetAttribute(k16f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
            cudaFuncSetAttribute(k16b, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
            cudaFuncSetAttribute(k16f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spk::FcSmem<T>::bytes) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k16b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spk::FcSmem<T>::bytes) ==
                cudaSuccess) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(16);
            cfg.blockDim = dim3(spk::FC_THREADS);
            cfg.dynamicSmemBytes = spk::FcSmem<T>::bytes;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = 16;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, (void*)k16f, &cfg) == cudaSuccess && nclusters >= 1)
                h->fc16 = true;
        }
        cudaGetLastError();   // a refused query leaves clusters of 8
    }
    if (std::is_same<T, float>::value) {
        CU(h, cudaFuncSetAttribute(spk::k_tc_update<spk::TC_TRAIL, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   spk::umma::PSMEM));
        CU(h, cudaFuncSetAttribute(spk::k_tc_update<spk::TC_SCHUR, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   spk::umma::PSMEM));
        CU(h, cudaFuncSetAttribute(spk::k_tc_update<spk::TC_TRAIL, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   spk::umma::PSMEM));
        CU(h, cudaFuncSetAttribute(spk::k_tc_update<spk::TC_SCHUR, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   spk::umma::PSMEM));
        CU(h, cudaFuncSetAttribute(spk::k_tc_update<spk::TC_SCHUR, false, 2>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, spk::umma::PGeo<2>::SMEM));
        CU(h, cudaFuncSetAttribute(spk::k_tc_update<spk::TC_SCHUR, true, 2>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, spk::umma::PGeo<2>::SMEM));
    }
    P.built = true;
    return SPK_OK;
}

static void free_plan(Plan& P) {
    void* ptrs[] = {P.d_fronts,     P.d_blk_c0,      P.d_blk_c1,   P.d_blk_p0,     P.d_blk_np,    P.d_blk_inv2,
                    P.d_blk_lpack,  P.d_blk_upack,   P.d_blk_front, P.d_inv_ids,   P.d_sched_ids, P.d_sched_prefix,
                    P.d_q_order,    P.d_q_parent,    P.d_q_deps0,  P.d_q_deps,     P.d_q_next};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    P = Plan();
}

template <typename T>
static Storage<T>& storage(spk_handle* h);
template <>
Storage<double>& storage<double>(spk_handle* h) { return h->s64[h->sym]; }
template <>
Storage<float>& storage<float>(spk_handle* h) { return h->fmode ? h->s16[h->sym] : h->s32[h->sym]; }

template <typename T>
static int ensure_storage(spk_handle* h) {
    int rc = ensure_plan<T>(h);
    if (rc) return rc;
    Storage<T>& S = storage<T>(h);
    if (!S.d) CU(h, cudaMalloc((void**)&S.d, sizeof(T) * std::max<i64>(h->fsize, 1)));
    if (!S.inv2) CU(h, cudaMalloc((void**)&S.inv2, sizeof(T) * std::max<ll>(h->plan[plan_index<T>(h)].inv2_size, 1)));
    // BF16 packs take a quarter of the TF32 hi + lo bytes (same tiles and chunks)
    const ll pack_bytes = h->plan[plan_index<T>(h)].pack_size / (std::is_same<T, float>::value && h->fmode ? 4 : 1);
    if (!S.pack && pack_bytes > 0) CU(h, cudaMalloc((void**)&S.pack, (size_t)pack_bytes));
    return SPK_OK;
}

static int ensure_rhs(spk_handle* h, i64 nrhs) {
    if (nrhs <= h->rhs_cap) return SPK_OK;
    drop_solve_graphs(h);
    cudaFree(h->d_wb); cudaFree(h->d_wy); cudaFree(h->d_wx);
    cudaFree(h->d_rhs); cudaFree(h->d_x); cudaFree(h->d_r); cudaFree(h->d_sums);
    h->d_wb = h->d_wy = h->d_wx = nullptr;
    h->d_rhs = h->d_x = h->d_r = h->d_sums = nullptr;
    h->rhs_cap = 0;
    const i64 chunk = std::min<i64>(nrhs, spk::MAXRHS);
    const size_t wbytes = sizeof(double) * (size_t)h->n * (size_t)chunk;
    const size_t bytes = sizeof(double) * (size_t)h->n * (size_t)nrhs;
    CU(h, cudaMalloc(&h->d_wb, wbytes));
    CU(h, cudaMalloc(&h->d_wy, wbytes));
    CU(h, cudaMalloc(&h->d_wx, wbytes));
    CU(h, cudaMalloc((void**)&h->d_rhs, bytes));
    CU(h, cudaMalloc((void**)&h->d_x, bytes));
    CU(h, cudaMalloc((void**)&h->d_r, bytes));
    CU(h, cudaMalloc((void**)&h->d_sums, sizeof(double) * 2 * (size_t)nrhs));
    h->rhs_cap = nrhs;
    return SPK_OK;
}

// ---------------------------------------------------------------------------
// numeric phases
// ---------------------------------------------------------------------------
// Launch a solve kernel with programmatic stream serialisation: it may start
// while its predecessor drains and waits for it with griddepcontrol.wait
// after prefetching the factor data it needs.  The first chained kernel of a
// solve follows the plain launch of k_permute, which starts only after the
// factorisation has completed, so the factor data read before the wait is
// final.
template <typename... KArgs, typename... Args>
static cudaError_t launch_chained(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t st,
                                  Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, ((KArgs)args)...);
}

// k_leaf_factor of width class c over the fronts of `la`.
template <typename T>
static cudaError_t launch_leaf(int c, const spk::Launch& la, T* fac, int* ipiv, int* info, const spk::Sched& S,
                               cudaStream_t st) {
    const int grid = (la.count + spk::LF_WARPS - 1) / spk::LF_WARPS, block = 32 * spk::LF_WARPS;
    switch (c) {
    case 0: spk::k_leaf_factor<T, 4><<<grid, block, spk::LeafSmem<T, 4>::bytes, st>>>(fac, ipiv, info, S, la); break;
    case 1: spk::k_leaf_factor<T, 8><<<grid, block, spk::LeafSmem<T, 8>::bytes, st>>>(fac, ipiv, info, S, la); break;
    case 2: spk::k_leaf_factor<T, 16><<<grid, block, spk::LeafSmem<T, 16>::bytes, st>>>(fac, ipiv, info, S, la); break;
    default: spk::k_leaf_factor<T, 32><<<grid, block, spk::LeafSmem<T, 32>::bytes, st>>>(fac, ipiv, info, S, la); break;
    }
    return cudaGetLastError();
}

template <typename T>
static int solve_fwd_levels(spk_handle* h, int nrhs, size_t l0, size_t l1, cudaStream_t st);

// Levels whose forward substitution a fused factorisation + solve runs
// inside the factorisation: those below inv_split, on the second stream
// once their block operators are formed (not while timing kernels one by
// one, when nothing runs on the side streams).
template <typename T>
static size_t fused_split(const spk_handle* h) {
    const Plan& PL = h->plan[plan_index<T>(h)];
    return h->prof_mask == 0 && PL.inv_split > 0 ? (size_t)PL.inv_split : 0;
}

// The factorisation's launches.  fs_nrhs > 0: also the forward
// substitution of the levels below fused_split for fs_nrhs right-hand sides
// held in d_rhs (leading dimension n), overlapped with the last levels.
template <typename T>
static int factor_launches(spk_handle* h, int fs_nrhs = 0) {
    constexpr int BM = spk::BlockMax<T>::value;
    T* fac = storage<T>(h).d;
    const Plan& PL = h->plan[plan_index<T>(h)];
    const spk::Sched& S = PL.sched;
    // Look ahead (not while timing kernels one by one): see spk_handle::side.
    const bool ahead = h->prof_mask == 0;
    const int bf16 = std::is_same<T, float>::value ? h->fmode : 0;
    bool pending = false, pending_inv = false;
    // The whole-block solve operators of level group g (k_block_inv).
    auto launch_inv = [&](int g, cudaStream_t st) {
        for (int c = 0; c < 3; ++c) {
            const int cnt = PL.inv_off[g][c + 1] - PL.inv_off[g][c];
            if (cnt <= 0) continue;
            LaunchScope ls(h, SPK_K_BLOCKINV, 0.0, 0.0);
            const int* ent = PL.d_inv_ids + PL.inv_off[g][c];
            T* inv2 = storage<T>(h).inv2;
            if (c == 0) {   // a warp per block, by width class
                for (int wc = 0; wc < spk::LF_CLASSES; ++wc) {
                    const int n = PL.inv_sub[g][wc + 1] - PL.inv_sub[g][wc];
                    if (n <= 0) continue;
                    const int* e = PL.d_inv_ids + PL.inv_sub[g][wc];
                    const int grid = spk::cdiv(n, spk::BI_WARPS), blk = 32 * spk::BI_WARPS;
                    switch (wc) {
                    case 0: spk::k_block_inv_small<T, 4><<<grid, blk, 0, st>>>(fac, h->d_ipiv, inv2, S, PL.d_blk_front, e, n); break;
                    case 1: spk::k_block_inv_small<T, 8><<<grid, blk, 0, st>>>(fac, h->d_ipiv, inv2, S, PL.d_blk_front, e, n); break;
                    case 2: spk::k_block_inv_small<T, 16><<<grid, blk, 0, st>>>(fac, h->d_ipiv, inv2, S, PL.d_blk_front, e, n); break;
                    default: spk::k_block_inv_small<T, 32><<<grid, blk, 0, st>>>(fac, h->d_ipiv, inv2, S, PL.d_blk_front, e, n); break;
                    }
                }
            } else if (c == 1)
                spk::k_block_inv<T, 64><<<cnt, 256, sweep_smem<T, 64>(1), st>>>(fac, h->d_ipiv, inv2, S,
                                                                                  PL.d_blk_front, ent);
            else
                spk::k_block_inv<T, BM><<<cnt, 256, sweep_smem<T, BM>(1), st>>>(fac, h->d_ipiv, inv2, S,
                                                                                  PL.d_blk_front, ent);
        }
    };
    const bool queue = h->leaf_queue != 0 && PL.nq > 0;
    if (queue) {   // the bottom subtrees first, in one persistent launch
        CU(h, cudaMemcpyAsync(PL.d_q_deps, PL.d_q_deps0, sizeof(int) * h->fronts.size(), cudaMemcpyDeviceToDevice,
                              h->stream));
        CU(h, cudaMemsetAsync(PL.d_q_next, 0, sizeof(int), h->stream));
        LaunchScope ls(h, SPK_K_GETRF, PL.q_flops, PL.q_words * sizeof(T));
        const unsigned budget = (unsigned)std::min<long long>(h->wait_budget, 0xffffffffLL);
        spk::k_leaf_queue<T><<<PL.q_grid, 32 * spk::LF_WARPS, spk::LeafSmem<T, 32>::bytes, h->stream>>>(
            fac, h->d_ipiv, h->d_info, S, PL.d_q_order, PL.d_q_parent, PL.nq, PL.d_q_next, PL.d_q_deps, budget,
            h->stall_test, h->d_info + 2);
    }
    bool far_pending[2] = {false, false};   // far Schur tiles of level l in flight on side3 (slot l % 2)
    const int far_sms = h->schur_far_sms > 0 ? std::min(h->schur_far_sms, h->nsm) : std::max(1, h->nsm * 7 / 8);
    for (size_t lvl = 0; lvl < PL.levels.size(); ++lvl) {
        const LevelPlan& P = PL.levels[lvl];
        if (far_pending[lvl & 1]) {   // level lvl - 2's far tiles target this level and above
            CU(h, cudaStreamWaitEvent(h->stream, h->evF[lvl & 1], 0));
            far_pending[lvl & 1] = false;
        }
        const bool fs_here = fs_nrhs > 0 && (size_t)lvl == fused_split<T>(h) && lvl > 0;
        if (ahead && (int)lvl == PL.inv_split && (PL.inv_off[0][3] > PL.inv_off[0][0] || fs_here)) {
            // group 0's blocks are final: their operators beside the last levels
            CU(h, cudaEventRecord(h->evP2, h->stream));
            CU(h, cudaStreamWaitEvent(h->side2, h->evP2, 0));
            launch_inv(0, h->side2);
            if (fs_here) {   // and the forward substitution of those levels (a plain launch first)
                const ll tot = (ll)h->n * fs_nrhs;
                LaunchScope ls(h, SPK_K_PERMUTE, 0.0, (double)tot * (8 + 4 + sizeof(T)));
                spk::k_permute<double, T><<<(int)((tot + 255) / 256), 256, 0, h->side2>>>(
                    h->d_rhs, h->n, (T*)h->d_wb, (int)h->n, h->d_rperm, (int)h->n, fs_nrhs);
                int rc = solve_fwd_levels<T>(h, fs_nrhs, 0, lvl, h->side2);
                if (rc) return rc;
            }
            CU(h, cudaEventRecord(h->evI, h->side2));
            pending_inv = true;
        }
        for (int c = 0; c < spk::LF_CLASSES; ++c) {
            if (P.leaf_factor[c].tiles > 0) {
                LaunchScope ls(h, SPK_K_GETRF, P.leaf_factor[c].flops, P.leaf_factor[c].words * sizeof(T));
                CU(h, launch_leaf<T>(c, launch_of(PL, P.leaf_factor[c]), fac, h->d_ipiv, h->d_info, S, h->stream));
            }
            if (!queue && P.leaf_q[c].tiles > 0) {
                LaunchScope ls(h, SPK_K_GETRF, P.leaf_q[c].flops, P.leaf_q[c].words * sizeof(T));
                CU(h, launch_leaf<T>(c, launch_of(PL, P.leaf_q[c]), fac, h->d_ipiv, h->d_info, S, h->stream));
            }
        }
        for (size_t t = 0; t < P.blu.size(); ++t) {
            const int bw = P.blu[t].bw;
            if (P.blu[t].tiles > 0) {
                LaunchScope ls(h, SPK_K_GETRF, P.blu[t].flops, P.blu[t].words * sizeof(T));
                if (bw <= 32)
                    spk::k_block_lu_small<T><<<(P.blu[t].count + 3) / 4, 128, 0, h->stream>>>(
                        fac, h->d_ipiv, h->d_info, S, launch_of(PL, P.blu[t]), (int)t);
                else if (h->lu_pieces && P.blu_pc[t])
                    spk::k_block_lu_pc<T><<<P.blu[t].tiles, spk::PC_THREADS, spk::PcLu<T>::smem, h->stream>>>(
                        fac, h->d_ipiv, h->d_info, h->d_bmap, S, launch_of(PL, P.blu[t]), (int)t);
                else
                    spk::k_block_lu<T><<<P.blu[t].tiles, spk::LuThreads<T>::value, 0, h->stream>>>(
                        fac, h->d_ipiv, h->d_info, h->d_bmap, S, launch_of(PL, P.blu[t]), (int)t);
            }
            if (pending) {   // the panels read what the previous step's trailing update wrote
                CU(h, cudaStreamWaitEvent(h->stream, h->evB, 0));
                pending = false;
            }
            // Panel split (float forms looking ahead, a step whose trailing
            // update is all on the tensor cores): the near tiles on the launch
            // stream ahead of tile 0, the far ones on the side stream beside
            // them, ahead of the rest of the trailing update.
            bool split = false;
            if constexpr (std::is_same<T, float>::value)
                split = ahead && h->panel_split && P.btrail[t].tiles == 0 && P.btrail_tc[t].tiles > 0 &&
                        P.bpanel_far[t].tiles > 0 && P.bpanel_near[t].tiles > 0;
            auto panel = [&](const LaunchRec& rec, int part, cudaStream_t st) {
                if (rec.tiles <= 0) return;
                LaunchScope ls(h, SPK_K_PANEL, rec.flops, rec.words * sizeof(T));
                const spk::Launch la = launch_of(PL, rec);
                if (bw <= 32)
                    spk::k_block_panel<T, 32><<<rec.tiles, 256, sweep_smem<T, 32>(1), st>>>(
                        fac, h->d_ipiv, h->d_bmap, S, la, (int)t, storage<T>(h).pack, bf16, part);
                else if (bw <= 64)
                    spk::k_block_panel<T, 64><<<rec.tiles, 256, sweep_smem<T, 64>(1), st>>>(
                        fac, h->d_ipiv, h->d_bmap, S, la, (int)t, storage<T>(h).pack, bf16, part);
                else
                    spk::k_block_panel<T, BM><<<rec.tiles, panel_threads<T, BM>(), panel_smem<T, BM>(), st>>>(
                        fac, h->d_ipiv, h->d_bmap, S, la, (int)t, storage<T>(h).pack, bf16, part);
            };
            if (split) {   // the side stream: after this block LU (and the last trailing update)
                CU(h, cudaEventRecord(h->evP, h->stream));
                CU(h, cudaStreamWaitEvent(h->side, h->evP, 0));
                panel(P.bpanel_near[t], 1, h->stream);
                panel(P.bpanel_far[t], 2, h->side);
            } else {
                panel(P.bpanel[t], 0, h->stream);
            }
            if (P.btrail[t].tiles > 0) {
                LaunchScope ls(h, SPK_K_TRAIL, P.btrail[t].flops, P.btrail[t].words * sizeof(T));
                spk::k_block_trail<T><<<P.btrail[t].tiles, 256, 0, h->stream>>>(fac, S, launch_of(PL, P.btrail[t]),
                                                                                 (int)t);
            }
            if constexpr (std::is_same<T, float>::value) {
                // Tiles 1.. of the tensor-core trailing update: on the side
                // stream when looking ahead, on as many SMs as the next
                // block LU and tile 0 leave free; the next panels wait for it.
                if (P.btrail_tc[t].tiles > 0) {
                    const int nt = P.btrail_tc[t].tiles;
                    int grid = std::min(nt, h->nsm);
                    cudaStream_t st = h->stream;
                    if (ahead) {
                        const int reserve = std::max(P.btrail_tc0[t].tiles,
                                                     t + 1 < P.blu.size() ? P.blu[t + 1].tiles : 0);
                        grid = std::max(std::min(nt, h->nsm - reserve), std::min(nt, h->nsm / 2));
                        CU(h, cudaEventRecord(h->evP, h->stream));   // with a split: the near tiles done
                        CU(h, cudaStreamWaitEvent(h->side, h->evP, 0));
                        st = h->side;
                    }
                    LaunchScope ls(h, SPK_K_TC_TRAIL, P.btrail_tc[t].flops, P.btrail_tc[t].words * sizeof(T));
                    auto kern = bf16 ? spk::k_tc_update<spk::TC_TRAIL, true> : spk::k_tc_update<spk::TC_TRAIL, false>;
                    kern<<<grid, spk::TC_THREADS, spk::umma::PSMEM, st>>>(
                        fac, storage<T>(h).pack, S, launch_of(PL, P.btrail_tc[t]), (int)t, nt, 1, 0, h->d_info + 1);
                    if (ahead) {
                        CU(h, cudaEventRecord(h->evB, h->side));
                        pending = true;
                    }
                }
                // Tile 0 (the next block's diagonal block) on the launch stream.
                if (P.btrail_tc0[t].tiles > 0) {
                    LaunchScope ls(h, SPK_K_TC_TRAIL, P.btrail_tc0[t].flops, P.btrail_tc0[t].words * sizeof(T));
                    const int nt = P.btrail_tc0[t].tiles;
                    auto kern = bf16 ? spk::k_tc_update<spk::TC_TRAIL, true> : spk::k_tc_update<spk::TC_TRAIL, false>;
                    kern<<<std::min(nt, h->nsm), spk::TC_THREADS, spk::umma::PSMEM, h->stream>>>(
                        fac, storage<T>(h).pack, S, launch_of(PL, P.btrail_tc0[t]), (int)t, nt, 0, 0, h->d_info + 1);
                }
            }
        }
        if (pending) {   // the level's Schur complement needs every trailing update
            CU(h, cudaStreamWaitEvent(h->stream, h->evB, 0));
            pending = false;
        }
        if (P.schur.tiles > 0) {
            LaunchScope ls(h, SPK_K_SCHUR, P.schur.flops, P.schur.words * sizeof(T));
            spk::k_schur<T><<<P.schur.tiles, 256, 0, h->stream>>>(fac, S, launch_of(PL, P.schur));
        }
        if constexpr (std::is_same<T, float>::value) {
            auto schur_tc = [&](const LaunchRec& rec, int part, int grid, cudaStream_t st) {
                if (rec.tiles <= 0) return;
                LaunchScope ls(h, SPK_K_TC_SCHUR, rec.flops, rec.words * sizeof(T));
                const int nt = rec.tiles;
                const spk::Launch la = launch_of(PL, rec);
                if (PL.schur_nh == 2) {   // 128 x 256 tiles
                    auto kern = bf16 ? spk::k_tc_update<spk::TC_SCHUR, true, 2> : spk::k_tc_update<spk::TC_SCHUR, false, 2>;
                    kern<<<std::min(nt, grid), spk::TC_THREADS, spk::umma::PGeo<2>::SMEM, st>>>(
                        fac, storage<T>(h).pack, S, la, 0, nt, 0, part, h->d_info + 1);
                } else {
                    auto kern = bf16 ? spk::k_tc_update<spk::TC_SCHUR, true> : spk::k_tc_update<spk::TC_SCHUR, false>;
                    kern<<<std::min(nt, grid), spk::TC_THREADS, spk::umma::PSMEM, st>>>(
                        fac, storage<T>(h).pack, S, la, 0, nt, 0, part, h->d_info + 1);
                }
            };
            // Far tiles (targets two or more levels up) on side3, on far_sms
            // SMs, beside the near tiles and the next level; every scatter is
            // an atomic add, so they may overlap the other levels' updates of
            // the same fronts.
            if (ahead && h->schur_split && P.schur_tc_far.tiles > 0) {
                CU(h, cudaEventRecord(h->evS, h->stream));
                schur_tc(P.schur_tc_near, 1, h->nsm, h->stream);
                CU(h, cudaStreamWaitEvent(h->side3, h->evS, 0));
                schur_tc(P.schur_tc_far, 2, far_sms, h->side3);
                CU(h, cudaEventRecord(h->evF[lvl & 1], h->side3));
                far_pending[lvl & 1] = true;
            } else {
                schur_tc(P.schur_tc, 0, h->nsm, h->stream);
            }
        }
    }
    for (int k = 0; k < 2; ++k)   // join side3 (nothing is left to target, but the graph must rejoin)
        if (far_pending[k]) CU(h, cudaStreamWaitEvent(h->stream, h->evF[k], 0));
    if (pending_inv) CU(h, cudaStreamWaitEvent(h->stream, h->evI, 0));
    else launch_inv(0, h->stream);
    launch_inv(1, h->stream);
    CU(h, cudaGetLastError());
    return SPK_OK;
}


template <typename T>
static int run_factor(spk_handle* h) {
    static const int init[3] = {INT_MAX, 0, 0};
    int rc = ensure_plan<T>(h);   // rebuilt after an option dropped it
    if (rc) return rc;
    CU(h, cudaMemcpyAsync(h->d_info, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    return via_graph(h, h->g_factor[graph_index<T>(h)], [&] { return factor_launches<T>(h); });
}

// k_solve_leaf of width class c over `count` fronts (chained launch).
template <typename T, bool FWD>
static cudaError_t launch_solve_leaf(int c, int count, cudaStream_t st, const T* fac, const T* inv, T* in, T* out,
                                     const T* xs, int n, int nrhs, const spk::Sched& S, const spk::Launch& la) {
    const int grid = (count + 7) / 8;
    if (nrhs == 1) {   // one right-hand side: passes of one
        switch (c) {
        case 0: return launch_chained(spk::k_solve_leaf<T, FWD, 4, 1>, grid, 256, 0, st, fac, inv, in, out, xs, n, nrhs, S, la);
        case 1: return launch_chained(spk::k_solve_leaf<T, FWD, 8, 1>, grid, 256, 0, st, fac, inv, in, out, xs, n, nrhs, S, la);
        case 2: return launch_chained(spk::k_solve_leaf<T, FWD, 16, 1>, grid, 256, 0, st, fac, inv, in, out, xs, n, nrhs, S, la);
        default: return launch_chained(spk::k_solve_leaf<T, FWD, 32, 1>, grid, 256, 0, st, fac, inv, in, out, xs, n, nrhs, S, la);
        }
    }
    switch (c) {
    case 0: return launch_chained(spk::k_solve_leaf<T, FWD, 4, 4>, grid, 256, 0, st, fac, inv, in, out, xs, n, nrhs, S, la);
    case 1: return launch_chained(spk::k_solve_leaf<T, FWD, 8, 4>, grid, 256, 0, st, fac, inv, in, out, xs, n, nrhs, S, la);
    case 2: return launch_chained(spk::k_solve_leaf<T, FWD, 16, 4>, grid, 256, 0, st, fac, inv, in, out, xs, n, nrhs, S, la);
    default: return launch_chained(spk::k_solve_leaf<T, FWD, 32, 4>, grid, 256, 0, st, fac, inv, in, out, xs, n, nrhs, S, la);
    }
}

// The forward substitution over levels [l0, l1) on the permuted work
// vectors (wb, consumed, -> wy), launched on `st`.
template <typename T>
static int solve_fwd_levels(spk_handle* h, int nrhs, size_t l0, size_t l1, cudaStream_t st) {
    const T* fac = storage<T>(h).d;
    const T* inv = storage<T>(h).inv2;
    const Plan& PL = h->plan[plan_index<T>(h)];
    const spk::Sched& S = PL.sched;
    T* b = (T*)h->d_wb;
    T* y = (T*)h->d_wy;
    const int n = (int)h->n;
    constexpr size_t fc_smem = spk::FcSmem<T>::bytes;
    for (size_t l = l0; l < l1; ++l) {
        const LevelPlan& P = PL.levels[l];
        for (int c = 0; c < spk::LF_CLASSES; ++c) {
            const LaunchRec& R = P.front_leaf[c];
            if (R.tiles == 0) continue;
            LaunchScope ls(h, SPK_K_FWD, R.flops * nrhs, R.words * sizeof(T));
            CU(h, (launch_solve_leaf<T, true>(c, R.count, st, fac, inv, b, y, (const T*)nullptr, n, nrhs, S,
                                              launch_of(PL, R))));
        }
        if (P.front_big.tiles > 0) {
            LaunchScope ls(h, SPK_K_FWD, P.front_big.flops * nrhs, P.front_big.words * sizeof(T));
            if (h->fc16)
                spk::k_front_solve<T, true, 16><<<16 * P.front_big.tiles, spk::FC_THREADS, fc_smem, st>>>(
                    fac, inv, b, y, n, nrhs, S, launch_of(PL, P.front_big));
            else
                spk::k_front_solve<T, true, spk::FC><<<spk::FC * P.front_big.tiles, spk::FC_THREADS, fc_smem,
                                                       st>>>(fac, inv, b, y, n, nrhs, S,
                                                                    launch_of(PL, P.front_big));
        }
        if (P.front_l21.tiles > 0) {
            LaunchScope ls(h, SPK_K_FWD, P.front_l21.flops * nrhs, P.front_l21.words * sizeof(T));
            CU(h, launch_chained(spk::k_fwd_l21<T>, P.front_l21.tiles, 256, 0, st, fac, b, (const T*)y, n, nrhs,
                                 S, launch_of(PL, P.front_l21)));
        }
        for (size_t c = 0; c < P.chunks.size(); ++c) {   // chunked root fronts, chunks in order
            const LevelPlan::SolveChunk& ch = P.chunks[c];
            {
                LaunchScope ls(h, SPK_K_FWD, ch.rec.flops * nrhs, ch.rec.words * sizeof(T));
                if (h->fc16)
                    spk::k_front_solve<T, true, 16><<<16, spk::FC_THREADS, fc_smem, st>>>(fac, inv, b, y, n, nrhs, S,
                                                                                         launch_of(PL, ch.rec));
                else
                    spk::k_front_solve<T, true, spk::FC><<<spk::FC, spk::FC_THREADS, fc_smem, st>>>(
                        fac, inv, b, y, n, nrhs, S, launch_of(PL, ch.rec));
            }
            if (c + 1 < P.chunks.size() && P.chunks[c + 1].front == ch.front) {   // rows below the chunk
                const HFront& F = h->fronts[ch.front];
                const int r0 = ch.hi, r1 = F.nf;
                LaunchScope ls(h, SPK_K_FWD, 2.0 * (r1 - r0) * (ch.hi - ch.lo) * nrhs,
                               (double)(r1 - r0) * (ch.hi - ch.lo) * sizeof(T));
                const int grid = spk::cdiv(r1 - r0, spk::L21_ROWS) * spk::cdiv(ch.hi - ch.lo, spk::L21_COLS);
                spk::k_front_gemv<T><<<grid, 256, 0, st>>>(fac, b, (const T*)y, n, nrhs, F.loff, F.nf + F.m,
                                                          (int)F.f, r0, r1, ch.lo, ch.hi);
            }
        }
        for (size_t t = 0; t < P.fwd_small.size(); ++t)
            if (P.fwd_small[t].tiles > 0) {
                LaunchScope ls(h, SPK_K_FWD, P.fwd_small[t].flops * nrhs, P.fwd_small[t].words * sizeof(T));
                CU(h, launch_chained(spk::k_fwd<T>, P.fwd_small[t].tiles, spk::TS, 0, st, fac, inv, b, y, n,
                                     nrhs, S, launch_of(PL, P.fwd_small[t]), (int)t));
            }
    }
    CU(h, cudaGetLastError());
    return SPK_OK;
}

// The backward substitution over every level (wy -> wx), launched on `st`.
template <typename T>
static int solve_bwd_levels(spk_handle* h, int nrhs, cudaStream_t st) {
    const T* fac = storage<T>(h).d;
    const T* inv = storage<T>(h).inv2;
    const Plan& PL = h->plan[plan_index<T>(h)];
    const spk::Sched& S = PL.sched;
    T* y = (T*)h->d_wy;
    T* x = (T*)h->d_wx;
    const int n = (int)h->n;
    constexpr size_t fc_smem = spk::FcSmem<T>::bytes;
    for (size_t l = PL.levels.size(); l-- > 0;) {
        const LevelPlan& P = PL.levels[l];
        for (int c = 0; c < spk::LF_CLASSES; ++c) {
            const LaunchRec& R = P.front_leaf[c];
            if (R.tiles == 0) continue;
            LaunchScope ls(h, SPK_K_BWD, R.flops * nrhs, R.words * sizeof(T));
            CU(h, (launch_solve_leaf<T, false>(c, R.count, st, fac, inv, y, x, (const T*)x, n, nrhs, S,
                                               launch_of(PL, R))));
        }
        if (P.bwdu_small.tiles > 0) {
            LaunchScope ls(h, SPK_K_BWD, P.bwdu_small.flops * nrhs, P.bwdu_small.words * sizeof(T));
            CU(h, launch_chained(spk::k_bwd_u12<T>, P.bwdu_small.tiles, 256, 0, st, fac, y, x, n, nrhs, S,
                                 launch_of(PL, P.bwdu_small)));
        }
        if (P.front_big.tiles > 0) {
            LaunchScope ls(h, SPK_K_BWD, P.front_big.flops * nrhs, P.front_big.words * sizeof(T));
            if (h->fc16)
                spk::k_front_solve<T, false, 16><<<16 * P.front_big.tiles, spk::FC_THREADS, fc_smem, st>>>(
                    fac, inv, y, x, n, nrhs, S, launch_of(PL, P.front_big));
            else
                spk::k_front_solve<T, false, spk::FC><<<spk::FC * P.front_big.tiles, spk::FC_THREADS, fc_smem,
                                                        st>>>(fac, inv, y, x, n, nrhs, S,
                                                                     launch_of(PL, P.front_big));
        }
        for (size_t c = P.chunks.size(); c-- > 0;) {   // chunked root fronts, chunks in reverse
            const LevelPlan::SolveChunk& ch = P.chunks[c];
            {
                LaunchScope ls(h, SPK_K_BWD, ch.rec.flops * nrhs, ch.rec.words * sizeof(T));
                if (h->fc16)
                    spk::k_front_solve<T, false, 16><<<16, spk::FC_THREADS, fc_smem, st>>>(fac, inv, y, x, n, nrhs,
                                                                                          S, launch_of(PL, ch.rec));
                else
                    spk::k_front_solve<T, false, spk::FC><<<spk::FC, spk::FC_THREADS, fc_smem, st>>>(
                        fac, inv, y, x, n, nrhs, S, launch_of(PL, ch.rec));
            }
            if (c > 0 && P.chunks[c - 1].front == ch.front) {   // rows above the chunk
                const HFront& F = h->fronts[ch.front];
                const int r0 = 0, r1 = ch.lo;
                LaunchScope ls(h, SPK_K_BWD, 2.0 * (r1 - r0) * (ch.hi - ch.lo) * nrhs,
                               (double)(r1 - r0) * (ch.hi - ch.lo) * sizeof(T));
                const int grid = spk::cdiv(r1 - r0, spk::L21_ROWS) * spk::cdiv(ch.hi - ch.lo, spk::L21_COLS);
                spk::k_front_gemv<T><<<grid, 256, 0, st>>>(fac, y, (const T*)x, n, nrhs, F.loff, F.nf + F.m,
                                                          (int)F.f, r0, r1, ch.lo, ch.hi);
            }
        }
        for (size_t t = 0; t < P.bwd_small.size(); ++t)
            if (P.bwd_small[t].tiles > 0) {
                LaunchScope ls(h, SPK_K_BWD, P.bwd_small[t].flops * nrhs, P.bwd_small[t].words * sizeof(T));
                CU(h, launch_chained(spk::k_bwd<T>, P.bwd_small[t].tiles, spk::TS, 0, st, fac, inv, y, x, n,
                                     nrhs, S, launch_of(PL, P.bwd_small[t]), (int)t));
            }
    }
    CU(h, cudaGetLastError());
    return SPK_OK;
}

// Solve in place on the permuted work vectors: wb (rhs, consumed) -> wx.
template <typename T>
static int run_solve_permuted(spk_handle* h, int nrhs, bool transpose) {
    const T* fac = storage<T>(h).d;
    const T* inv = storage<T>(h).inv2;
    const Plan& PL = h->plan[plan_index<T>(h)];
    const spk::Sched& S = PL.sched;
    T* b = (T*)h->d_wb;
    T* y = (T*)h->d_wy;
    T* x = (T*)h->d_wx;
    const int n = (int)h->n;
    if (transpose) {   // A^T: U^T pass in block order, then L^T pass top-down with blocks reversed
        for (const LevelPlan& P : PL.levels)
            for (size_t t = 0; t < P.fwd.size(); ++t)
                if (P.fwd[t].tiles > 0) {
                    LaunchScope ls(h, SPK_K_FWD, P.fwd[t].flops * nrhs, P.fwd[t].words * sizeof(T));
                    CU(h, launch_chained(spk::k_tfwd<T>, P.fwd[t].tiles, spk::TS, 0, h->stream, fac, inv, b, y, n, nrhs, S,
                                         launch_of(PL, P.fwd[t]), (int)t));
                }
        for (size_t l = PL.levels.size(); l-- > 0;) {
            const LevelPlan& P = PL.levels[l];
            if (P.bwdu.tiles > 0) {
                LaunchScope ls(h, SPK_K_BWD, P.bwdu.flops * nrhs, P.bwdu.words * sizeof(T));
                CU(h, launch_chained(spk::k_tbwd_l21<T>, P.bwdu.tiles, 256, 0, h->stream, fac, y, x, n, nrhs, S,
                                     launch_of(PL, P.bwdu)));
            }
            for (size_t t = 0; t < P.bwd.size(); ++t)
                if (P.bwd[t].tiles > 0) {
                    LaunchScope ls(h, SPK_K_BWD, P.bwd[t].flops * nrhs, P.bwd[t].words * sizeof(T));
                    CU(h, launch_chained(spk::k_tbwd<T>, P.bwd[t].tiles, spk::TS, 0, h->stream, fac, inv, y, x, n, nrhs, S,
                                         launch_of(PL, P.bwd[t]), (int)t));
                }
        }
        CU(h, cudaGetLastError());
        return SPK_OK;
    }
    int rc = solve_fwd_levels<T>(h, nrhs, 0, PL.levels.size(), h->stream);
    if (rc) return rc;
    return solve_bwd_levels<T>(h, nrhs, h->stream);
}

// x(:, 0:nrhs) (=|+=) A^{-1} rhs(:, 0:nrhs) (A^{-T} with `transpose`), both
// device FP64, original order.
template <typename T>
static int solve_device(spk_handle* h, const double* rhs, i64 ldr, double* x, i64 ldx, i64 nrhs, int accumulate,
                        bool transpose = false) {
    const int n = (int)h->n;
    int rc0 = ensure_plan<T>(h);   // rebuilt after an option dropped it (the factors are kept)
    if (rc0) return rc0;
    for (i64 c0 = 0; c0 < nrhs; c0 += spk::MAXRHS) {
        int nc = (int)std::min<i64>(spk::MAXRHS, nrhs - c0);
        ll tot = (ll)n * nc;
        int blocks = (int)((tot + 255) / 256);
        {
            LaunchScope ls(h, SPK_K_PERMUTE, 0.0, (double)tot * (8 + 4 + sizeof(T)));
            spk::k_permute<double, T><<<blocks, 256, 0, h->stream>>>(rhs + c0 * ldr, ldr, (T*)h->d_wb, n, h->d_rperm,
                                                                     n, nc);
        }
        GraphRec& g = transpose ? h->g_tsolve[graph_index<T>(h)][nc] : h->g_solve[graph_index<T>(h)][nc];
        int rc = via_graph(h, g, [&] { return run_solve_permuted<T>(h, nc, transpose); });
        if (rc) return rc;
        {
            LaunchScope ls(h, SPK_K_PERMUTE, 0.0, (double)tot * (8 * (accumulate ? 2 : 1) + 4 + sizeof(T)));
            spk::k_unpermute<T><<<blocks, 256, 0, h->stream>>>((const T*)h->d_wx, n, x + c0 * ldx, ldx, h->d_rinvp, n,
                                                               nc, accumulate);
        }
    }
    CU(h, cudaGetLastError());
    return SPK_OK;
}

static int residual_device(spk_handle* h, const double* b, i64 ldb, const double* x, i64 ldx, i64 nrhs,
                           double* relres, bool transpose = false, std::vector<double>* sq = nullptr) {
    const int n = (int)h->n;
    CU(h, cudaMemsetAsync(h->d_sums, 0, sizeof(double) * 2 * (size_t)nrhs, h->stream));
    dim3 grid(std::min((n + 255) / 256, 8 * h->nsm));   // grid-stride rows: few partial sums per norm
    {
        LaunchScope ls(h, SPK_K_RESIDUAL, 2.0 * h->nnz * nrhs, (double)h->nnz * (8 + 4 + 8) + 8.0 * h->nnz * nrhs +
                                                                  24.0 * n * nrhs);
        if (transpose)   // rows of A^T = A's CSC columns, values in order
            spk::k_residual<<<grid, 256, 0, h->stream>>>(h->d_aval, h->d_ccolptr, h->d_crow, nullptr, x, ldx, b, ldb,
                                                         h->d_r, n, (int)nrhs, h->d_sums);
        else
            spk::k_residual<<<grid, 256, 0, h->stream>>>(h->d_acsr, h->d_rowptr, h->d_col, nullptr, x, ldx, b, ldb,
                                                         h->d_r, n, (int)nrhs, h->d_sums);
    }
    CU(h, cudaGetLastError());
    std::vector<double> sums(2 * nrhs);
    CU(h, cudaMemcpyAsync(sums.data(), h->d_sums, sizeof(double) * 2 * nrhs, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    double worst = 0.0;
    for (i64 j = 0; j < nrhs; ++j) {
        double nb = std::sqrt(sums[2 * j + 1]), nr = std::sqrt(sums[2 * j]);
        double rel = nb > 0.0 ? nr / nb : nr;
        if (!(rel <= worst)) worst = rel;   // NaN propagates
    }
    *relres = worst;
    if (sq) *sq = sums;   // ||r_j||^2, ||b_j||^2 interleaved
    return SPK_OK;
}

// ---------------------------------------------------------------------------
// GMRES-IR: restarted GMRES (cycles of at most GM_M iterations) on A d = r
// in FP64, preconditioned on the right by the factor of the selected float
// form (z = M^-1 v is one triangular solve), classical Gram-Schmidt with
// reorthogonalisation, Givens rotations on the host.  Every cycle starts
// from the true FP64 residual of x and ends with x += Z y.  Right-hand sides
// in groups of spk::GM_MAXRHS, each with its own Krylov space.
// ---------------------------------------------------------------------------
constexpr int GM_M = 30;

static int ensure_gmres(spk_handle* h) {
    if (h->gm_V) return SPK_OK;
    const size_t blk = sizeof(double) * (size_t)h->n * spk::GM_MAXRHS;
    CU(h, cudaMalloc((void**)&h->gm_V, blk * (GM_M + 1)));
    CU(h, cudaMalloc((void**)&h->gm_Z, blk * GM_M));
    CU(h, cudaMalloc((void**)&h->gm_w, blk));
    CU(h, cudaMalloc((void**)&h->gm_c, sizeof(double) * (2 * (GM_M + 1) + 1) * spk::GM_MAXRHS));
    return SPK_OK;
}

// Columns [0, nrhs) of b / x (nrhs <= GM_MAXRHS).  `budget` preconditioned
// solves at most; *used receives the number made, *cycles the restarts.
template <typename T>
static int gmres_ir(spk_handle* h, const double* b, i64 ldb, double* x, i64 ldx, int nrhs, double tol, int budget,
                    double* relres, int* used, int* cycles) {
    int rc = ensure_gmres(h);
    if (rc) return rc;
    const int n = (int)h->n;
    const ll tot = (ll)n * nrhs;
    const int vgrid = (int)std::min<ll>((tot + 255) / 256, 8LL * h->nsm);
    const int dgrid = std::max(1, std::min((n + 255) / 256, 2 * h->nsm));
    double* c = h->gm_c;                       // [h1 (GM_M+1) x nrhs | h2 (GM_M+1) x nrhs | norm^2 nrhs]
    double* h1 = c;
    double* h2 = c + (GM_M + 1) * nrhs;
    double* nrm = c + 2 * (GM_M + 1) * nrhs;
    std::vector<double> H((size_t)nrhs * (GM_M + 1) * GM_M), cs((size_t)nrhs * GM_M), sn((size_t)nrhs * GM_M),
        g((size_t)nrhs * (GM_M + 1)), hc(2 * (GM_M + 1) * nrhs + nrhs), y((size_t)GM_M * nrhs);
    std::vector<int> k(nrhs);
    std::vector<double> sq;
    *used = 0;
    *cycles = 0;
    double rel = 0.0;
    for (;;) {
        if ((rc = residual_device(h, b, ldb, x, ldx, nrhs, &rel, false, &sq))) return rc;
        if (rel <= tol || *used >= budget || rel != rel) break;
        ++*cycles;
        std::vector<double> beta2(nrhs), target(nrhs);
        std::vector<char> active(nrhs);
        for (int r = 0; r < nrhs; ++r) {
            beta2[r] = sq[2 * r];
            const double nb = std::sqrt(sq[2 * r + 1]);
            target[r] = 0.5 * tol * (nb > 0.0 ? nb : 1.0);
            active[r] = std::sqrt(beta2[r]) > target[r];
            g[(size_t)r * (GM_M + 1)] = std::sqrt(beta2[r]);
            k[r] = 0;
        }
        // V_0 = r / ||r|| (the residual kernel left r in d_r, leading dimension n)
        CU(h, cudaMemcpyAsync(nrm, beta2.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, h->stream));
        spk::k_gm_scale<<<vgrid, 256, 0, h->stream>>>(h->d_r, nrm, h->gm_V, n, nrhs);
        for (int j = 0; j < GM_M && *used < budget; ++j) {
            double* Vj = h->gm_V + (ll)j * tot;
            double* Zj = h->gm_Z + (ll)j * tot;
            if ((rc = solve_device<T>(h, Vj, n, Zj, n, nrhs, 0, false))) return rc;
            ++*used;
            {
                LaunchScope ls(h, SPK_K_RESIDUAL, 2.0 * h->nnz * nrhs, (double)h->nnz * (8 + 4 + 8) + 8.0 * h->nnz * nrhs);
                spk::k_gm_spmv<<<(n + 255) / 256, 256, 0, h->stream>>>(h->d_acsr, h->d_rowptr, h->d_col, nullptr, Zj,
                                                                       h->gm_w, n, nrhs);
            }
            CU(h, cudaMemsetAsync(c, 0, sizeof(double) * (2 * (GM_M + 1) + 1) * nrhs, h->stream));
            spk::k_gm_dots<<<dim3(dgrid, j + 1), 256, 0, h->stream>>>(h->gm_V, h->gm_w, n, nrhs, h1);
            spk::k_gm_axpy<<<vgrid, 256, 0, h->stream>>>(h->gm_V, h1, h->gm_w, n, n, nrhs, j + 1, -1.0);
            spk::k_gm_dots<<<dim3(dgrid, j + 1), 256, 0, h->stream>>>(h->gm_V, h->gm_w, n, nrhs, h2);
            spk::k_gm_axpy<<<vgrid, 256, 0, h->stream>>>(h->gm_V, h2, h->gm_w, n, n, nrhs, j + 1, -1.0);
            spk::k_gm_dots<<<dim3(dgrid, 1), 256, 0, h->stream>>>(h->gm_w, h->gm_w, n, nrhs, nrm);
            spk::k_gm_scale<<<vgrid, 256, 0, h->stream>>>(h->gm_w, nrm, h->gm_V + (ll)(j + 1) * tot, n, nrhs);
            CU(h, cudaGetLastError());
            CU(h, cudaMemcpyAsync(hc.data(), c, sizeof(double) * hc.size(), cudaMemcpyDeviceToHost, h->stream));
            CU(h, cudaStreamSynchronize(h->stream));
            bool any = false;
            for (int r = 0; r < nrhs; ++r) {
                if (!active[r]) continue;
                double* col = H.data() + ((size_t)r * GM_M + j) * (GM_M + 1);
                for (int i = 0; i <= j; ++i) col[i] = hc[(size_t)i * nrhs + r] + hc[(size_t)(GM_M + 1 + i) * nrhs + r];
                col[j + 1] = std::sqrt(std::max(hc[(size_t)2 * (GM_M + 1) * nrhs + r], 0.0));
                double* csr = cs.data() + (size_t)r * GM_M;
                double* snr = sn.data() + (size_t)r * GM_M;
                for (int i = 0; i < j; ++i) {   // earlier rotations
                    const double a = col[i], bb = col[i + 1];
                    col[i] = csr[i] * a + snr[i] * bb;
                    col[i + 1] = -snr[i] * a + csr[i] * bb;
                }
                const double a = col[j], bb = col[j + 1], rr = std::hypot(a, bb);
                csr[j] = rr > 0.0 ? a / rr : 1.0;
                snr[j] = rr > 0.0 ? bb / rr : 0.0;
                col[j] = rr;
                col[j + 1] = 0.0;
                double* gr = g.data() + (size_t)r * (GM_M + 1);
                gr[j + 1] = -snr[j] * gr[j];
                gr[j] = csr[j] * gr[j];
                k[r] = j + 1;
                const double hn = std::sqrt(std::max(hc[(size_t)2 * (GM_M + 1) * nrhs + r], 0.0));
                if (std::fabs(gr[j + 1]) <= target[r] || hn == 0.0) active[r] = 0;
                else any = true;
            }
            if (!any) break;
        }
        // x += Z y, y from the rotated Hessenberg systems
        int kmax = 0;
        std::fill(y.begin(), y.end(), 0.0);
        for (int r = 0; r < nrhs; ++r) {
            const int kr = k[r];
            kmax = std::max(kmax, kr);
            const double* gr = g.data() + (size_t)r * (GM_M + 1);
            for (int i = kr - 1; i >= 0; --i) {
                double t = gr[i];
                for (int l = i + 1; l < kr; ++l) t -= H[((size_t)r * GM_M + l) * (GM_M + 1) + i] * y[(size_t)l * nrhs + r];
                const double d = H[((size_t)r * GM_M + i) * (GM_M + 1) + i];
                y[(size_t)i * nrhs + r] = d != 0.0 ? t / d : 0.0;
            }
        }
        if (kmax == 0) break;
        CU(h, cudaMemcpyAsync(c, y.data(), sizeof(double) * (size_t)kmax * nrhs, cudaMemcpyHostToDevice, h->stream));
        spk::k_gm_axpy<<<vgrid, 256, 0, h->stream>>>(h->gm_Z, c, x, ldx, n, nrhs, kmax, 1.0);
        CU(h, cudaGetLastError());
    }
    *relres = rel;
    return SPK_OK;
}

static int check_h(spk_handle* h) {
    if (!h) return SPK_EARG;
    if (h->device >= 0) {
        cudaError_t e = cudaSetDevice(h->device);
        if (e != cudaSuccess) return set_err(h, SPK_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    }
    return SPK_OK;
}

// A precision code: SPK_FP64, SPK_FP32 or SPK_BF16S, optionally | SPK_SPD.
static int base_precision(int p) { return p & ~SPK_SPD; }
static bool valid_precision(int p) {
    const int b = base_precision(p);
    return b == SPK_FP64 || b == SPK_FP32 || b == SPK_BF16S;
}
static bool is_fp64(int p) { return base_precision(p) == SPK_FP64; }

// Point the float paths at the storage of the given float form.
static void select_form(spk_handle* h, int precision) {
    h->fmode = base_precision(precision) == SPK_BF16S ? 1 : 0;
    h->sym = (precision & SPK_SPD) ? 1 : 0;
}

static Storage<float>& float_storage(spk_handle* h, int precision) {
    const int y = (precision & SPK_SPD) ? 1 : 0;
    return base_precision(precision) == SPK_BF16S ? h->s16[y] : h->s32[y];
}

template <typename T>
static int load_into(spk_handle* h) {
    int rc = ensure_storage<T>(h);
    if (rc) return rc;
    Storage<T>& S = storage<T>(h);
    CU(h, cudaMemsetAsync(S.d, 0, sizeof(T) * (size_t)h->fsize, h->stream));
    if (h->nnz > 0) {
        int blocks = (int)std::min<i64>((h->nnz + 255) / 256, 152 * 16);
        LaunchScope ls(h, SPK_K_ASSEMBLE, 0.0, (double)h->nnz * (8 + 8 + 2 * sizeof(T)));
        spk::k_scatter_values<T><<<blocks, 256, 0, h->stream>>>(h->d_aval, h->d_slot, S.d, h->nnz);
    }
    CU(h, cudaGetLastError());
    S.loaded = true;
    S.factored = false;
    return SPK_OK;
}

template <typename T>
static int fetch_factor(spk_handle* h, std::vector<double>& out) {
    std::vector<T> tmp(h->fsize);
    CU(h, cudaMemcpyAsync(tmp.data(), storage<T>(h).d, sizeof(T) * h->fsize, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    out.assign(tmp.begin(), tmp.end());
    return SPK_OK;
}

static bool factored(spk_handle* h, int precision) {
    return is_fp64(precision) ? h->s64[(precision & SPK_SPD) ? 1 : 0].factored : float_storage(h, precision).factored;
}

// Does (i, j) (permuted, 0-based) belong to the reference's structure?  L
// part (i >= first column of j's supernode): i in that supernode's rows;
// otherwise U part: j in the off-diagonal rows of i's supernode.
static bool in_structure(const spk_handle* h, int i, int j) {
    const int sj = h->col_snode[j];
    int s = (i >= h->xs[sj]) ? sj : h->col_snode[i];
    int key = (i >= h->xs[sj]) ? i : j;
    const int* a = h->lindx0.data() + h->xlindx0[s];
    const int* b = h->lindx0.data() + h->xlindx0[s + 1];
    if (s != sj) a += h->xs[s + 1] - h->xs[s];
    const int* q = std::lower_bound(a, b, key);
    return q != b && *q == key;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int spk_create(int64_t n, int64_t nsuper, const int64_t* xsuper, const int64_t* snode, const int64_t* xlindx,
               const int64_t* lindx, const int64_t* xlnz, const int64_t* xunz, int index_base, spk_handle** out) {
    if (!out) return SPK_EARG;
    *out = nullptr;
    g_create_err = "spk_create: bad arguments";
    if (n <= 0 || nsuper <= 0 || nsuper > n || n > INT_MAX || !xsuper || !snode || !xlindx || !lindx || !xlnz ||
        !xunz || (index_base != 0 && index_base != 1))
        return SPK_EARG;
    spk_handle* h = nullptr;
    try {
        h = new spk_handle();
    } catch (const std::bad_alloc&) {
        return SPK_ENOMEM;
    }
    h->n = n;
    h->nsuper = nsuper;
    int rc;
    try {
        rc = analyse(h, xsuper, snode, xlindx, lindx, xlnz, xunz, index_base);

    } catch (const std::bad_alloc&) {
        rc = set_err(h, SPK_ENOMEM, "host allocation failed while analysing the structure");
    }
    if (rc == SPK_OK) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) rc = set_err(h, SPK_ECUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
        else {
            h->device = dev;
            if (cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || h->nsm < 1)
                h->nsm = 1;
            // the launch stream (the factorisation's block chain, captured
            // from it) ahead of the look-ahead streams when SMs free up
            int lo = 0, hi = 0;
            if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) lo = hi = 0;
            e = cudaStreamCreateWithPriority(&h->own, cudaStreamNonBlocking, hi);
            if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, lo);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->evP, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->evB, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&h->side2, cudaStreamNonBlocking, lo);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->evP2, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->evI, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&h->side3, cudaStreamNonBlocking, lo);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->evS, cudaEventDisableTiming);
            for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&h->evF[k], cudaEventDisableTiming);
            if (e != cudaSuccess) rc = set_err(h, SPK_ECUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
            h->stream = h->own;
        }
    }
    if (rc == SPK_OK) rc = upload_structure(h);
    if (rc != SPK_OK) {
        g_create_err = h->err;
        spk_destroy(h);
        return rc;
    }
    *out = h;
    return SPK_OK;
}

int spk_set_stream(spk_handle* h, void* stream) {
    int rc = check_h(h);
    if (rc) return rc;
    h->stream = stream ? (cudaStream_t)stream : h->own;
    return SPK_OK;
}

int spk_set_pattern(spk_handle* h, int64_t ncols, const int64_t* colptr, const int64_t* rowval, const int64_t* rperm,
                    const int64_t* rinvp, int index_base) {
    int rc = check_h(h);
    if (rc) return rc;
    const i64 n = h->n;
    if (ncols != n || !colptr || !rowval || !rperm || !rinvp || (index_base != 0 && index_base != 1))
        return set_err(h, SPK_EARG, "spk_set_pattern: bad arguments");
    const int b = index_base;
    h->rperm0.resize(n);
    h->rinvp0.resize(n);
    for (i64 i = 0; i < n; ++i) {
        i64 p = rperm[i] - b, q = rinvp[i] - b;
        if (p < 0 || p >= n || q < 0 || q >= n) return set_err(h, SPK_EARG, "spk_set_pattern: permutation out of range");
        h->rperm0[i] = (int)p;
        h->rinvp0[i] = (int)q;
    }
    for (i64 i = 0; i < n; ++i)
        if (h->rinvp0[h->rperm0[i]] != i) return set_err(h, SPK_EARG, "spk_set_pattern: rperm and rinvp are not inverse");
    const i64 nnz = colptr[n] - colptr[0];
    if (nnz < 0) return set_err(h, SPK_EARG, "spk_set_pattern: bad colptr");
    std::vector<ll> slot(nnz);
    std::vector<int> rowcount(n + 1, 0);
    for (i64 j = 0; j < n; ++j) {
        for (i64 k = colptr[j] - b; k < colptr[j + 1] - b; ++k) {
            i64 i = rowval[k] - b;
            if (i < 0 || i >= n) return set_err(h, SPK_EARG, "spk_set_pattern: row index out of range");
            rowcount[i + 1]++;
            const int inew = h->rinvp0[i], jnew = h->rinvp0[j];
            const HFront& F = h->fronts[h->col_front[jnew]];
            ll s = -1;
            if (!in_structure(h, inew, jnew)) {
                s = -1;
            } else if (inew >= F.f && inew < F.f + F.nf) {
                s = F.loff + (ll)(jnew - F.f) * (F.nf + F.m) + (inew - F.f);
            } else if (inew > jnew) {
                const int* R = h->rows.data() + F.rows_off;
                const int* q = std::lower_bound(R, R + F.m, inew);
                if (q != R + F.m && *q == inew) s = F.loff + (ll)(jnew - F.f) * (F.nf + F.m) + F.nf + (q - R);
            } else {
                const HFront& G = h->fronts[h->col_front[inew]];
                const int* R = h->rows.data() + G.rows_off;
                const int* q = std::lower_bound(R, R + G.m, jnew);
                if (q != R + G.m && *q == jnew) s = G.uoff + (ll)(inew - G.f) * G.m + (q - R);
            }
            if (s < 0) {
                char buf[160];
                std::snprintf(buf, sizeof buf, "No space for matrix element (%lld, %lld).", (long long)inew + 1,
                              (long long)jnew + 1);
                return set_err(h, SPK_ESTRUCT, buf);
            }
            slot[k - (colptr[0] - b)] = s;
        }
    }
    // row-ordered pattern for the residual
    for (i64 i = 0; i < n; ++i) rowcount[i + 1] += rowcount[i];
    std::vector<int> rowptr(rowcount), col(nnz);
    std::vector<ll> src(nnz);
    {
        std::vector<int> next(rowcount.begin(), rowcount.end() - 1);
        for (i64 j = 0; j < n; ++j)
            for (i64 k = colptr[j] - b; k < colptr[j + 1] - b; ++k) {
                i64 i = rowval[k] - b;
                int at = next[i]++;
                col[at] = (int)j;
                src[at] = k - (colptr[0] - b);
            }
    }
    std::vector<int> ccolptr(n + 1), crow(nnz), ccol(nnz);
    for (i64 j = 0; j <= n; ++j) ccolptr[j] = (int)(colptr[j] - colptr[0]);
    for (i64 j = 0; j < n; ++j)
        for (i64 k = colptr[j] - b; k < colptr[j + 1] - b; ++k) {
            crow[k - (colptr[0] - b)] = (int)(rowval[k] - b);
            ccol[k - (colptr[0] - b)] = (int)j;
        }
    cudaFree(h->d_ccolptr); cudaFree(h->d_crow); cudaFree(h->d_ccol);
    h->d_ccolptr = h->d_crow = h->d_ccol = nullptr;
    if ((rc = upload(h, &h->d_ccolptr, ccolptr))) return rc;
    if ((rc = upload(h, &h->d_crow, crow))) return rc;
    if ((rc = upload(h, &h->d_ccol, ccol))) return rc;
    cudaFree(h->d_slot); cudaFree(h->d_aval); cudaFree(h->d_acsr); cudaFree(h->d_rowptr); cudaFree(h->d_col);
    cudaFree(h->d_src);
    cudaFree(h->d_rperm); cudaFree(h->d_rinvp);
    h->d_slot = nullptr; h->d_aval = nullptr; h->d_acsr = nullptr; h->d_rowptr = h->d_col = nullptr; h->d_src = nullptr;
    h->d_rperm = h->d_rinvp = nullptr;
    if ((rc = upload(h, &h->d_slot, slot))) return rc;
    if ((rc = upload(h, &h->d_rowptr, rowptr))) return rc;
    if ((rc = upload(h, &h->d_col, col))) return rc;
    if ((rc = upload(h, &h->d_src, src))) return rc;
    if ((rc = upload(h, &h->d_rperm, h->rperm0))) return rc;
    if ((rc = upload(h, &h->d_rinvp, h->rinvp0))) return rc;
    CU(h, cudaMalloc((void**)&h->d_aval, sizeof(double) * std::max<i64>(nnz, 1)));
    CU(h, cudaMalloc((void**)&h->d_acsr, sizeof(double) * std::max<i64>(nnz, 1)));
    h->nnz = nnz;
    h->have_pattern = true;
    h->have_values = false;
    for (int y = 0; y < 2; ++y) {
        h->s64[y].loaded = h->s64[y].factored = false;
        h->s32[y].loaded = h->s32[y].factored = false;
        h->s16[y].loaded = h->s16[y].factored = false;
    }
    return SPK_OK;
}


int spk_load_values(spk_handle* h, const double* nzval, int where, int precision) {
    int rc = check_h(h);
    if (rc) return rc;
    if (!h->have_pattern) return set_err(h, SPK_ESEQ, "Sequence error. Pattern not set yet.");
    if ((!nzval && h->nnz > 0) || (where != SPK_HOST && where != SPK_DEVICE) || !valid_precision(precision))
        return set_err(h, SPK_EARG, "spk_load_values: bad arguments");
    if (h->nnz > 0) {
        CU(h, cudaMemcpyAsync(h->d_aval, nzval, sizeof(double) * (size_t)h->nnz,
                              where == SPK_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, h->stream));
        LaunchScope ls(h, SPK_K_ASSEMBLE, 0.0, (double)h->nnz * (8 + 8 + 8));
        spk::k_gather_csr<<<(int)std::min<i64>((h->nnz + 255) / 256, 152 * 16), 256, 0, h->stream>>>(
            h->d_aval, h->d_src, h->d_acsr, h->nnz);
    }
    h->have_values = true;
    // a new A invalidates every factor
    for (int y = 0; y < 2; ++y) {
        h->s64[y].loaded = h->s64[y].factored = false;
        h->s32[y].loaded = h->s32[y].factored = false;
        h->s16[y].loaded = h->s16[y].factored = false;
    }
    select_form(h, precision);
    rc = is_fp64(precision) ? load_into<double>(h) : load_into<float>(h);
    if (rc) return rc;
    if (where == SPK_HOST) CU(h, cudaStreamSynchronize(h->stream));
    return SPK_OK;
}

int spk_factor(spk_handle* h, int precision, int64_t* first_singular) {
    int rc = check_h(h);
    if (rc) return rc;
    if (first_singular) *first_singular = 0;
    if (!valid_precision(precision)) return set_err(h, SPK_EARG, "spk_factor: bad precision");
    if (!h->have_values) return set_err(h, SPK_ESEQ, "Sequence error. Matrix input not done yet.");
    select_form(h, precision);
    if (is_fp64(precision)) {
        if (!storage<double>(h).loaded && (rc = load_into<double>(h))) return rc;
        if ((rc = run_factor<double>(h))) return rc;
    } else {
        if (!float_storage(h, precision).loaded && (rc = load_into<float>(h))) return rc;
        if ((rc = run_factor<float>(h))) return rc;
    }
    int info2[3] = {INT_MAX, 0, 0};
    CU(h, cudaMemcpyAsync(info2, h->d_info, sizeof(info2), cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    const int info = info2[0];
    if (info2[1] || info2[2]) {   // the factors are invalid; the next factor reassembles A
        if (is_fp64(precision)) storage<double>(h).loaded = storage<double>(h).factored = false;
        else float_storage(h, precision).loaded = float_storage(h, precision).factored = false;
        return set_err(h, SPK_ETIMEOUT, info2[2] ? "spk_factor: a leaf-queue dependency wait timed out"
                                                 : "spk_factor: a tensor-core wait timed out");
    }
    if (is_fp64(precision)) { storage<double>(h).loaded = false; storage<double>(h).factored = true; }
    else { float_storage(h, precision).loaded = false; float_storage(h, precision).factored = true; }
    if (info != INT_MAX) {
        if (first_singular) *first_singular = info;
        char buf[128];
        std::snprintf(buf, sizeof buf, "zero pivot in the diagonal block of supernode %d", info);
        return set_err(h, SPK_ESINGULAR, buf);
    }
    return SPK_OK;
}


// Drop what depends on the float plans' tensor-core partition: the plans,
// their packs, graphs and factors (the next factor reassembles A).
static void reset_float_plans(spk_handle* h) {
    for (int y = 0; y < 2; ++y) {
        free_plan(h->plan[1 + 2 * y]);
        for (Storage<float>* S : {&h->s32[y], &h->s16[y]}) {
            if (S->pack) cudaFree(S->pack);
            S->pack = nullptr;
            S->loaded = S->factored = false;
        }
    }
    drop_factor_graphs(h);
    drop_solve_graphs(h);
}

// Drop every plan and captured graph but keep the factors (an option that
// changes only the solves' launch lists).
static void reset_plans_keep_factors(spk_handle* h) {
    for (Plan& P : h->plan) free_plan(P);
    drop_factor_graphs(h);
    drop_solve_graphs(h);
}

int spk_set_option(spk_handle* h, int option, int64_t value) {
    int rc = check_h(h);
    if (rc) return rc;
    switch (option) {
    case SPK_OPT_LEAF_QUEUE:
        if (value != 0 && value != 1) break;
        h->leaf_queue = (int)value;
        drop_factor_graphs(h);
        return SPK_OK;
    case SPK_OPT_WAIT_BUDGET:
        if (value < 1 || value > 0xffffffffLL) break;
        h->wait_budget = value;
        drop_factor_graphs(h);
        return SPK_OK;
    case SPK_OPT_STALL_TEST:
        if (value < -1 || value > INT_MAX) break;
        h->stall_test = (int)value;
        drop_factor_graphs(h);
        return SPK_OK;
    case SPK_OPT_SOLVE_CLUSTER_MINB:
        if (value < 2 || value > spk::FC * spk::FC_OWN) break;
        if (h->fc_minb != (int)value) {
            h->fc_minb = (int)value;
            reset_plans_keep_factors(h);
        }
        return SPK_OK;
    case SPK_OPT_LU_PIECES:
        if (value != 0 && value != 1) break;
        h->lu_pieces = (int)value;
        drop_factor_graphs(h);
        return SPK_OK;
    case SPK_OPT_PANEL_SPLIT:
        if (value != 0 && value != 1) break;
        h->panel_split = (int)value;
        drop_factor_graphs(h);
        return SPK_OK;
    case SPK_OPT_SCHUR_SPLIT:
        if (value != 0 && value != 1) break;
        h->schur_split = (int)value;
        drop_factor_graphs(h);
        return SPK_OK;
    case SPK_OPT_SCHUR_FAR_SMS:
        if (value < 0 || value > 4096) break;
        h->schur_far_sms = (int)value;
        drop_factor_graphs(h);
        return SPK_OK;
    case SPK_OPT_SOLVE_CHUNK:
        if (value != 0 && value != 1) break;
        if (h->solve_chunk != (int)value) {
            h->solve_chunk = (int)value;
            reset_plans_keep_factors(h);
        }
        return SPK_OK;
    case SPK_OPT_TC_SCHUR_M:
    case SPK_OPT_TC_TRAIL_ROWS:
    case SPK_OPT_TC_WIDE: {
        if (value < (option == SPK_OPT_TC_WIDE ? 0 : 1) || value > (option == SPK_OPT_TC_WIDE ? 1 : INT_MAX)) break;
        int& field = option == SPK_OPT_TC_SCHUR_M ? h->tc_schur_m
                     : option == SPK_OPT_TC_TRAIL_ROWS ? h->tc_trail_rows : h->tc_wide;
        if (field != (int)value) {
            field = (int)value;
            reset_float_plans(h);
        }
        return SPK_OK;
    }
    default:
        break;
    }
    return set_err(h, SPK_EARG, "spk_set_option: unknown option or value out of range");
}

int spk_get_option(spk_handle* h, int option, int64_t* value) {
    int rc = check_h(h);
    if (rc) return rc;
    if (!value) return set_err(h, SPK_EARG, "spk_get_option: value is NULL");
    switch (option) {
    case SPK_OPT_LEAF_QUEUE: *value = h->leaf_queue; return SPK_OK;
    case SPK_OPT_WAIT_BUDGET: *value = h->wait_budget; return SPK_OK;
    case SPK_OPT_STALL_TEST: *value = h->stall_test; return SPK_OK;
    case SPK_OPT_TC_SCHUR_M: *value = h->tc_schur_m; return SPK_OK;
    case SPK_OPT_TC_TRAIL_ROWS: *value = h->tc_trail_rows; return SPK_OK;
    case SPK_OPT_TC_WIDE: *value = h->tc_wide; return SPK_OK;
    case SPK_OPT_LU_PIECES: *value = h->lu_pieces; return SPK_OK;
    case SPK_OPT_SOLVE_CLUSTER_MINB: *value = h->fc_minb; return SPK_OK;
    case SPK_OPT_PANEL_SPLIT: *value = h->panel_split; return SPK_OK;
    case SPK_OPT_SCHUR_SPLIT: *value = h->schur_split; return SPK_OK;
    case SPK_OPT_SCHUR_FAR_SMS: *value = h->schur_far_sms; return SPK_OK;
    case SPK_OPT_SOLVE_CHUNK: *value = h->solve_chunk; return SPK_OK;
    default: return set_err(h, SPK_EARG, "spk_get_option: unknown option");
    }
}

}  // extern "C"

// Factor time of the current options: `reps` timed factorisations (CUDA
// events on the handle's stream) after one untimed, each of freshly
// assembled values; the median.
template <typename T>
static int time_factor(spk_handle* h, int reps, double* ms) {
    cudaEvent_t e0, e1;
    CU(h, cudaEventCreate(&e0));
    CU(h, cudaEventCreate(&e1));
    std::vector<double> t;
    int rc = SPK_OK;
    for (int r = 0; r <= reps && rc == SPK_OK; ++r) {
        if ((rc = load_into<T>(h))) break;
        if (cudaEventRecord(e0, h->stream) != cudaSuccess) { rc = set_err(h, SPK_ECUDA, "cudaEventRecord"); break; }
        if ((rc = run_factor<T>(h))) break;
        if (cudaEventRecord(e1, h->stream) != cudaSuccess) { rc = set_err(h, SPK_ECUDA, "cudaEventRecord"); break; }
        int info[3] = {INT_MAX, 0, 0};
        float f = 0.f;
        if (cudaMemcpyAsync(info, h->d_info, sizeof(info), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess || cudaEventElapsedTime(&f, e0, e1) != cudaSuccess) {
            rc = set_err(h, SPK_ECUDA, "spk_autotune: timing failed");
            break;
        }
        if (info[1] || info[2]) rc = set_err(h, SPK_ETIMEOUT, "spk_autotune: a device wait timed out");
        if (r > 0) t.push_back(f);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return SPK_OK;
}

extern "C" {

int spk_autotune(spk_handle* h, int precision, int reps, double* best_ms) {
    int rc = check_h(h);
    if (rc) return rc;
    if (!valid_precision(precision) || reps < 1) return set_err(h, SPK_EARG, "spk_autotune: bad arguments");
    if (!h->have_values) return set_err(h, SPK_ESEQ, "Sequence error. Matrix input not done yet.");
    if (h->prof_mask) return set_err(h, SPK_ESEQ, "spk_autotune: event timing (spk_profile) is on");
    select_form(h, precision);
    const bool f64 = is_fp64(precision);
    auto measure = [&](double* ms) { return f64 ? time_factor<double>(h, reps, ms) : time_factor<float>(h, reps, ms); };
    // the leaf queue on or off
    double best = 0.0, ms = 0.0;
    int best_q = h->leaf_queue;
    for (int q = 0; q < 2; ++q) {
        if ((rc = spk_set_option(h, SPK_OPT_LEAF_QUEUE, q))) return rc;
        if ((rc = measure(&ms))) return rc;
        if (q == 0 || ms < best) { best = ms; best_q = q; }
    }
    if ((rc = spk_set_option(h, SPK_OPT_LEAF_QUEUE, best_q))) return rc;
    if (!f64) {   // the tensor-core partition of the float forms
        static const int cand[][2] = {{96, 128}, {64, 128}, {128, 128}, {192, 128}, {96, 256}, {128, 256}, {256, 256}};
        const int s0 = h->tc_schur_m, t0 = h->tc_trail_rows;   // `best` was measured with these
        int bs = s0, bt = t0;
        for (const auto& c : cand) {
            if (c[0] == s0 && c[1] == t0) continue;
            if ((rc = spk_set_option(h, SPK_OPT_TC_SCHUR_M, c[0]))) return rc;
            if ((rc = spk_set_option(h, SPK_OPT_TC_TRAIL_ROWS, c[1]))) return rc;
            if ((rc = measure(&ms))) return rc;
            if (ms < best) { best = ms; bs = c[0]; bt = c[1]; }
        }
        if ((rc = spk_set_option(h, SPK_OPT_TC_SCHUR_M, bs))) return rc;
        if ((rc = spk_set_option(h, SPK_OPT_TC_TRAIL_ROWS, bt))) return rc;
        const int w0 = h->tc_wide;   // then the Schur tile width
        if ((rc = spk_set_option(h, SPK_OPT_TC_WIDE, 1 - w0))) return rc;
        if ((rc = measure(&ms))) return rc;
        if (ms < best) best = ms;
        else if ((rc = spk_set_option(h, SPK_OPT_TC_WIDE, w0))) return rc;
    }
    // leave A assembled in the chosen form, ready for spk_factor
    if ((rc = f64 ? load_into<double>(h) : load_into<float>(h))) return rc;
    CU(h, cudaStreamSynchronize(h->stream));
    if (best_ms) *best_ms = best;
    return SPK_OK;
}

static int solve_impl(spk_handle* h, double* b, int64_t nrhs, int64_t ldb, int where, int precision, bool transpose) {
    int rc = check_h(h);
    if (rc) return rc;
    if (!valid_precision(precision) || nrhs < 0 || (nrhs > 0 && (!b || ldb < h->n)) ||
        (where != SPK_HOST && where != SPK_DEVICE))
        return set_err(h, SPK_EARG, "spk_solve: bad arguments");
    if (!factored(h, precision)) return set_err(h, SPK_ESEQ, "Sequence error. Factorization not done yet.");
    if (nrhs == 0) return SPK_OK;
    if ((rc = ensure_rhs(h, nrhs))) return rc;
    select_form(h, precision);
    const i64 n = h->n;
    double* src;
    i64 ld;
    if (where == SPK_HOST) {
        CU(h, cudaMemcpy2DAsync(h->d_rhs, sizeof(double) * n, b, sizeof(double) * ldb, sizeof(double) * n, nrhs,
                                cudaMemcpyHostToDevice, h->stream));
        src = h->d_rhs;
        ld = n;
    } else {
        src = b;
        ld = ldb;
    }
    rc = is_fp64(precision) ? solve_device<double>(h, src, ld, h->d_x, n, nrhs, 0, transpose)
                               : solve_device<float>(h, src, ld, h->d_x, n, nrhs, 0, transpose);
    if (rc) return rc;
    CU(h, cudaMemcpy2DAsync(b, sizeof(double) * ldb, h->d_x, sizeof(double) * n, sizeof(double) * n, nrhs,
                            where == SPK_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    return SPK_OK;
}

int spk_solve(spk_handle* h, double* b, int64_t nrhs, int64_t ldb, int where, int precision) {
    return solve_impl(h, b, nrhs, ldb, where, precision, false);
}

int spk_solve_transpose(spk_handle* h, double* b, int64_t nrhs, int64_t ldb, int where, int precision) {
    return solve_impl(h, b, nrhs, ldb, where, precision, true);
}

int spk_residual(spk_handle* h, const double* b, const double* x, int64_t nrhs, int64_t ld, int where,
                 double* relres) {
    int rc = check_h(h);
    if (rc) return rc;
    if (!relres || nrhs <= 0 || !b || !x || ld < h->n || (where != SPK_HOST && where != SPK_DEVICE))
        return set_err(h, SPK_EARG, "spk_residual: bad arguments");
    if (!h->have_values) return set_err(h, SPK_ESEQ, "Sequence error. Matrix input not done yet.");
    if ((rc = ensure_rhs(h, nrhs))) return rc;
    const i64 n = h->n;
    const double *db = b, *dx = x;
    i64 ldb = ld, ldx = ld;
    if (where == SPK_HOST) {
        CU(h, cudaMemcpy2DAsync(h->d_rhs, sizeof(double) * n, b, sizeof(double) * ld, sizeof(double) * n, nrhs,
                                cudaMemcpyHostToDevice, h->stream));
        CU(h, cudaMemcpy2DAsync(h->d_x, sizeof(double) * n, x, sizeof(double) * ld, sizeof(double) * n, nrhs,
                                cudaMemcpyHostToDevice, h->stream));
        db = h->d_rhs;
        dx = h->d_x;
        ldb = ldx = n;
    }
    return residual_device(h, db, ldb, dx, ldx, nrhs, relres);
}

}  // extern "C"

// Work space of spk_residual_noalloc: the two sums of squares of each
// right-hand side.  A file-scope device array, so the entry point allocates
// nothing; every device that loads this library holds it until exit.  Host
// code only sees a stand-in for it: its device address is fetched once per
// device with cudaGetSymbolAddress (with that device current) and cached.
static __device__ __align__(256) double g_noalloc_sums[2 * SPK_NOALLOC_MAX_RHS];
static std::mutex g_noalloc_mutex;
static double* g_noalloc_ptr[64];

static int noalloc_scratch(spk_handle* h, double** out) {
    if (h->device < 0 || h->device >= 64) return set_err(h, SPK_EARG, "spk_residual_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[h->device]) {
        double* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_sums);
        if (e != cudaSuccess)
            return set_err(h, SPK_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_ptr[h->device] = p;
    }
    *out = g_noalloc_ptr[h->device];
    return SPK_OK;
}

extern "C" {

int spk_residual_noalloc(spk_handle* h, const double* b, const double* x, int64_t nrhs, int64_t ld, double* relres) {
    int rc = check_h(h);
    if (rc) return rc;
    if (!relres || !b || !x || nrhs <= 0 || ld < h->n) return set_err(h, SPK_EARG, "spk_residual_noalloc: bad arguments");
    if (nrhs > SPK_NOALLOC_MAX_RHS)
        return set_err(h, SPK_EARG, "spk_residual_noalloc: at most SPK_NOALLOC_MAX_RHS (64) right-hand sides per call");
    if (!h->have_values) return set_err(h, SPK_ESEQ, "Sequence error. Matrix input not done yet.");
    {   // the call ends with a wait for the stream, which a capture does not allow: refuse before any work
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CU(h, cudaStreamIsCapturing(h->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return set_err(h, SPK_ESEQ, "spk_residual_noalloc: the handle's stream is being captured (the call waits "
                                        "for the stream); call it outside the capture");
    }
    double* sums = nullptr;
    if ((rc = noalloc_scratch(h, &sums))) return rc;
    const int n = (int)h->n;
    CU(h, cudaMemsetAsync(sums, 0, sizeof(double) * 2 * (size_t)nrhs, h->stream));
    dim3 grid(std::min((n + 255) / 256, 8 * h->nsm));
    spk::k_residual_norms<<<grid, 256, 0, h->stream>>>(h->d_acsr, h->d_rowptr, h->d_col, nullptr, x, ld, b, ld, n,
                                                       (int)nrhs, sums);
    CU(h, cudaGetLastError());
    double host[2 * SPK_NOALLOC_MAX_RHS];
    CU(h, cudaMemcpyAsync(host, sums, sizeof(double) * 2 * (size_t)nrhs, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    double worst = 0.0;
    for (i64 j = 0; j < nrhs; ++j) {
        double nb = std::sqrt(host[2 * j + 1]), nr = std::sqrt(host[2 * j]);
        double rel = nb > 0.0 ? nr / nb : nr;
        if (!(rel <= worst)) worst = rel;
    }
    *relres = worst;
    return SPK_OK;
}

// first_done: the first solve has run (spk_factor_refine): its solution is
// in x (device) or d_x (host b), and a host b is already in d_rhs.
static int refine_impl(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where, int precision,
                       double tol, int max_iter, int solver, int* iters, double* relres, int* solver_used,
                       bool transpose, bool first_done = false) {
    int rc = check_h(h);
    if (rc) return rc;
    if (iters) *iters = 0;
    if (solver_used) *solver_used = SPK_SOLVER_IR;
    if (!valid_precision(precision) || nrhs <= 0 || !b || !x || ld < h->n || max_iter < 0 ||
        (where != SPK_HOST && where != SPK_DEVICE) || solver < SPK_SOLVER_AUTO || solver > SPK_SOLVER_GMRES ||
        (transpose && solver == SPK_SOLVER_GMRES))
        return set_err(h, SPK_EARG, "spk_refine: bad arguments");
    if (!factored(h, precision)) return set_err(h, SPK_ESEQ, "Sequence error. Factorization not done yet.");
    if ((rc = ensure_rhs(h, nrhs))) return rc;
    select_form(h, precision);
    const i64 n = h->n;
    const double* db;
    double* dx;
    i64 ldb, ldx;
    if (where == SPK_HOST) {
        if (!first_done)
            CU(h, cudaMemcpy2DAsync(h->d_rhs, sizeof(double) * n, b, sizeof(double) * ld, sizeof(double) * n, nrhs,
                                    cudaMemcpyHostToDevice, h->stream));
        db = h->d_rhs;
        dx = h->d_x;
        ldb = ldx = n;
    } else {
        db = b;
        dx = x;
        ldb = ldx = ld;
    }
    auto solve_into = [&](const double* rhs, i64 ldr, int acc) {
        return is_fp64(precision) ? solve_device<double>(h, rhs, ldr, dx, ldx, nrhs, acc, transpose)
                                     : solve_device<float>(h, rhs, ldr, dx, ldx, nrhs, acc, transpose);
    };
    if (!first_done && (rc = solve_into(db, ldb, 0))) return rc;
    double rel = 0.0, prev = 0.0;
    int it = 0;
    bool gmres = solver == SPK_SOLVER_GMRES;
    // AUTO: plain refinement while every correction at least halves the
    // residual; on the first that does not, take back a correction that made
    // it worse and continue with GMRES-IR from there (not for A^T).
    const bool can_switch = solver == SPK_SOLVER_AUTO && !transpose;
    const bool backup = can_switch && nrhs <= spk::GM_MAXRHS;   // x before each correction, in gm_w
    for (;;) {
        if ((rc = residual_device(h, db, ldb, dx, ldx, nrhs, &rel, transpose))) return rc;
        if (rel <= tol || it >= max_iter || rel != rel) break;
        if (it > 0 && can_switch && !(rel <= 0.5 * prev)) {
            if (backup && !(rel <= prev)) {   // take the last correction back
                CU(h, cudaMemcpy2DAsync(dx, sizeof(double) * ldx, h->gm_w, sizeof(double) * n, sizeof(double) * n,
                                        nrhs, cudaMemcpyDeviceToDevice, h->stream));
                rel = prev;
            }
            gmres = true;
        }
        if (gmres) break;
        if (backup) {
            if ((rc = ensure_gmres(h))) return rc;
            CU(h, cudaMemcpy2DAsync(h->gm_w, sizeof(double) * n, dx, sizeof(double) * ldx, sizeof(double) * n, nrhs,
                                    cudaMemcpyDeviceToDevice, h->stream));
        }
        prev = rel;
        if ((rc = solve_into(h->d_r, n, 1))) return rc;
        ++it;
    }
    if (gmres && !(rel <= tol) && rel == rel) {
        if (solver_used) *solver_used = SPK_SOLVER_GMRES;
        double worst = 0.0;
        for (i64 c0 = 0; c0 < nrhs; c0 += spk::GM_MAXRHS) {
            const int nc = (int)std::min<i64>(spk::GM_MAXRHS, nrhs - c0);
            double r = 0.0;
            int used = 0, cycles = 0;
            rc = is_fp64(precision)
                     ? gmres_ir<double>(h, db + c0 * ldb, ldb, dx + c0 * ldx, ldx, nc, tol, max_iter - it, &r, &used, &cycles)
                     : gmres_ir<float>(h, db + c0 * ldb, ldb, dx + c0 * ldx, ldx, nc, tol, max_iter - it, &r, &used, &cycles);
            if (rc) return rc;
            it += used;
            if (!(r <= worst)) worst = r;
        }
        rel = worst;
    }
    if (where == SPK_HOST)
        CU(h, cudaMemcpy2DAsync(x, sizeof(double) * ld, dx, sizeof(double) * n, sizeof(double) * n, nrhs,
                                cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    if (iters) *iters = it;
    if (relres) *relres = rel;
    if (!(rel <= tol)) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "refinement stopped at relative residual %.3e after %d preconditioned solves",
                      rel, it);
        return set_err(h, SPK_ENOCONV, buf);
    }
    return SPK_OK;
}

int spk_refine(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where, int precision,
               double tol, int max_iter, int* iters, double* relres) {
    return refine_impl(h, b, x, nrhs, ld, where, precision, tol, max_iter, SPK_SOLVER_AUTO, iters, relres, nullptr,
                       false);
}

int spk_refine_ex(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where, int precision,
                  double tol, int max_iter, int solver, int* iters, double* relres, int* solver_used) {
    return refine_impl(h, b, x, nrhs, ld, where, precision, tol, max_iter, solver, iters, relres, solver_used, false);
}

}  // extern "C"

// Factorisation and the first solve of the refinement, the forward
// substitution of the lower levels overlapped with the last levels of the
// factorisation; then refinement as spk_refine_ex.
template <typename T>
static int factor_refine_first(spk_handle* h, int nrhs, double* dx, i64 ldx, int64_t* first_singular) {
    static const int init[3] = {INT_MAX, 0, 0};
    int rc = ensure_plan<T>(h);
    if (rc) return rc;
    CU(h, cudaMemcpyAsync(h->d_info, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    const int gi = graph_index<T>(h);
    if ((rc = via_graph(h, h->g_factor_fs[gi][nrhs], [&] { return factor_launches<T>(h, nrhs); }))) return rc;
    int info[3] = {INT_MAX, 0, 0};
    CU(h, cudaMemcpyAsync(info, h->d_info, sizeof(info), cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    Storage<T>& St = storage<T>(h);
    St.loaded = false;
    if (info[1] || info[2]) {
        St.factored = false;
        return set_err(h, SPK_ETIMEOUT, info[2] ? "spk_factor_refine: a leaf-queue dependency wait timed out"
                                                : "spk_factor_refine: a tensor-core wait timed out");
    }
    St.factored = true;
    if (info[0] != INT_MAX) {
        if (first_singular) *first_singular = info[0];
        char buf[128];
        std::snprintf(buf, sizeof buf, "zero pivot in the diagonal block of supernode %d", info[0]);
        return set_err(h, SPK_ESINGULAR, buf);
    }
    const size_t split = fused_split<T>(h);
    const Plan& PL = h->plan[plan_index<T>(h)];
    rc = via_graph(h, h->g_fs_tail[gi][nrhs], [&] {
        if (split == 0) {   // nothing of this solve ran beside the factorisation
            const ll tot = (ll)h->n * nrhs;
            LaunchScope ls(h, SPK_K_PERMUTE, 0.0, (double)tot * (8 + 4 + sizeof(T)));
            spk::k_permute<double, T><<<(int)((tot + 255) / 256), 256, 0, h->stream>>>(
                h->d_rhs, h->n, (T*)h->d_wb, (int)h->n, h->d_rperm, (int)h->n, nrhs);
        }
        int r = solve_fwd_levels<T>(h, nrhs, split, PL.levels.size(), h->stream);
        return r ? r : solve_bwd_levels<T>(h, nrhs, h->stream);
    });
    if (rc) return rc;
    const ll tot = (ll)h->n * nrhs;
    LaunchScope ls(h, SPK_K_PERMUTE, 0.0, (double)tot * (8 + 4 + sizeof(T)));
    spk::k_unpermute<T><<<(int)((tot + 255) / 256), 256, 0, h->stream>>>((const T*)h->d_wx, (int)h->n, dx, ldx,
                                                                        h->d_rinvp, (int)h->n, nrhs, 0);
    CU(h, cudaGetLastError());
    return SPK_OK;
}

extern "C" {

int spk_factor_refine(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where, int precision,
                      double tol, int max_iter, int solver, int* iters, double* relres, int* solver_used,
                      int64_t* first_singular) {
    int rc = check_h(h);
    if (rc) return rc;
    if (first_singular) *first_singular = 0;
    if (!valid_precision(precision) || nrhs <= 0 || !b || !x || ld < h->n || max_iter < 0 ||
        (where != SPK_HOST && where != SPK_DEVICE) || solver < SPK_SOLVER_AUTO || solver > SPK_SOLVER_GMRES)
        return set_err(h, SPK_EARG, "spk_factor_refine: bad arguments");
    if (!h->have_values) return set_err(h, SPK_ESEQ, "Sequence error. Matrix input not done yet.");
    if (nrhs > spk::MAXRHS) {   // beyond one solve pass: factor, then refine
        if ((rc = spk_factor(h, precision, first_singular))) return rc;
        return refine_impl(h, b, x, nrhs, ld, where, precision, tol, max_iter, solver, iters, relres, solver_used,
                           false);
    }
    select_form(h, precision);
    const bool f64 = is_fp64(precision);
    if (f64 ? !storage<double>(h).loaded : !float_storage(h, precision).loaded)
        if ((rc = f64 ? load_into<double>(h) : load_into<float>(h))) return rc;
    if ((rc = ensure_rhs(h, nrhs))) return rc;
    const i64 n = h->n;
    CU(h, cudaMemcpy2DAsync(h->d_rhs, sizeof(double) * n, b, sizeof(double) * ld, sizeof(double) * n, nrhs,
                            where == SPK_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, h->stream));
    double* dx = where == SPK_HOST ? h->d_x : x;
    const i64 ldx = where == SPK_HOST ? n : ld;
    rc = f64 ? factor_refine_first<double>(h, (int)nrhs, dx, ldx, first_singular)
             : factor_refine_first<float>(h, (int)nrhs, dx, ldx, first_singular);
    if (rc) return rc;
    return refine_impl(h, b, x, nrhs, ld, where, precision, tol, max_iter, solver, iters, relres, solver_used, false,
                       true);
}

int spk_refine_transpose(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where, int precision,
                         double tol, int max_iter, int* iters, double* relres) {
    return refine_impl(h, b, x, nrhs, ld, where, precision, tol, max_iter, SPK_SOLVER_IR, iters, relres, nullptr,
                       true);
}

int spk_grad_pattern(spk_handle* h, const double* lambda, const double* x, int64_t nrhs, int64_t ld, int where,
                     double* dA) {
    int rc = check_h(h);
    if (rc) return rc;
    if (!h->have_pattern) return set_err(h, SPK_ESEQ, "Sequence error. Pattern not set yet.");
    if (nrhs <= 0 || ld < h->n || !lambda || !x || (!dA && h->nnz > 0) || (where != SPK_HOST && where != SPK_DEVICE))
        return set_err(h, SPK_EARG, "spk_grad_pattern: bad arguments");
    if (h->nnz == 0) return SPK_OK;
    const i64 n = h->n;
    const double *dl = lambda, *dxp = x;
    double* dg = dA;
    double* tmp = nullptr;
    i64 ldd = ld;
    if (where == SPK_HOST) {   // staged through the handle's work vectors
        if ((rc = ensure_rhs(h, nrhs))) return rc;
        CU(h, cudaMemcpy2DAsync(h->d_rhs, sizeof(double) * n, lambda, sizeof(double) * ld, sizeof(double) * n, nrhs,
                                cudaMemcpyHostToDevice, h->stream));
        CU(h, cudaMemcpy2DAsync(h->d_x, sizeof(double) * n, x, sizeof(double) * ld, sizeof(double) * n, nrhs,
                                cudaMemcpyHostToDevice, h->stream));
        CU(h, cudaMallocAsync((void**)&tmp, sizeof(double) * (size_t)h->nnz, h->stream));
        dl = h->d_rhs;
        dxp = h->d_x;
        dg = tmp;
        ldd = n;
    }
    const int blocks = (int)std::min<i64>((h->nnz + 255) / 256, 152 * 16);
    spk::k_grad_pattern<<<blocks, 256, 0, h->stream>>>(h->d_crow, h->d_ccol, dl, dxp, ldd, (int)nrhs, dg, h->nnz);
    CU(h, cudaGetLastError());
    if (where == SPK_HOST) {
        CU(h, cudaMemcpyAsync(dA, tmp, sizeof(double) * (size_t)h->nnz, cudaMemcpyDeviceToHost, h->stream));
        CU(h, cudaFreeAsync(tmp, h->stream));
    }
    CU(h, cudaStreamSynchronize(h->stream));
    return SPK_OK;
}

int spk_get_factors(spk_handle* h, int precision, double* lnz, double* unz, int64_t* ipiv) {
    int rc = check_h(h);
    if (rc) return rc;
    if (!valid_precision(precision)) return set_err(h, SPK_EARG, "spk_get_factors: bad precision");
    const bool done = factored(h, precision);
    const bool loaded = is_fp64(precision) ? h->s64[(precision & SPK_SPD) ? 1 : 0].loaded : float_storage(h, precision).loaded;
    select_form(h, precision);
    if (!done && !loaded) return set_err(h, SPK_ESEQ, "Sequence error. Matrix input not done yet.");
    std::vector<double> fac;
    rc = is_fp64(precision) ? fetch_factor<double>(h, fac) : fetch_factor<float>(h, fac);
    if (rc) return rc;
    // SPD form: the stored factor is the unit lower L and U = D L^T; the
    // Cholesky factor is C = L D^1/2 (A = C C^T), returned in both layouts
    // (lnz: C in the lower part of each supernode, C^T above the diagonal;
    // unz: the rows of C^T right of the diagonal block)
    const bool chol = (precision & SPK_SPD) && done;
    std::vector<double> sq;
    for (const HFront& F : h->fronts) {
        const int ld = F.nf + F.m;
        const int* R = h->rows.data() + F.rows_off;
        std::vector<int> pos;
        if (chol) {
            sq.resize(F.nf);
            for (int x = 0; x < F.nf; ++x) {
                const double d = fac[F.loff + (i64)x * ld + x];
                if (!(d > 0.0)) {
                    char buf[160];
                    std::snprintf(buf, sizeof buf, "not positive definite: pivot %.3e at column %lld", d,
                                  (long long)(F.f + x + 1));
                    return set_err(h, SPK_ESINGULAR, buf);
                }
                sq[x] = std::sqrt(d);
            }
        }
        for (int s = F.piece0; s < F.piece0 + F.npieces; ++s) {
            const int p0 = h->xs[s] - (int)F.f, w = h->xs[s + 1] - h->xs[s];
            const i64 a = h->xlindx0[s], jlen = h->xlindx0[s + 1] - a;
            // position of each of the piece's rows in the (padded) front
            pos.resize(jlen);
            for (i64 t = 0; t < jlen; ++t) {
                int row = h->lindx0[a + t];
                pos[t] = row < F.f + F.nf ? (int)(row - F.f)
                                          : F.nf + (int)(std::lower_bound(R, R + F.m, row) - R);
            }
            const i64 lbase = h->xlnz0[h->xs[s]], ubase = h->xunz0[h->xs[s]];
            for (int k = 0; k < w; ++k) {
                const int col = p0 + k;
                if (lnz)
                    for (i64 t = 0; t < jlen; ++t) {
                        double v = fac[F.loff + (i64)col * ld + pos[t]];
                        if (chol) v = pos[t] > col ? v * sq[col] : pos[t] == col ? sq[col] : v / sq[pos[t]];
                        lnz[lbase + k * jlen + t] = v;
                    }
                if (unz)
                    for (i64 i = 0; i < jlen - w; ++i) {
                        const int c = pos[w + i];
                        double v = c < F.nf ? fac[F.loff + (i64)c * ld + col] : fac[F.uoff + (i64)col * F.m + (c - F.nf)];
                        if (chol) v /= sq[col];
                        unz[ubase + k * (jlen - w) + i] = v;
                    }
            }
        }
    }
    if (ipiv && !done) {
        for (i64 j = 0; j < h->n; ++j) ipiv[j] = 0;   // as _inmatrix! leaves it
    } else if (ipiv) {
        std::vector<int> p(h->n);
        CU(h, cudaMemcpyAsync(p.data(), h->d_ipiv, sizeof(int) * h->n, cudaMemcpyDeviceToHost, h->stream));
        CU(h, cudaStreamSynchronize(h->stream));
        for (i64 j = 0; j < h->n; ++j) ipiv[j] = p[j] + 1;
    }
    return SPK_OK;
}

int spk_stats(spk_handle* h, int64_t* nfronts, int64_t* nlevels, int64_t* factor_entries, double* lu_flops) {
    if (!h) return SPK_EARG;
    if (nfronts) *nfronts = (int64_t)h->fronts.size();
    if (nlevels) *nlevels = (int64_t)h->nlevels;
    if (factor_entries) *factor_entries = h->fsize;
    if (lu_flops) *lu_flops = h->lu_flops;
    return SPK_OK;
}

int spk_profile(spk_handle* h, unsigned mask) {
    int rc = check_h(h);
    if (rc) return rc;
    h->prof_mask = mask;
    return SPK_OK;
}

int spk_profile_reset(spk_handle* h) {
    int rc = check_h(h);
    if (rc) return rc;
    collect_events(h);
    for (int k = 0; k < SPK_K_COUNT; ++k) {
        h->prof_ms[k] = h->prof_flops[k] = h->prof_bytes[k] = 0.0;
        h->prof_launches[k] = 0;
    }
    return SPK_OK;
}

int spk_profile_read(spk_handle* h, int kind, double* ms, int64_t* launches, double* flops, double* bytes) {
    int rc = check_h(h);
    if (rc) return rc;
    if (kind < 0 || kind >= SPK_K_COUNT) return set_err(h, SPK_EARG, "spk_profile_read: bad kernel class");
    collect_events(h);
    if (ms) *ms = h->prof_ms[kind];
    if (launches) *launches = h->prof_launches[kind];
    if (flops) *flops = h->prof_flops[kind];
    if (bytes) *bytes = h->prof_bytes[kind];
    return SPK_OK;
}

const char* spk_last_error(spk_handle* h) { return h ? h->err.c_str() : g_create_err.c_str(); }

void spk_destroy(spk_handle* h) {
    if (!h) return;
    if (h->device >= 0) cudaSetDevice(h->device);
    if (h->own) cudaStreamSynchronize(h->own);
    for (Plan& P : h->plan) free_plan(P);
    void* ptrs[] = {h->d_xs, h->d_rows, h->d_runid, h->d_run_tgt, h->d_run_start, h->d_run_rel,
                    h->d_rel, h->d_ipiv, h->d_bmap, h->d_info, h->d_slot, h->d_aval, h->d_acsr,
                    h->d_rowptr, h->d_col, h->d_src, h->d_ccolptr, h->d_crow, h->d_ccol, h->d_rperm, h->d_rinvp, h->d_wb,
                    h->d_wy, h->d_wx, h->d_rhs, h->d_x, h->d_r, h->d_sums, h->gm_V, h->gm_Z, h->gm_w, h->gm_c};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (int y = 0; y < 2; ++y) {
        void* st[] = {h->s64[y].d, h->s64[y].inv2, h->s64[y].pack, h->s32[y].d, h->s32[y].inv2, h->s32[y].pack,
                      h->s16[y].d, h->s16[y].inv2, h->s16[y].pack};
        for (void* p : st)
            if (p) cudaFree(p);
    }
    collect_events(h);
    for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
    drop_factor_graphs(h);
    drop_solve_graphs(h);
    if (h->side) cudaStreamSynchronize(h->side);
    if (h->side2) cudaStreamSynchronize(h->side2);
    if (h->side3) cudaStreamSynchronize(h->side3);
    if (h->evP) cudaEventDestroy(h->evP);
    if (h->evB) cudaEventDestroy(h->evB);
    if (h->evP2) cudaEventDestroy(h->evP2);
    if (h->evI) cudaEventDestroy(h->evI);
    if (h->evS) cudaEventDestroy(h->evS);
    for (cudaEvent_t e : h->evF)
        if (e) cudaEventDestroy(e);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->side2) cudaStreamDestroy(h->side2);
    if (h->side3) cudaStreamDestroy(h->side3);
    if (h->own) cudaStreamDestroy(h->own);
    delete h;
}

}  // extern "C"
