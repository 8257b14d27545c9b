// oz_capi.cu -- the C ABI (include/oz_gb300.h): handles, the drop-in
// setup/DGEMM pair on host arrays, the device-pointer and grouped entry points,
// options, dumps for parity tests.
//
// Reference interface replaced (atlarge-research/ozAIE include/oz_aie.h):
//   ozAIE_setup :182-300, ozAIE_DGEMM :311-349, convert_paired_i64_to_double_matrix
//   :92-150, cleanup_xrt :153-170.  No CPU fallback: every compute entry point
//   needs a CUDA device and reports OZGB_ERR_NO_DEVICE otherwise.
#include <cuda_runtime.h>

#include <algorithm>
#include <bit>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "oz_gb300.h"
#include "oz_gemm.cuh"
#include "oz_internal.h"
#include "oz_plan.h"

using namespace ozgb;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    bool ensure(size_t bytes) {
        if (bytes <= cap && p) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, std::max<size_t>(bytes, 256)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return false;
        }
        cap = std::max<size_t>(bytes, 256);
        return true;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

}  // namespace

struct ozgb_context {
    std::mutex mu;
    int device = -1;
    bool setup_done = false;
    int M = 0, N = 0, K = 0, mode = OZGB_MODE_FAST;
    // options
    int profile = OZGB_PROFILE_GB300;
    int opt_bits = 0, opt_slices = 0, opt_bins = 0, opt_rounding = OZGB_ROUND_DEFAULT, opt_format = 0;
    double err_bound = 0.0;
    int sched_any = 1;             // precision knob: search every pair set (1) or the triangular one only (0)
    int err_crit = KNOB_NORMWISE;  // precision knob: normwise or elementwise criterion
    double err_tail = 1e-4;        // elementwise: entries within err_tail sigma of zero left out
    int use_graph = 0;
    unsigned long long timeout_ns = 2000000000ull;
    bool have_plan_hint = false;  // ozgb_set_plan_hint: fixed GEMM plan choices for single calls
    PlanHints plan_hint{};
    // last effective plan
    Plan last{};
    bool have_last = false;
    // buffers
    DevBuf a, b, c, at, bt, er, ec, err, raw, knob, kpart;
    // K-split of a launch's last wave: group sums and counters, kept zero between
    // launches by the kernel itself (zeroed here only when (re)allocated or after a
    // device error)
    DevBuf split;
    bool split_dirty = true;
    KnobJob kjob{};  // the last stage-(a) statistics, for the precision knob
    DevBuf gstat, gslice, gtab;  // grouped calls: statistics, slice planes, job/problem tables
    DevBuf gprob;                // grouped calls: per-launch problem tables of the slice-pair GEMMs
    int grouped_launch = 1;      // 1: one persistent GEMM launch per plan class; 0: one per problem
    cudaStream_t stream = nullptr;       // used by the host-array entry points
    // grouped calls: the per-problem GEMMs run on auxiliary streams forked from
    // and joined back into the caller's stream
    static constexpr int kAux = 32;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kAux] = {};
    // host-array calls: the GEMM's first part done / its rows copied back (aux[0])
    cudaEvent_t ev_part = nullptr, ev_part_copied = nullptr;
    // grouped calls under CUDA graphs (ozgb_set_graph): the two captured phases and
    // the inputs they were captured for; the knob statistics land in pinned memory
    std::vector<long long> gkey1, gkey2;
    cudaGraphExec_t gexec1 = nullptr, gexec2 = nullptr;
    KnobStats *knob_host = nullptr;
    size_t knob_host_n = 0;
    cudaStream_t last_stream = nullptr;  // stream of the last enqueued call
    // profiling
    bool profiling = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ev_recorded = false;
    long long launches = 0;  // kernels this handle has launched
    std::string msg;
};

namespace {

ozgb_status fail(ozgb_handle h, ozgb_status st, const std::string &m) {
    if (h) h->msg = m;
    return st;
}

ozgb_status cuda_fail(ozgb_handle h, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidDeviceFunction) return fail(h, OZGB_ERR_IMAGE, m);
    if (e == cudaErrorMemoryAllocation) return fail(h, OZGB_ERR_ALLOC, m);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return fail(h, OZGB_ERR_NO_DEVICE, m);
    return fail(h, OZGB_ERR_EXEC, m);
}

ozgb_status ensure_device(ozgb_handle h) {
    if (h->device >= 0) {
        cudaError_t e = cudaSetDevice(h->device);
        return e == cudaSuccess ? OZGB_OK : cuda_fail(h, e, "cudaSetDevice");
    }
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n < 1) {
        cudaGetLastError();
        return fail(h, OZGB_ERR_NO_DEVICE, "no CUDA device available (no CPU fallback)");
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return fail(h, OZGB_ERR_NO_DEVICE, "device query failed");
    if (prop.major != 10 || prop.minor != 3)
        return fail(h, OZGB_ERR_IMAGE, std::string("kernels are built for sm_103a; device is ") + prop.name);
    if ((e = cudaSetDevice(dev)) != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(h, e, "cudaStreamCreate");
    for (auto &ev : h->ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return cuda_fail(h, e, "cudaEventCreate");
    if (!h->err.ensure(sizeof(int))) return fail(h, OZGB_ERR_ALLOC, "device error word");
    cudaMemset(h->err.p, 0, sizeof(int));
    h->device = dev;
    return OZGB_OK;
}

// Effective (b, s, J, rounding) for a call with inner dimension K.
OzConfig resolve_config(ozgb_handle h, int K, int mode) {
    OzConfig c;
    if (h->profile == OZGB_PROFILE_REFERENCE) {
        reference_table(K, mode, &c.b, &c.s);
        c.J = c.s;
        c.rounding = OUT_RZ_REF;
    } else {
        c.b = 7;
        c.s = 8;
        c.J = (mode == OZGB_MODE_FAST) ? c.s : 2 * c.s - 1;
        c.rounding = OUT_RN;
    }
    if (h->opt_bits > 0) c.b = h->opt_bits;
    if (h->opt_slices > 0) {
        const bool full = (c.J == 2 * c.s - 1) && c.s > 1;
        c.s = h->opt_slices;
        c.J = full ? 2 * c.s - 1 : c.s;
    }
    if (h->opt_bins == -1) c.J = 2 * c.s - 1;
    else if (h->opt_bins > 0) c.J = h->opt_bins;
    if (h->opt_rounding >= 0) c.rounding = h->opt_rounding;
    c.carrier = h->opt_format;
    return c;
}

struct Operands {
    int M, N, K;
    const double *A;
    long lda;
    const double *B;
    long ldb;
    double *C;
    long ldc;
    bool ta = false, tb = false;  // A stored K x M, B stored N x K
    double alpha = 1.0, beta = 0.0;
};

// Statistics layout of one operand pass (launch_stats2d on a rows x cols matrix):
// partials of its rows at p, of its columns after them.
struct StatsLayout {
    size_t row_n, col_n;  // entries
    int rparts, cparts;
};
StatsLayout stats_layout(int rows, int cols) {
    StatsLayout l;
    l.rparts = (cols + kStatsCols - 1) / kStatsCols;
    l.cparts = (rows + kStatsRows - 1) / kStatsRows;
    l.row_n = static_cast<size_t>(rows) * l.rparts;
    l.col_n = static_cast<size_t>(l.cparts) * cols;
    return l;
}
StatParts row_parts(const unsigned long long *p, int rows, const StatsLayout &l) {
    return StatParts{p, rows, l.rparts, l.rparts, 1};
}
StatParts col_parts(const unsigned long long *p, int cols, const StatsLayout &l) {
    return StatParts{p + l.row_n, cols, l.cparts, 1, cols};
}

// The knob's inputs for op(A) (M x K) and op(B) (K x N) whose stored operands
// have had launch_stats2d run into pa / pb (rows x cols as stored).
KnobJob knob_job(const Operands &o, const int32_t *er, const int32_t *ec, const unsigned long long *pa,
                 const unsigned long long *pb) {
    KnobJob j{};
    j.er = er;
    j.M = o.M;
    j.ec = ec;
    j.N = o.N;
    j.K = o.K;
    if (!o.ta) {  // A stored M x K: its rows are op(A)'s rows, its columns the k units
        const StatsLayout la = stats_layout(o.M, o.K);
        j.ra = row_parts(pa, o.M, la);
        j.ka = col_parts(pa, o.K, la);
    } else {  // A stored K x M
        const StatsLayout la = stats_layout(o.K, o.M);
        j.ka = row_parts(pa, o.K, la);
        j.ra = col_parts(pa, o.M, la);
    }
    if (!o.tb) {  // B stored K x N: its rows are the k units, its columns op(B)'s columns
        const StatsLayout lb = stats_layout(o.K, o.N);
        j.kb = row_parts(pb, o.K, lb);
        j.cb = col_parts(pb, o.N, lb);
    } else {  // B stored N x K
        const StatsLayout lb = stats_layout(o.N, o.K);
        j.cb = row_parts(pb, o.N, lb);
        j.kb = col_parts(pb, o.K, lb);
    }
    return j;
}

size_t stats_entries(int rows, int cols) {
    const StatsLayout l = stats_layout(rows, cols);
    return l.row_n + l.col_n;
}

// Stage (a): exponents; when the precision knob needs them, one fused pass per
// operand also leaves the partial sums of squares of its rows and columns.
ozgb_status enqueue_exponents(ozgb_handle h, const Operands &o, bool want_ss, cudaStream_t st) {
    if (!h->er.ensure(sizeof(int32_t) * o.M) || !h->ec.ensure(sizeof(int32_t) * o.N))
        return fail(h, OZGB_ERR_ALLOC, "exponent buffers");
    int32_t *er = static_cast<int32_t *>(h->er.p), *ec = static_cast<int32_t *>(h->ec.p);
    cudaMemsetAsync(ec, 0, sizeof(int32_t) * o.N, st);
    if (want_ss) {
        const int ar = o.ta ? o.K : o.M, ac = o.ta ? o.M : o.K;  // A as stored
        const int br = o.tb ? o.N : o.K, bc = o.tb ? o.K : o.N;  // B as stored
        const size_t na = stats_entries(ar, ac), nb = stats_entries(br, bc);
        if (!h->kpart.ensure(sizeof(unsigned long long) * (na + nb)))
            return fail(h, OZGB_ERR_ALLOC, "statistics buffers");
        unsigned long long *pa = static_cast<unsigned long long *>(h->kpart.p), *pb = pa + na;
        cudaMemsetAsync(er, 0, sizeof(int32_t) * o.M, st);
        const StatsLayout la = stats_layout(ar, ac), lb = stats_layout(br, bc);
        // both operands' fused passes in one launch
        StageJob ja{}, jb{};
        ja.kind = JOB_STATS, ja.X = o.A, ja.ld = o.lda, ja.rows = ar, ja.cols = ac;
        ja.e_out = o.ta ? nullptr : er, ja.e_out2 = o.ta ? er : nullptr, ja.prow = pa, ja.pcol = pa + la.row_n;
        jb.kind = JOB_STATS, jb.X = o.B, jb.ld = o.ldb, jb.rows = br, jb.cols = bc;
        jb.e_out = o.tb ? ec : nullptr, jb.e_out2 = o.tb ? nullptr : ec, jb.prow = pb, jb.pcol = pb + lb.row_n;
        launch_stage_pair(ja, jb, st);
        h->kjob = knob_job(o, er, ec, pa, pb);
    } else {
        // exponent maxima of the rows of op(A) and the columns of op(B), one launch
        StageJob ja{}, jb{};
        if (o.ta) {  // rows of op(A) are columns of A
            cudaMemsetAsync(er, 0, sizeof(int32_t) * o.M, st);
            ja.kind = JOB_COLMAX, ja.rows = o.K, ja.cols = o.M;
        } else {
            ja.kind = JOB_ROWMAX, ja.rows = o.M, ja.cols = o.K;
        }
        ja.X = o.A, ja.ld = o.lda, ja.e_out = er;
        if (o.tb) {  // columns of op(B) are rows of B
            jb.kind = JOB_ROWMAX, jb.rows = o.N, jb.cols = o.K;
        } else {
            jb.kind = JOB_COLMAX, jb.rows = o.K, jb.cols = o.N;
        }
        jb.X = o.B, jb.ld = o.ldb, jb.e_out = ec;
        launch_stage_pair(ja, jb, st);
    }
    h->launches += 1;
    return OZGB_OK;
}

int sm_count(int dev);

ozgb_status choose_config(ozgb_handle h, const Operands &o, int mode, cudaStream_t st, OzConfig *cfg) {
    *cfg = resolve_config(h, o.K, mode);
    if (h->err_bound > 0.0 && h->opt_slices <= 0) {
        // precision knob: the stage-(a) partial sums are reduced on the device to
        // five scaled sums, and only those cross to the host
        if (!h->knob.ensure(sizeof(KnobStats))) return fail(h, OZGB_ERR_ALLOC, "knob buffer");
        KnobJob j = h->kjob;
        j.out = static_cast<double *>(h->knob.p);
        launch_knob_stats(j, st);
        h->launches += 1;
        KnobStats ks;
        cudaMemcpyAsync(&ks, h->knob.p, sizeof ks, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(h, e, "statistics readback");
        // the cheapest slice schedule (slices and pair set) whose estimate meets the bound
        const Schedule sc = choose_schedule(ks, o.M, o.N, o.K, *cfg, h->err_bound, 2, 16, h->err_crit, h->err_tail,
                                            h->sched_any != 0, sm_count(h->device));
        cfg->s = sc.s;
        cfg->J = sc.J;
    }
    return OZGB_OK;
}

// GEMM launch arguments that follow from the plan alone (shared by all problems
// of a grouped launch); operands, sizes and tiles are set by the caller.
void gemm_args_from_plan(GemmArgs *g, const Plan &p, int out_mode, int *err, unsigned long long timeout_ns) {
    memset(g, 0, sizeof *g);
    g->KC = p.KC;
    g->s = p.cfg.s;
    g->J = p.cfg.J;
    g->b = p.cfg.b;
    g->out_mode = out_mode;
    g->stages = p.stages;
    g->stage_bytes = p.stage_bytes;
    g->a_block_bytes = p.a_block_bytes;
    g->b_block_bytes = p.b_block_bytes;
    g->b_pad_lo_bytes = static_cast<uint32_t>(p.pad_lo) * p.b_slice_bytes;
    g->b_region_bytes = p.b_region_bytes;
    g->tmem_cols = p.tmem_cols;
    g->err = err;
    g->timeout_ns = timeout_ns;
    g->alpha = 1.0;
    g->beta = 0.0;
    g->n_acc = p.n_acc;
    g->n_iss = p.n_iss;
    for (int a = 0; a < kMaxAcc; ++a) g->acc_t0[a] = p.acc_t0[a];
    g->G = p.G;
    for (int i = 0; i < p.G; ++i) {
        g->blk_lo[i] = p.blk_lo[i];
        g->blk_nb[i] = p.blk_nb[i];
        g->blk_p0[i] = p.blk_p0[i];
        g->blk_p1[i] = p.blk_p1[i];
        g->blk_period[i] = p.blk_period[i];
        g->blk_off[i] = p.blk_off[i];
        g->blk_col1[i] = p.blk_col1[i];
    }
    g->dbl_mask = p.dbl_mask;
}

// Auxiliary streams and their events, created on first use.
ozgb_status ensure_aux(ozgb_handle h) {
    if (h->ev_fork) return OZGB_OK;
    bool okc = cudaEventCreateWithFlags(&h->ev_part, cudaEventDisableTiming) == cudaSuccess &&
               cudaEventCreateWithFlags(&h->ev_part_copied, cudaEventDisableTiming) == cudaSuccess;
    for (int a = 0; okc && a < ozgb_context::kAux; ++a)
        okc = cudaStreamCreateWithFlags(&h->aux[a], cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&h->ev_join[a], cudaEventDisableTiming) == cudaSuccess;
    okc = okc && cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) == cudaSuccess;
    if (!okc) return cuda_fail(h, cudaGetLastError(), "auxiliary streams");
    return OZGB_OK;
}

int sm_count(int dev) {
    static int cached[64] = {0};
    if (dev < 0 || dev >= 64) return 148;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
        cached[dev] = n;
    }
    return cached[dev];
}

// K-split of the last partial wave of a launch over tiles [begin, end): its R
// tiles are each split into P K ranges of at least 4 chunks, P <= SMs / R, so
// that wave fills the SMs; a single-wave launch with fewer tiles than SMs is
// split the same way.  P = 1: no split.
struct TailSplit {
    int R = 0, P = 1;
    size_t acc_bytes = 0, bytes = 0;  // scratch: group sums, then R counters
};
TailSplit tail_split_shape(const Plan &p, int out_mode, int begin, int end, int sms) {
    TailSplit ts;
    if (out_mode != OUT_RN && out_mode != OUT_RZ_REF) return ts;
    const int n = end - begin;
    const int R = n <= sms ? n : n % sms;
    if (R == 0) return ts;
    const int P = std::min({sms / R, p.n_kc / 4, 16});
    if (P < 2) return ts;
    const int NA = p.W > 2 ? p.W - 1 : 1;
    ts.R = R;
    ts.P = P;
    ts.acc_bytes = static_cast<size_t>(R) * NA * p.BN * BM * 8;
    ts.bytes = ts.acc_bytes + static_cast<size_t>(R) * sizeof(int);
    return ts;
}
void apply_tail_split(GemmArgs *g, const TailSplit &ts, int begin, int end, void *scratch) {
    g->tile_begin = begin;
    g->total_tiles = end;
    g->split_parts = 1;
    g->split_start = end;
    if (ts.P < 2) return;
    g->split_parts = ts.P;
    g->split_start = end - ts.R;
    g->total_tiles = end - ts.R + ts.R * ts.P;
    g->split_acc = static_cast<unsigned long long *>(scratch);
    g->split_cnt = reinterpret_cast<int *>(static_cast<char *>(scratch) + ts.acc_bytes);
}
// Grows buf to at least bytes; a new allocation (or dirty contents) is zeroed.
bool ensure_zeroed(DevBuf &buf, bool &dirty, size_t bytes, cudaStream_t st) {
    const void *old = buf.p;
    if (!buf.ensure(bytes)) return false;
    if (buf.p != old || dirty) {
        if (cudaMemsetAsync(buf.p, 0, buf.cap, st) != cudaSuccess) return false;
        dirty = false;
    }
    return true;
}
ozgb_status set_tail_split(ozgb_handle h, const Plan &p, int begin, int end, cudaStream_t st, GemmArgs *g) {
    const TailSplit ts = tail_split_shape(p, g->out_mode, begin, end, sm_count(h->device));
    if (ts.P > 1 && !ensure_zeroed(h->split, h->split_dirty, ts.bytes, st))
        return fail(h, OZGB_ERR_ALLOC, "split scratch");
    apply_tail_split(g, ts, begin, end, h->split.p);
    return OZGB_OK;
}

// Host destination of C (the host-array entry point, C dense with N columns).
// When C has more than one group of 8 row tiles, the GEMM runs as two launches:
// the first covers full waves up to the end of the last group but one, and the
// rows it completes are copied back on an auxiliary stream while the second
// launch runs.  Splitting at a multiple of the grid keeps the number of waves.
struct HostOut {
    double *C;
    bool copied;  // set when the split path has enqueued every copy of C
};

// Stages (b) and (c)+(d) for one problem whose exponents are in h->er / h->ec.
ozgb_status enqueue_split_gemm(ozgb_handle h, const Operands &o, const Plan &p, int out_mode, int32_t *raw,
                               cudaStream_t st, HostOut *ho = nullptr) {
    if (!h->at.ensure(p.a_bytes) || !h->bt.ensure(p.b_bytes))
        return fail(h, OZGB_ERR_ALLOC, "slice buffers");
    uint16_t *at = static_cast<uint16_t *>(h->at.p), *bt = static_cast<uint16_t *>(h->bt.p);
    // small operands: both splits in one launch (one launch gap less); large ones
    // run the separate kernels, whose lighter register and shared-memory use
    // measured faster (4096^3: 0.270 against 0.291 ms)
    const double elems = static_cast<double>(p.Mp + p.Np) * p.n_kc * p.KC;
    if (elems > 16.0 * 1024 * 1024) {
        launch_split_a(o.A, o.lda, o.M, o.K, static_cast<int32_t *>(h->er.p), p.cfg.b, p.cfg.s, p.KC, p.n_kc, p.Mp, at,
                       st, o.ta, p.f8);
        launch_split_b(o.B, o.ldb, o.K, o.N, static_cast<int32_t *>(h->ec.p), p.cfg.b, p.cfg.s, p.KC, p.n_kc, p.BN,
                       p.Np, bt, st, o.tb, p.f8);
        h->launches += 2;
    } else {
        StageJob ja{}, jb{};
        ja.kind = JOB_SPLIT_A, ja.X = o.A, ja.ld = o.lda, ja.rows = o.M, ja.cols = o.K;
        ja.e_in = static_cast<int32_t *>(h->er.p), ja.padded = p.Mp, ja.trans = o.ta ? 1 : 0, ja.tiles = at;
        jb.kind = JOB_SPLIT_B, jb.X = o.B, jb.ld = o.ldb, jb.rows = o.K, jb.cols = o.N;
        jb.e_in = static_cast<int32_t *>(h->ec.p), jb.padded = p.Np, jb.trans = o.tb ? 1 : 0, jb.tiles = bt;
        for (StageJob *j : {&ja, &jb}) {
            j->b = p.cfg.b, j->s = p.cfg.s, j->KC = p.KC, j->n_kc = p.n_kc, j->BN = p.BN;
            j->f8 = p.f8 ? 1 : 0;
        }
        launch_stage_pair(ja, jb, st);
        h->launches += 1;
    }
    if (h->profiling) cudaEventRecord(h->ev[2], st);
    GemmArgs g;
    gemm_args_from_plan(&g, p, out_mode, static_cast<int *>(h->err.p), h->timeout_ns);
    g.a_tiles = at;
    g.b_tiles = bt;
    g.er = static_cast<int32_t *>(h->er.p);
    g.ec = static_cast<int32_t *>(h->ec.p);
    g.c = o.C;
    g.ldc = o.ldc;
    g.raw = raw;
    g.M = o.M;
    g.N = o.N;
    g.n_kc = p.n_kc;
    g.tiles_m = p.tiles_m;
    g.tiles_n = p.tiles_n;
    g.total_tiles = p.tiles_m * p.tiles_n;
    g.alpha = o.alpha;
    g.beta = o.beta;
    if (out_mode == OUT_PAIRS) {
        // the reference's two sums: bins t < g0 and t >= g0, each modulo 2^64
        g.pair_g0 = reference_first_group(o.K, p.cfg.b, p.cfg.s);
        g.n_acc = g.pair_g0 < p.cfg.J ? 2 : 1;
        g.acc_t0[0] = 0;
        g.acc_t0[1] = g.pair_g0;
    }
    const int total = p.tiles_m * p.tiles_n;
    int t_split = 0, rows_split = 0;
    if (ho && (out_mode == OUT_RN || out_mode == OUT_RZ_REF) && o.ldc == o.N) {
        const int grid = std::min(total, sm_count(h->device));
        const int groups = (p.tiles_m + 7) / 8;  // grouped rasterisation: 8 row tiles per group
        if (groups >= 2) {
            const int before_last = (groups - 1) * 8 * p.tiles_n;
            const int t1 = ((before_last + grid - 1) / grid) * grid;
            if (t1 < total) {
                t_split = t1;
                rows_split = (groups - 1) * 8 * BM;
            }
        }
    }
    cudaError_t e;
    if (t_split > 0) {
        ozgb_status rc = ensure_aux(h);
        if (rc) return rc;
        // A copy into pageable host memory returns only when it has completed, so
        // for pageable C both launches are enqueued before the first copy (else
        // the second launch would wait for the first part and its copy).  A copy
        // into page-locked memory is asynchronous; enqueued before the second
        // launch it starts as soon as the first part ends (measured at 4096^3:
        // 1.5 ms faster than enqueued after it).
        cudaPointerAttributes pa{};
        const bool pageable = cudaPointerGetAttributes(&pa, ho->C) != cudaSuccess ||
                              pa.type == cudaMemoryTypeUnregistered;
        cudaGetLastError();
        const size_t n1 = static_cast<size_t>(rows_split) * o.N;
        auto copy_first = [&]() -> ozgb_status {
            cudaStreamWaitEvent(h->aux[0], h->ev_part, 0);
            const cudaError_t ce = cudaMemcpyAsync(ho->C, o.C, n1 * 8, cudaMemcpyDeviceToHost, h->aux[0]);
            if (ce != cudaSuccess) return cuda_fail(h, ce, "copy C (first rows)");
            cudaEventRecord(h->ev_part_copied, h->aux[0]);
            return OZGB_OK;
        };
        if ((rc = set_tail_split(h, p, 0, t_split, st, &g))) return rc;
        p.fn(g, t_split, p.smem, st);
        cudaEventRecord(h->ev_part, st);
        if (!pageable && (rc = copy_first())) return rc;
        if ((rc = set_tail_split(h, p, t_split, total, st, &g))) return rc;
        p.fn(g, total - t_split, p.smem, st);
        h->launches += 2;
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(h, e, "slice-pair GEMM launch");
        if (h->profiling) {
            cudaEventRecord(h->ev[3], st);
            h->ev_recorded = true;
        }
        if (pageable && (rc = copy_first())) return rc;
        const size_t n2 = static_cast<size_t>(o.M - rows_split) * o.N;
        if ((e = cudaMemcpyAsync(ho->C + n1, o.C + n1, n2 * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            return cuda_fail(h, e, "copy C (last rows)");
        cudaStreamWaitEvent(st, h->ev_part_copied, 0);
        ho->copied = true;
        return OZGB_OK;
    }
    {
        const ozgb_status rc = set_tail_split(h, p, 0, total, st, &g);
        if (rc) return rc;
    }
    p.fn(g, total, p.smem, st);
    h->launches += 1;
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, "slice-pair GEMM launch");
    return OZGB_OK;
}

// The whole pipeline for one problem on device operands.
ozgb_status enqueue_dgemm(ozgb_handle h, const Operands &o, int mode, cudaStream_t st, int out_mode_override = -1,
                          int bin_lo = 0, int bin_hi = kMaxBins, int32_t *raw = nullptr, HostOut *ho = nullptr) {
    h->last_stream = st;
    if (h->profiling) cudaEventRecord(h->ev[0], st);
    const bool want_ss = h->err_bound > 0.0 && h->opt_slices <= 0;
    ozgb_status rc = enqueue_exponents(h, o, want_ss, st);
    if (rc) return rc;
    if (h->profiling) cudaEventRecord(h->ev[1], st);
    OzConfig cfg;
    if ((rc = choose_config(h, o, mode, st, &cfg))) return rc;
    // dumps read the slice planes back as bf16
    if (out_mode_override == OUT_RAW || out_mode_override == OUT_PAIRS) cfg.carrier = 1;
    Plan p;
    std::string why;
    PlanHints pairs_hint;
    const bool pairs = out_mode_override == OUT_PAIRS;
    if (pairs) {
        // the reference's paired output needs its d bins (triangular) and two
        // 64-bit sums, i.e. a variant with at least 4 accumulator words
        if (cfg.J != cfg.s) return fail(h, OZGB_ERR_UNSUPPORTED, "paired output needs the triangular pair set");
        pairs_hint.min_W = 4;
    }
    if (h->have_plan_hint) {
        const int min_w = pairs_hint.min_W;
        pairs_hint = h->plan_hint;
        pairs_hint.min_W = min_w;
    }
    if (!make_plan(o.M, o.N, o.K, cfg, &p, &why, bin_lo, bin_hi, pairs || h->have_plan_hint ? &pairs_hint : nullptr))
        return fail(h, OZGB_ERR_UNSUPPORTED, why);
    h->last = p;
    h->have_last = true;
    const int om = out_mode_override >= 0 ? out_mode_override : cfg.rounding;
    if ((rc = enqueue_split_gemm(h, o, p, om, raw, st, ho))) return rc;
    if (h->profiling && !(ho && ho->copied)) {
        cudaEventRecord(h->ev[3], st);
        h->ev_recorded = true;
    }
    return OZGB_OK;
}

ozgb_status check_device_error(ozgb_handle h, cudaStream_t st) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(h, e, "kernel execution");
    int word = 0;
    e = cudaMemcpy(&word, h->err.p, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(h, e, "error word readback");
    if (word != 0) {
        cudaMemset(h->err.p, 0, sizeof(int));
        h->split_dirty = true;  // a stopped kernel may have left split sums behind
        return fail(h, OZGB_ERR_TIMEOUT,
                    "a device-side wait ran out of time (code " + std::to_string(word) + "); the kernel stopped early");
    }
    return OZGB_OK;
}

// ------------------------------------------------------------ grouped calls
size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// Uploads a host table into the grouped-table buffer at byte offset *off.
template <typename T>
const T *put_table(ozgb_handle h, const std::vector<T> &v, size_t *off, cudaStream_t st) {
    uint8_t *dst = static_cast<uint8_t *>(h->gtab.p) + *off;
    cudaMemcpyAsync(dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st);
    *off += align256(sizeof(T) * v.size());
    return reinterpret_cast<const T *>(dst);
}

// All stage jobs of one grouped launch, with their block offsets.
struct JobList {
    std::vector<StageJob> jobs;
    std::vector<int> block0;
    int total = 0;
    void add(const StageJob &j0) {
        StageJob j = j0;
        stage_grid(j, &j.gx, &j.gy);
        block0.push_back(total);
        total += j.gx * j.gy;
        jobs.push_back(j);
    }
};

// Runs enqueue(stream) directly on st, or, with graphs enabled, replays the graph
// captured for the same key (capturing it first when the key changed).
template <typename F>
ozgb_status run_phase(ozgb_handle h, bool graph, const std::vector<long long> &key, std::vector<long long> *cached_key,
                      cudaGraphExec_t *exec, cudaStream_t st, F enqueue) {
    if (!graph) return enqueue(st);
    if (*exec && *cached_key == key) {
        const cudaError_t e = cudaGraphLaunch(*exec, st);
        return e == cudaSuccess ? OZGB_OK : cuda_fail(h, e, "graph launch");
    }
    if (*exec) {
        cudaGraphExecDestroy(*exec);
        *exec = nullptr;
    }
    cached_key->clear();
    // capture on the handle's own stream (the caller's may be the legacy default
    // stream, which cannot be captured), then launch on the caller's stream
    cudaStream_t cs = h->stream;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return cuda_fail(h, e, "begin capture");
    const ozgb_status rc = enqueue(cs);
    cudaGraph_t graph_ = nullptr;
    e = cudaStreamEndCapture(cs, &graph_);
    if (rc != OZGB_OK) {
        if (graph_) cudaGraphDestroy(graph_);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "end capture");
    e = cudaGraphInstantiate(exec, graph_, 0);
    cudaGraphDestroy(graph_);
    if (e != cudaSuccess) {
        *exec = nullptr;
        return cuda_fail(h, e, "graph instantiate");
    }
    *cached_key = key;
    e = cudaGraphLaunch(*exec, st);
    return e == cudaSuccess ? OZGB_OK : cuda_fail(h, e, "graph launch");
}

// One grouped slice-pair GEMM launch: the problems whose plans share the kernel
// variant and every launch-level GemmArgs field (stage layout, bin blocks, drain
// schedule, accumulator groups, rounding).  Its work units are the tiles of its
// problems, largest problems first, so that small problems fill the last waves.
struct GroupLaunch {
    GemmArgs g;         // launch-level fields (probs / tile_prob set when uploaded)
    const Plan *plan;   // the plan of its first problem: variant and shared memory
    std::vector<GroupProblem> probs;
    std::vector<int> tile_prob;
    double cost = 0.0;  // tiles x chunks x pairs
};

// The launch-level fields of a plan's GemmArgs as a fixed array (no allocation):
// problems with equal arrays share a grouped launch.
constexpr int kLaunchFields = 18 + kMaxAcc + 7 * kMaxGroups;
struct LaunchFields {
    long long v[kLaunchFields];
    int n = 0;
    unsigned long long hash = 0;
};
LaunchFields launch_fields(const GemmArgs &g, const Plan &p) {
    LaunchFields f;
    const long long head[18] = {reinterpret_cast<long long>(p.fn), static_cast<long long>(p.smem), g.KC, g.s, g.J,
                                g.b, g.out_mode, g.stages, g.stage_bytes, g.a_block_bytes, g.b_block_bytes,
                                g.b_pad_lo_bytes, g.b_region_bytes, g.tmem_cols, g.n_acc, g.n_iss, g.G, g.dbl_mask};
    for (long long x : head) f.v[f.n++] = x;
    for (int a = 0; a < kMaxAcc; ++a) f.v[f.n++] = g.acc_t0[a];
    for (int i = 0; i < g.G; ++i)
        for (long long x : {g.blk_lo[i], g.blk_nb[i], g.blk_p0[i], g.blk_p1[i], g.blk_period[i], g.blk_off[i],
                            g.blk_col1[i]})
            f.v[f.n++] = x;
    unsigned long long h = 1469598103934665603ull;  // FNV-1a over the words
    for (int i = 0; i < f.n; ++i) h = (h ^ static_cast<unsigned long long>(f.v[i])) * 1099511628211ull;
    f.hash = h;
    return f;
}
bool same_launch(const LaunchFields &x, const LaunchFields &y) {
    return x.hash == y.hash && x.n == y.n && std::equal(x.v, x.v + x.n, y.v);
}
std::vector<long long> launch_key(const GemmArgs &g, const Plan &p) {
    const LaunchFields f = launch_fields(g, p);
    return std::vector<long long>(f.v, f.v + f.n);
}

// The grouped launches of n problems with the given plans and device addresses
// of their slice blocks and exponents.
std::vector<GroupLaunch> build_group_launches(const ozgb_problem *probs, int n, const std::vector<Plan> &plans,
                                              const std::vector<const uint8_t *> &a_tiles,
                                              const std::vector<const uint8_t *> &b_tiles,
                                              const std::vector<const int32_t *> &er,
                                              const std::vector<const int32_t *> &ec, int *err,
                                              unsigned long long timeout_ns) {
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    auto cost = [&](int i) {
        return static_cast<double>(plans[i].tiles_m) * plans[i].tiles_n * plans[i].n_kc * plans[i].pairs;
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
    std::vector<GroupLaunch> out;
    std::vector<LaunchFields> keys;  // of out's launches (few: a linear scan of hashes)
    for (int i : order) {
        const Plan &p = plans[i];
        GemmArgs g;
        gemm_args_from_plan(&g, p, p.cfg.rounding, err, timeout_ns);
        const LaunchFields key = launch_fields(g, p);
        size_t li = 0;
        while (li < keys.size() && !same_launch(keys[li], key)) ++li;
        if (li == keys.size()) {
            keys.push_back(key);
            out.emplace_back();
            out.back().g = g;
            out.back().plan = &p;
        }
        GroupLaunch &L = out[li];
        GroupProblem gp{};
        gp.a_tiles = a_tiles[i];
        gp.b_tiles = b_tiles[i];
        gp.er = er[i];
        gp.ec = ec[i];
        gp.c = probs[i].C;
        gp.ldc = probs[i].ldc;
        gp.M = probs[i].M;
        gp.N = probs[i].N;
        gp.n_kc = p.n_kc;
        gp.tiles_m = p.tiles_m;
        gp.tiles_n = p.tiles_n;
        gp.tile0 = static_cast<int>(L.tile_prob.size());
        const int idx = static_cast<int>(L.probs.size());
        L.probs.push_back(gp);
        L.tile_prob.insert(L.tile_prob.end(), static_cast<size_t>(p.tiles_m) * p.tiles_n, idx);
        L.cost += cost(i);
    }
    for (GroupLaunch &L : out) {
        L.g.tile_begin = 0;
        L.g.total_tiles = static_cast<int>(L.tile_prob.size());
        L.g.split_parts = 1;  // no K-split: the problems side by side fill the SMs
        L.g.split_start = L.g.total_tiles;
    }
    std::stable_sort(out.begin(), out.end(), [](const GroupLaunch &x, const GroupLaunch &y) { return x.cost > y.cost; });
    return out;
}

// The grouped pipeline: one launch for every problem's stage (a) (and the knob's
// statistics), one grouped knob reduction and a single read-back when any
// problem asks for an error bound, one launch for every problem's split, and the
// persistent slice-pair GEMMs.  With graphs enabled both halves are captured once
// and replayed while the problems (and, for the second half, the slice counts)
// stay the same.
ozgb_status enqueue_grouped(ozgb_handle h, ozgb_problem *probs, int n, int mode, cudaStream_t st) {
    const bool graph = h->use_graph != 0;
    // a call without graphs rewrites the job and problem tables that captured
    // graphs read: those graphs may not be replayed afterwards
    if (!graph) {
        h->gkey1.clear();
        h->gkey2.clear();
    }
    const bool prof = h->profiling && !graph;
    std::vector<double> bound(n, 0.0);
    std::vector<int> adapt_idx(n, -1);
    int n_adapt = 0;
    for (int i = 0; i < n; ++i) {
        double bd = probs[i].error_bound;
        if (!(bd > 0.0) && h->err_bound > 0.0 && h->opt_slices <= 0) bd = h->err_bound;
        bound[i] = bd > 0.0 ? bd : 0.0;
        if (bound[i] > 0.0) adapt_idx[i] = n_adapt++;
    }
    // ---- statistics scratch: er, ec (int32); for adaptive problems the partial
    // sums of squares of A's and B's rows and columns; the knob outputs of all
    // adaptive problems contiguous at the end
    struct StatOff {
        size_t er, ec, pa, pb;
    };
    std::vector<StatOff> so(n);
    size_t total = 0;
    for (int i = 0; i < n; ++i) {
        const ozgb_problem &pb = probs[i];
        so[i] = StatOff{};
        so[i].er = total;
        total += align256(sizeof(int32_t) * pb.M);
        so[i].ec = total;
        total += align256(sizeof(int32_t) * pb.N);
        if (bound[i] > 0.0) {
            so[i].pa = total;
            total += align256(sizeof(unsigned long long) * stats_entries(pb.M, pb.K));
            so[i].pb = total;
            total += align256(sizeof(unsigned long long) * stats_entries(pb.K, pb.N));
        }
    }
    const size_t knob_off = total;
    total += align256(sizeof(KnobStats) * (n_adapt + 1));
    if (!h->gstat.ensure(total)) return fail(h, OZGB_ERR_ALLOC, "grouped statistics buffer");
    // job tables of both halves (phase 2: two split jobs per problem)
    const size_t tab_bytes = align256(sizeof(StageJob) * 4 * n) + align256(sizeof(int) * (4 * n + 1)) +
                             align256(sizeof(KnobJob) * (n_adapt + 1)) + align256(sizeof(StageJob) * 2 * n) +
                             align256(sizeof(int) * (2 * n + 1));
    if (!h->gtab.ensure(tab_bytes)) return fail(h, OZGB_ERR_ALLOC, "grouped table buffer");
    if (n_adapt > 0 && h->knob_host_n < static_cast<size_t>(n_adapt)) {
        if (h->knob_host) cudaFreeHost(h->knob_host);
        h->knob_host = nullptr;
        h->knob_host_n = 0;
        if (cudaMallocHost(&h->knob_host, sizeof(KnobStats) * n_adapt) != cudaSuccess)
            return fail(h, OZGB_ERR_ALLOC, "pinned knob buffer");
        h->knob_host_n = n_adapt;
    }
    uint8_t *gs = static_cast<uint8_t *>(h->gstat.p);
    auto at = [&](size_t off) { return gs + off; };
    KnobStats *knob_dev = reinterpret_cast<KnobStats *>(at(knob_off));

    // ---- phase 1: stage (a) and the knob statistics
    std::vector<long long> key1 = {n, mode, reinterpret_cast<long long>(gs), reinterpret_cast<long long>(h->gtab.p),
                                   reinterpret_cast<long long>(h->knob_host)};
    for (int i = 0; i < n; ++i) {
        const ozgb_problem &pb = probs[i];
        key1.insert(key1.end(), {pb.M, pb.N, pb.K, reinterpret_cast<long long>(pb.A), pb.lda,
                                 reinterpret_cast<long long>(pb.B), pb.ldb, bound[i] > 0.0 ? 1 : 0});
    }
    const bool replay1 = graph && h->gexec1 && h->gkey1 == key1;
    size_t toff = 0;
    JobList ja;
    std::vector<KnobJob> kj;
    const StageJob *dja = nullptr;
    const int *dba = nullptr;
    const KnobJob *dkj = nullptr;
    for (int i = 0; i < n; ++i) {
        const ozgb_problem &pb = probs[i];
        int32_t *er = reinterpret_cast<int32_t *>(at(so[i].er)), *ec = reinterpret_cast<int32_t *>(at(so[i].ec));
        StageJob j{};
        if (bound[i] > 0.0) {
            // one pass per operand: exponents and the partial sums of squares
            unsigned long long *pa = reinterpret_cast<unsigned long long *>(at(so[i].pa));
            unsigned long long *pbp = reinterpret_cast<unsigned long long *>(at(so[i].pb));
            j.kind = JOB_STATS, j.X = pb.A, j.ld = pb.lda, j.rows = pb.M, j.cols = pb.K;
            j.e_out = er, j.e_out2 = nullptr, j.prow = pa, j.pcol = pa + stats_layout(pb.M, pb.K).row_n;
            ja.add(j);
            j = StageJob{};
            j.kind = JOB_STATS, j.X = pb.B, j.ld = pb.ldb, j.rows = pb.K, j.cols = pb.N;
            j.e_out = nullptr, j.e_out2 = ec, j.prow = pbp, j.pcol = pbp + stats_layout(pb.K, pb.N).row_n;
            ja.add(j);
            Operands op{pb.M, pb.N, pb.K, pb.A, pb.lda, pb.B, pb.ldb, pb.C, pb.ldc};
            KnobJob kjb = knob_job(op, er, ec, pa, pbp);
            kjb.out = reinterpret_cast<double *>(knob_dev + adapt_idx[i]);
            kj.push_back(kjb);
        } else {
            j.kind = JOB_ROWMAX, j.X = pb.A, j.ld = pb.lda, j.rows = pb.M, j.cols = pb.K;
            j.e_out = er;
            ja.add(j);
            j = StageJob{};
            j.kind = JOB_COLMAX, j.X = pb.B, j.ld = pb.ldb, j.rows = pb.K, j.cols = pb.N;
            j.e_out = ec;
            ja.add(j);
        }
    }
    ja.block0.push_back(ja.total);
    if (!replay1) {
        dja = put_table(h, ja.jobs, &toff, st);
        dba = put_table(h, ja.block0, &toff, st);
        if (!kj.empty()) dkj = put_table(h, kj, &toff, st);
    }
    const size_t toff2 = align256(sizeof(StageJob) * 4 * n) + align256(sizeof(int) * (4 * n + 1)) +
                         align256(sizeof(KnobJob) * (n_adapt + 1));
    if (prof) cudaEventRecord(h->ev[0], st);
    ozgb_status rc = run_phase(h, graph, key1, &h->gkey1, &h->gexec1, st, [&](cudaStream_t s) -> ozgb_status {
        // column maxima and sums are accumulated atomically: start from zero
        cudaMemsetAsync(gs, 0, total, s);
        launch_stage_jobs(dja, dba, static_cast<int>(ja.jobs.size()), ja.total, s);
        if (n_adapt > 0) {
            launch_knob_grouped(dkj, n_adapt, s);
            cudaMemcpyAsync(h->knob_host, knob_dev, sizeof(KnobStats) * n_adapt, cudaMemcpyDeviceToHost, s);
        }
        return OZGB_OK;
    });
    if (rc) return rc;
    h->launches += 1 + (n_adapt > 0 ? 1 : 0);
    if (prof) cudaEventRecord(h->ev[1], st);

    // ---- precision knob: slice counts from the read-back statistics
    std::vector<Schedule> s_pick(n);
    if (n_adapt > 0) {
        const cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(h, e, "grouped statistics readback");
        for (int i = 0; i < n; ++i)
            if (bound[i] > 0.0) {
                OzConfig base = resolve_config(h, probs[i].K, mode);
                base.b = 7;
                s_pick[i] = choose_schedule(h->knob_host[adapt_idx[i]], probs[i].M, probs[i].N, probs[i].K, base,
                                            bound[i], 2, 16, h->err_crit, h->err_tail, h->sched_any != 0,
                                            sm_count(h->device));
            }
    }

    // ---- plans
    std::vector<Plan> plans(n);
    for (int i = 0; i < n; ++i) {
        OzConfig cfg = resolve_config(h, probs[i].K, mode);
        if (s_pick[i].s > 0) {
            cfg.b = 7;
            cfg.s = s_pick[i].s;
            cfg.J = s_pick[i].J;
        }
        std::string why;
        if (!make_plan(probs[i].M, probs[i].N, probs[i].K, cfg, &plans[i], &why))
            return fail(h, OZGB_ERR_UNSUPPORTED, "problem " + std::to_string(i) + ": " + why);
        probs[i].slices_used = plans[i].cfg.s;
        probs[i].bins_used = plans[i].cfg.J;
    }
    // ---- phase 2: stage (b) for every problem (one launch) and the GEMMs
    std::vector<size_t> a_off(n), b_off(n);
    size_t sl_total = 0;
    for (int i = 0; i < n; ++i) {
        a_off[i] = sl_total;
        sl_total += align256(plans[i].a_bytes);
        b_off[i] = sl_total;
        sl_total += align256(plans[i].b_bytes);
    }
    if (!h->gslice.ensure(sl_total)) return fail(h, OZGB_ERR_ALLOC, "grouped slice buffer");
    uint8_t *gsl = static_cast<uint8_t *>(h->gslice.p);
    if ((rc = ensure_aux(h))) return rc;
    std::vector<long long> key2 = key1;
    key2.insert(key2.end(), {reinterpret_cast<long long>(gsl), reinterpret_cast<long long>(h->err.p),
                             static_cast<long long>(h->timeout_ns)});
    for (int i = 0; i < n; ++i) {
        const Plan &p = plans[i];
        key2.insert(key2.end(), {reinterpret_cast<long long>(probs[i].C), probs[i].ldc, p.cfg.b, p.cfg.s, p.cfg.J,
                                 p.cfg.rounding, p.BN, p.KC, p.stages, p.G});
    }
    // grouped GEMM launches (one per plan class) and their problem tables; the
    // tables are uploaded unless the captured graph of the same calls is replayed
    std::vector<GroupLaunch> launches;
    if (h->grouped_launch) {
        std::vector<const uint8_t *> a_t(n), b_t(n);
        std::vector<const int32_t *> e_r(n), e_c(n);
        for (int i = 0; i < n; ++i) {
            a_t[i] = gsl + a_off[i];
            b_t[i] = gsl + b_off[i];
            e_r[i] = reinterpret_cast<const int32_t *>(at(so[i].er));
            e_c[i] = reinterpret_cast<const int32_t *>(at(so[i].ec));
        }
        launches = build_group_launches(probs, n, plans, a_t, b_t, e_r, e_c, static_cast<int *>(h->err.p),
                                        h->timeout_ns);
        size_t bytes = 0;
        for (const GroupLaunch &L : launches)
            bytes += align256(sizeof(GroupProblem) * L.probs.size()) + align256(sizeof(int) * L.tile_prob.size());
        if (!h->gprob.ensure(bytes)) return fail(h, OZGB_ERR_ALLOC, "grouped problem tables");
        uint8_t *base = static_cast<uint8_t *>(h->gprob.p);
        size_t off = 0;
        for (GroupLaunch &L : launches) {
            L.g.probs = reinterpret_cast<GroupProblem *>(base + off);
            off += align256(sizeof(GroupProblem) * L.probs.size());
            L.g.tile_prob = reinterpret_cast<int *>(base + off);
            off += align256(sizeof(int) * L.tile_prob.size());
            const std::vector<long long> lk = launch_key(L.g, *L.plan);
            key2.insert(key2.end(), lk.begin(), lk.end());
            key2.insert(key2.end(), {reinterpret_cast<long long>(L.g.probs), static_cast<long long>(L.probs.size())});
        }
    }
    key2.push_back(h->grouped_launch);
    const bool replay2 = graph && h->gexec2 && h->gkey2 == key2;
    if (h->grouped_launch && !replay2) {
        for (GroupLaunch &L : launches) {
            const cudaError_t e1 = cudaMemcpyAsync(const_cast<GroupProblem *>(L.g.probs), L.probs.data(),
                                                   sizeof(GroupProblem) * L.probs.size(), cudaMemcpyHostToDevice, st);
            const cudaError_t e2 = cudaMemcpyAsync(const_cast<int *>(L.g.tile_prob), L.tile_prob.data(),
                                                   sizeof(int) * L.tile_prob.size(), cudaMemcpyHostToDevice, st);
            if (e1 != cudaSuccess || e2 != cudaSuccess)
                return cuda_fail(h, e1 != cudaSuccess ? e1 : e2, "grouped problem table upload");
        }
    }
    JobList jb;
    for (int i = 0; i < n; ++i) {
        const ozgb_problem &pb = probs[i];
        const Plan &p = plans[i];
        StageJob j{};
        j.kind = JOB_SPLIT_A, j.X = pb.A, j.ld = pb.lda, j.rows = pb.M, j.cols = pb.K;
        j.e_in = reinterpret_cast<int32_t *>(at(so[i].er));
        j.b = p.cfg.b, j.s = p.cfg.s, j.KC = p.KC, j.n_kc = p.n_kc, j.padded = p.Mp, j.BN = p.BN;
        j.f8 = p.f8 ? 1 : 0;
        j.tiles = reinterpret_cast<uint16_t *>(gsl + a_off[i]);
        jb.add(j);
        j.kind = JOB_SPLIT_B, j.X = pb.B, j.ld = pb.ldb, j.rows = pb.K, j.cols = pb.N;
        j.e_in = reinterpret_cast<int32_t *>(at(so[i].ec));
        j.padded = p.Np;
        j.tiles = reinterpret_cast<uint16_t *>(gsl + b_off[i]);
        jb.add(j);
    }
    jb.block0.push_back(jb.total);
    const StageJob *djb = nullptr;
    const int *dbb = nullptr;
    if (!replay2) {
        toff = toff2;
        djb = put_table(h, jb.jobs, &toff, st);
        dbb = put_table(h, jb.block0, &toff, st);
    }
    // the GEMMs: one persistent launch per plan class (grouped_launch), or one per
    // problem, largest first, spread over the auxiliary streams
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return static_cast<double>(plans[x].tiles_m) * plans[x].tiles_n * plans[x].n_kc * plans[x].pairs >
               static_cast<double>(plans[y].tiles_m) * plans[y].tiles_n * plans[y].n_kc * plans[y].pairs;
    });
    const int n_streams = h->grouped_launch ? static_cast<int>(launches.size()) : n;
    const int n_aux = std::max(1, std::min(n_streams, static_cast<int>(ozgb_context::kAux)));
    rc = run_phase(h, graph, key2, &h->gkey2, &h->gexec2, st, [&](cudaStream_t s) -> ozgb_status {
        launch_stage_jobs(djb, dbb, static_cast<int>(jb.jobs.size()), jb.total, s);
        if (prof) cudaEventRecord(h->ev[2], s);
        cudaEventRecord(h->ev_fork, s);
        for (int a = 0; a < n_aux; ++a) cudaStreamWaitEvent(h->aux[a], h->ev_fork, 0);
        for (size_t l = 0; l < launches.size(); ++l) {
            const GroupLaunch &L = launches[l];
            L.plan->fn(L.g, L.g.total_tiles, L.plan->smem, h->aux[l % n_aux]);
        }
        for (int r = 0; r < n && !h->grouped_launch; ++r) {
            const int k = order[r];
            const Plan &p = plans[k];
            GemmArgs g;
            gemm_args_from_plan(&g, p, p.cfg.rounding, static_cast<int *>(h->err.p), h->timeout_ns);
            g.a_tiles = reinterpret_cast<const uint16_t *>(gsl + a_off[k]);
            g.b_tiles = reinterpret_cast<const uint16_t *>(gsl + b_off[k]);
            g.er = reinterpret_cast<const int32_t *>(at(so[k].er));
            g.ec = reinterpret_cast<const int32_t *>(at(so[k].ec));
            g.c = probs[k].C;
            g.ldc = probs[k].ldc;
            g.M = probs[k].M;
            g.N = probs[k].N;
            g.n_kc = p.n_kc;
            g.tiles_m = p.tiles_m;
            g.tiles_n = p.tiles_n;
            // no K-split here: the problems running side by side already fill the
            // SMs, and a split only adds work (measured: 7 % lower throughput)
            g.total_tiles = p.tiles_m * p.tiles_n;
            p.fn(g, g.total_tiles, p.smem, h->aux[r % n_aux]);
        }
        for (int a = 0; a < n_aux; ++a) {
            cudaEventRecord(h->ev_join[a], h->aux[a]);
            cudaStreamWaitEvent(s, h->ev_join[a], 0);
        }
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? OZGB_OK : cuda_fail(h, e, "grouped slice-pair GEMM launches");
    });
    if (rc) return rc;
    h->launches += 1 + (h->grouped_launch ? static_cast<long long>(launches.size()) : n);
    if (prof) {
        cudaEventRecord(h->ev[3], st);
        h->ev_recorded = true;
    }
    h->last = plans[n - 1];
    h->have_last = true;
    return OZGB_OK;
}

bool valid_mode(int mode) { return mode == OZGB_MODE_ACCURATE || mode == OZGB_MODE_FAST; }

void fill_blocks(const Plan &p, ozgb_config *out) {
    out->blocks = p.G;
    out->umma_per_kstep = p.mma_per_kstep;
    out->issuers = p.n_iss;
    out->slice_format = p.f8 ? 1 : 0;
    out->dbl_blocks = static_cast<int>(p.dbl_mask);
    for (int i = 0; i < 8; ++i) {
        out->block_lo[i] = i < p.G ? p.blk_lo[i] : 0;
        out->block_nb[i] = i < p.G ? p.blk_nb[i] : 0;
    }
}

}  // namespace

extern "C" {

const char *ozgb_version(void) { return "oz-gb300 0.1 (sm_103a, tcgen05 kind::f16 carrier)"; }

ozgb_status ozgb_create(ozgb_handle *out) {
    if (!out) return OZGB_ERR_ARG;
    *out = new (std::nothrow) ozgb_context();
    return *out ? OZGB_OK : OZGB_ERR_ALLOC;
}

ozgb_status ozgb_release(ozgb_handle h) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (h->device >= 0) cudaSetDevice(h->device);
    for (DevBuf *b : {&h->a, &h->b, &h->c, &h->at, &h->bt, &h->er, &h->ec, &h->raw, &h->knob, &h->kpart, &h->gstat,
                      &h->gslice, &h->gtab, &h->split})
        b->release();
    h->split_dirty = true;
    // captured grouped graphs refer to the released buffers
    if (h->gexec1) cudaGraphExecDestroy(h->gexec1);
    if (h->gexec2) cudaGraphExecDestroy(h->gexec2);
    h->gexec1 = h->gexec2 = nullptr;
    h->gkey1.clear();
    h->gkey2.clear();
    h->setup_done = false;
    return OZGB_OK;
}

ozgb_status ozgb_destroy(ozgb_handle h) {
    if (!h) return OZGB_ERR_ARG;
    ozgb_release(h);
    if (h->device >= 0) {
        cudaSetDevice(h->device);
        h->err.release();
        for (auto &ev : h->ev)
            if (ev) cudaEventDestroy(ev);
        if (h->stream) cudaStreamDestroy(h->stream);
        for (int i = 0; i < ozgb_context::kAux; ++i) {
            if (h->aux[i]) cudaStreamDestroy(h->aux[i]);
            if (h->ev_join[i]) cudaEventDestroy(h->ev_join[i]);
        }
        if (h->ev_fork) cudaEventDestroy(h->ev_fork);
        if (h->ev_part) cudaEventDestroy(h->ev_part);
        if (h->ev_part_copied) cudaEventDestroy(h->ev_part_copied);
        if (h->knob_host) cudaFreeHost(h->knob_host);
    }
    delete h;
    return OZGB_OK;
}

ozgb_status ozgb_setup(ozgb_handle h, int M, int N, int K, int mode) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (M < 1 || N < 1 || K < 1) return fail(h, OZGB_ERR_DIMS, "dimensions must be positive");
    if (!valid_mode(mode)) return fail(h, OZGB_ERR_ARG, "mode must be accurate (0) or fast (1)");
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    OzConfig cfg = resolve_config(h, K, mode);
    Plan p;
    std::string why;
    if (!make_plan(M, N, K, cfg, &p, &why)) return fail(h, OZGB_ERR_UNSUPPORTED, why);
    const size_t nA = static_cast<size_t>(M) * K, nB = static_cast<size_t>(K) * N, nC = static_cast<size_t>(M) * N;
    if (!h->a.ensure(nA * 8) || !h->b.ensure(nB * 8) || !h->c.ensure(nC * 8) || !h->at.ensure(p.a_bytes) ||
        !h->bt.ensure(p.b_bytes) || !h->er.ensure(4 * M) || !h->ec.ensure(4 * N))
        return fail(h, OZGB_ERR_ALLOC, "device buffers for the setup shape");
    h->M = M;
    h->N = N;
    h->K = K;
    h->mode = mode;
    h->setup_done = true;
    h->last = p;
    h->have_last = true;
    return OZGB_OK;
}

ozgb_status ozgb_dgemm(ozgb_handle h, int M, int N, int K, const double *A, const double *B, double *C) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->setup_done) return fail(h, OZGB_ERR_NOT_SETUP, "ozgb_setup must be called first");
    if (M != h->M || N != h->N || K != h->K)
        return fail(h, OZGB_ERR_DIM_MISMATCH, "dimensions differ from the last setup");
    if (!A || !B || !C) return fail(h, OZGB_ERR_ARG, "null matrix pointer");
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    const size_t nA = static_cast<size_t>(M) * K, nB = static_cast<size_t>(K) * N, nC = static_cast<size_t>(M) * N;
    if (!h->a.ensure(nA * 8) || !h->b.ensure(nB * 8) || !h->c.ensure(nC * 8))
        return fail(h, OZGB_ERR_ALLOC, "operand buffers");
    cudaStream_t st = h->stream;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h->a.p, A, nA * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(h, e, "copy A");
    if ((e = cudaMemcpyAsync(h->b.p, B, nB * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(h, e, "copy B");
    Operands o{M, N, K, static_cast<double *>(h->a.p), K, static_cast<double *>(h->b.p), N,
               static_cast<double *>(h->c.p), N};
    // (Storing C into host memory straight from the epilogue, which the device can
    // do over NVLink-C2C, measured slower than the copy at 1024^3 to 4096^3.)
    HostOut ho{C, false};
    if ((rc = enqueue_dgemm(h, o, h->mode, st, -1, 0, kMaxBins, nullptr, &ho))) {
        cudaStreamSynchronize(st);
        return rc;
    }
    if (!ho.copied && (e = cudaMemcpyAsync(C, h->c.p, nC * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "copy C");
    return check_device_error(h, st);
}

ozgb_status ozgb_dgemm_device(ozgb_handle h, int M, int N, int K, const double *dA, long lda, const double *dB,
                              long ldb, double *dC, long ldc, void *stream) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (M < 1 || N < 1 || K < 1) return fail(h, OZGB_ERR_DIMS, "dimensions must be positive");
    if (!dA || !dB || !dC) return fail(h, OZGB_ERR_ARG, "null matrix pointer");
    if (lda < K || ldb < N || ldc < N) return fail(h, OZGB_ERR_ARG, "leading dimension too small");
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL: the default (legacy) stream
    Operands o{M, N, K, dA, lda, dB, ldb, dC, ldc};
    return enqueue_dgemm(h, o, h->setup_done ? h->mode : OZGB_MODE_FAST, st);
}

ozgb_status ozgb_dgemm_ex(ozgb_handle h, int transa, int transb, int M, int N, int K, double alpha, const double *dA,
                          long lda, const double *dB, long ldb, double beta, double *dC, long ldc, void *stream) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (M < 1 || N < 1 || K < 1) return fail(h, OZGB_ERR_DIMS, "dimensions must be positive");
    if (!dA || !dB || !dC) return fail(h, OZGB_ERR_ARG, "null matrix pointer");
    if ((transa ? lda < M : lda < K) || (transb ? ldb < K : ldb < N) || ldc < N)
        return fail(h, OZGB_ERR_ARG, "leading dimension too small");
    if (!std::isfinite(alpha) || !std::isfinite(beta)) return fail(h, OZGB_ERR_ARG, "alpha and beta must be finite");
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Operands o{M, N, K, dA, lda, dB, ldb, dC, ldc};
    o.ta = transa != 0;
    o.tb = transb != 0;
    o.alpha = alpha;
    o.beta = beta;
    if (alpha == 0.0) {
        // C = beta * C: A and B are not read, as BLAS does
        h->last_stream = st;
        launch_scale(dC, ldc, M, N, beta, st);
        h->launches += 1;
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? OZGB_OK : cuda_fail(h, e, "scale launch");
    }
    return enqueue_dgemm(h, o, h->setup_done ? h->mode : OZGB_MODE_FAST, st);
}

ozgb_status ozgb_sync(ozgb_handle h) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (h->device < 0) return fail(h, OZGB_ERR_NO_DEVICE, "no call was made on a device");
    cudaSetDevice(h->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(h, e, "device synchronize");
    return check_device_error(h, h->last_stream);
}

ozgb_status ozgb_dgemm_grouped(ozgb_handle h, ozgb_problem *probs, int n, void *stream) {
    if (!h || (!probs && n > 0) || n < 0) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (n == 0) return OZGB_OK;
    for (int i = 0; i < n; ++i) {
        const ozgb_problem &pb = probs[i];
        if (pb.M < 1 || pb.N < 1 || pb.K < 1) return fail(h, OZGB_ERR_DIMS, "problem dimensions must be positive");
        if (!pb.A || !pb.B || !pb.C) return fail(h, OZGB_ERR_ARG, "null matrix pointer in a problem");
        if (pb.lda < pb.K || pb.ldb < pb.N || pb.ldc < pb.N)
            return fail(h, OZGB_ERR_ARG, "leading dimension too small in a problem");
    }
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    h->last_stream = st;
    const int mode = h->setup_done ? h->mode : OZGB_MODE_FAST;
    return enqueue_grouped(h, probs, n, mode, st);
}

ozgb_status ozgb_set_profile(ozgb_handle h, int profile) {
    if (!h || (profile != OZGB_PROFILE_GB300 && profile != OZGB_PROFILE_REFERENCE)) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->profile = profile;
    return OZGB_OK;
}
ozgb_status ozgb_set_bits(ozgb_handle h, int bits) {
    if (!h || bits < 0 || bits > 7) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->opt_bits = bits;
    return OZGB_OK;
}
ozgb_status ozgb_set_slices(ozgb_handle h, int slices) {
    if (!h || slices < 0 || slices > 40) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->opt_slices = slices;
    return OZGB_OK;
}
ozgb_status ozgb_set_bins(ozgb_handle h, int bins) {
    if (!h || bins < -1 || bins > kMaxBins) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->opt_bins = bins;
    return OZGB_OK;
}
ozgb_status ozgb_set_rounding(ozgb_handle h, int rounding) {
    if (!h || rounding < -1 || rounding > 1) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->opt_rounding = rounding;
    return OZGB_OK;
}
ozgb_status ozgb_set_slice_format(ozgb_handle h, int format) {
    if (!h || format < 0 || format > 1) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->opt_format = format;
    return OZGB_OK;
}
ozgb_status ozgb_set_plan_hint(ozgb_handle h, int tile_n, int k_chunk, int stages, int issuers, int dbl, int blocks,
                               const int *block_nb) {
    if (!h || tile_n < 0 || k_chunk < 0 || stages < 0 || issuers < 0 || issuers > kMaxIssuers || dbl < -1 ||
        dbl > 1 || blocks < 0 || blocks > kMaxGroups || (blocks > 0 && !block_nb))
        return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    PlanHints ph;
    ph.BN = tile_n;
    ph.KC = k_chunk;
    ph.stages = stages;
    ph.issuers = issuers;
    ph.dbl = dbl;
    ph.groups = blocks;
    for (int i = 0; i < blocks; ++i) ph.sizes[i] = block_nb[i];
    h->plan_hint = ph;
    h->have_plan_hint = tile_n || k_chunk || stages || issuers || dbl != -1 || blocks;
    return OZGB_OK;
}
ozgb_status ozgb_set_error_bound(ozgb_handle h, double bound) {
    if (!h || !(bound >= 0.0)) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->err_bound = bound;
    return OZGB_OK;
}
ozgb_status ozgb_set_error_criterion(ozgb_handle h, int criterion, double tail) {
    if (!h || (criterion != OZGB_CRIT_NORMWISE && criterion != OZGB_CRIT_ELEMENTWISE) || !(tail > 0.0) ||
        !(tail <= 1.0))
        return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->err_crit = criterion;
    h->err_tail = tail;
    return OZGB_OK;
}
ozgb_status ozgb_set_schedule_search(ozgb_handle h, int any_pair_set) {
    if (!h || any_pair_set < 0 || any_pair_set > 1) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->sched_any = any_pair_set;
    return OZGB_OK;
}
ozgb_status ozgb_set_grouped_launch(ozgb_handle h, int mode) {
    if (!h || mode < 0 || mode > 1) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->grouped_launch = mode;
    return OZGB_OK;
}
ozgb_status ozgb_set_graph(ozgb_handle h, int enable) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->use_graph = enable ? 1 : 0;
    return OZGB_OK;
}
ozgb_status ozgb_set_timeout_ms(ozgb_handle h, double ms) {
    if (!h || !(ms > 0.0)) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->timeout_ns = static_cast<unsigned long long>(ms * 1e6);
    return OZGB_OK;
}
ozgb_status ozgb_set_profiling(ozgb_handle h, int enable) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    h->profiling = enable != 0;
    h->ev_recorded = false;
    return OZGB_OK;
}

ozgb_status ozgb_stage_times(ozgb_handle h, float *ms, int n) {
    if (!h || !ms || n < 1) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->ev_recorded) return fail(h, OZGB_ERR_ARG, "no profiled call recorded");
    cudaEventSynchronize(h->ev[3]);
    float t[4] = {0, 0, 0, 0};
    cudaEventElapsedTime(&t[0], h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&t[1], h->ev[1], h->ev[2]);
    cudaEventElapsedTime(&t[2], h->ev[2], h->ev[3]);
    cudaEventElapsedTime(&t[3], h->ev[0], h->ev[3]);
    for (int i = 0; i < n && i < 4; ++i) ms[i] = t[i];
    return OZGB_OK;
}

ozgb_status ozgb_launch_count(ozgb_handle h, long long *count) {
    if (!h || !count) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    *count = h->launches;
    return OZGB_OK;
}

ozgb_status ozgb_get_config(ozgb_handle h, ozgb_config *out) {
    if (!h || !out) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->have_last) return fail(h, OZGB_ERR_NOT_SETUP, "no setup or call yet");
    const Plan &p = h->last;
    out->bits = p.cfg.b;
    out->slices = p.cfg.s;
    out->bins = p.cfg.J;
    out->rounding = p.cfg.rounding;
    out->tile_n = p.BN;
    out->k_chunk = p.KC;
    out->stages = p.stages;
    out->drain_chunks = p.min_period;
    out->acc_words = p.W;
    out->pairs = p.pairs;
    fill_blocks(p, out);
    return OZGB_OK;
}

const char *ozgb_last_error(ozgb_handle h) { return h ? h->msg.c_str() : "null handle"; }

ozgb_status ozgb_dump_pairs(ozgb_handle h, int M, int N, int K, const double *A, const double *B, int64_t *pairs) {
    if (!h || !A || !B || !pairs) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (M < 1 || N < 1 || K < 1) return fail(h, OZGB_ERR_DIMS, "dimensions must be positive");
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    cudaStream_t st = h->stream;
    const size_t nA = static_cast<size_t>(M) * K, nB = static_cast<size_t>(K) * N, nC = static_cast<size_t>(M) * N;
    if (!h->a.ensure(nA * 8) || !h->b.ensure(nB * 8) || !h->c.ensure(nC * 8) || !h->raw.ensure(nC * 16))
        return fail(h, OZGB_ERR_ALLOC, "dump buffers");
    cudaMemcpyAsync(h->a.p, A, nA * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(h->b.p, B, nB * 8, cudaMemcpyHostToDevice, st);
    Operands o{M, N, K, static_cast<double *>(h->a.p), K, static_cast<double *>(h->b.p), N,
               static_cast<double *>(h->c.p), N};
    if ((rc = enqueue_dgemm(h, o, h->setup_done ? h->mode : OZGB_MODE_FAST, st, OUT_PAIRS, 0, kMaxBins,
                            static_cast<int32_t *>(h->raw.p))))
        return rc;
    if ((rc = check_device_error(h, st))) return rc;
    const cudaError_t e = cudaMemcpy(pairs, h->raw.p, nC * 16, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? OZGB_OK : cuda_fail(h, e, "pairs readback");
}

ozgb_status ozgb_dump(ozgb_handle h, int M, int N, int K, const double *A, const double *B, int32_t *er, int32_t *ec,
                      int8_t *a_slices, int8_t *b_slices, int32_t *q, int bin_lo, int bin_hi) {
    if (!h || !A || !B) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (M < 1 || N < 1 || K < 1) return fail(h, OZGB_ERR_DIMS, "dimensions must be positive");
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    cudaStream_t st = h->stream;
    const size_t nA = static_cast<size_t>(M) * K, nB = static_cast<size_t>(K) * N, nC = static_cast<size_t>(M) * N;
    if (!h->a.ensure(nA * 8) || !h->b.ensure(nB * 8) || !h->c.ensure(nC * 8) || !h->raw.ensure(nC * 16))
        return fail(h, OZGB_ERR_ALLOC, "dump buffers");
    cudaMemcpyAsync(h->a.p, A, nA * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(h->b.p, B, nB * 8, cudaMemcpyHostToDevice, st);
    Operands o{M, N, K, static_cast<double *>(h->a.p), K, static_cast<double *>(h->b.p), N,
               static_cast<double *>(h->c.p), N};
    if ((rc = enqueue_dgemm(h, o, h->setup_done ? h->mode : OZGB_MODE_FAST, st, OUT_RAW, bin_lo, bin_hi,
                            static_cast<int32_t *>(h->raw.p))))
        return rc;
    if ((rc = check_device_error(h, st))) return rc;
    const Plan &p = h->last;
    if (er) cudaMemcpy(er, h->er.p, 4 * M, cudaMemcpyDeviceToHost);
    if (ec) cudaMemcpy(ec, h->ec.p, 4 * N, cudaMemcpyDeviceToHost);
    if (q) cudaMemcpy(q, h->raw.p, nC * 16, cudaMemcpyDeviceToHost);
    const int s = p.cfg.s;
    auto bf16_to_int = [](uint16_t v) {
        uint32_t u = static_cast<uint32_t>(v) << 16;
        float f;
        memcpy(&f, &u, 4);
        return static_cast<int8_t>(f);
    };
    if (a_slices) {
        std::vector<uint16_t> t(p.a_elems);
        cudaMemcpy(t.data(), h->at.p, p.a_elems * 2, cudaMemcpyDeviceToHost);
        for (int sl = 0; sl < s; ++sl)
            for (int m = 0; m < M; ++m)
                for (int k = 0; k < K; ++k) {
                    const size_t off = ((static_cast<size_t>(m >> 7) * p.n_kc + k / p.KC) * s + sl) * BM * p.KC +
                                       canon_offset(m & 127, k % p.KC, p.KC);
                    a_slices[(static_cast<size_t>(sl) * M + m) * K + k] = bf16_to_int(t[off]);
                }
    }
    if (b_slices) {
        std::vector<uint16_t> t(p.b_elems);
        cudaMemcpy(t.data(), h->bt.p, p.b_elems * 2, cudaMemcpyDeviceToHost);
        for (int sl = 0; sl < s; ++sl)
            for (int k = 0; k < K; ++k)
                for (int n = 0; n < N; ++n) {
                    const size_t off = ((static_cast<size_t>(n / p.BN) * p.n_kc + k / p.KC) * s + sl) *
                                           static_cast<size_t>(p.BN) * p.KC +
                                       canon_offset(n % p.BN, k % p.KC, p.KC);
                    b_slices[(static_cast<size_t>(sl) * K + k) * N + n] = bf16_to_int(t[off]);
                }
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? OZGB_OK : cuda_fail(h, e, "dump readback");
}

ozgb_status ozgb_selftest_timeout(ozgb_handle h, double timeout_ms) {
    if (!h || !(timeout_ms > 0.0)) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    launch_selftest_timeout(static_cast<int *>(h->err.p), static_cast<unsigned long long>(timeout_ms * 1e6),
                            h->stream);
    h->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, "selftest launch");
    return check_device_error(h, h->stream);
}

// include/oz_aie.h:92-150 restated on the host: int128 = lo + sext51(hi) << (g0 b),
// truncated to 53 bits, exponent from the embedded Er+Ec.
ozgb_status ozgb_convert_paired_i64_to_double(const int64_t *C, double *result, int M, int N, int K, int num_splits,
                                              int bits_per_slice) {
    if (!C || !result || M < 0 || N < 0 || K < 1 || num_splits < 1 || bits_per_slice < 1) return OZGB_ERR_ARG;
    const int b = bits_per_slice, d = num_splits;
    const int alignable = 31 / b + 1;
    const int numer = b * (d + 1) - 51 + std::countr_zero(static_cast<unsigned>(K));
    const int minfirst = numer < 0 ? 1 : numer / b + 1;
    const int g0 = std::min(d, std::max(minfirst, alignable));
    for (long i = 0; i < static_cast<long>(M) * N; ++i) {
        const int64_t lo = C[2 * i], hi = C[2 * i + 1];
        const uint64_t escale = (static_cast<uint64_t>(hi) >> 51) & 0xFFFu;
        uint64_t hm = static_cast<uint64_t>(hi) & 0x0007FFFFFFFFFFFFull;
        if (hi < 0) hm |= 0xFFF8000000000000ull;
        __int128 quad = static_cast<__int128>(lo) + (static_cast<__int128>(static_cast<int64_t>(hm)) << (g0 * b));
        const bool neg = quad < 0;
        unsigned __int128 mag = neg ? static_cast<unsigned __int128>(-quad) : static_cast<unsigned __int128>(quad);
        const uint64_t mh = static_cast<uint64_t>(mag >> 64), ml = static_cast<uint64_t>(mag);
        const int L = mh ? 128 - std::countl_zero(mh) : (ml ? 64 - std::countl_zero(ml) : 0);
        const long long exponent = static_cast<long long>(L) - b * (d + 1) - 1;
        const int shift = L - 53;
        uint64_t lu = shift > 0 ? static_cast<uint64_t>(mag >> shift) : static_cast<uint64_t>(mag << -shift);
        if (lu > 0) {
            lu -= 0x0010000000000000ull;
            lu += (neg ? 0x8000000000000000ull : 0ull) + (static_cast<uint64_t>(exponent + 1023) << 52) +
                  (static_cast<uint64_t>(static_cast<long long>(escale) + 2 - 2046) << 52);
        }
        memcpy(&result[i], &lu, 8);
    }
    return OZGB_OK;
}

// Host-only planning queries (no device needed): used by tests and tools.
ozgb_status ozgb_autotune(ozgb_handle h, int M, int N, int K, int bits, int slices, int bins, int max_candidates,
                          ozgb_config *best) {
    if (!h) return OZGB_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (M < 1 || N < 1 || K < 1) return fail(h, OZGB_ERR_DIMS, "dimensions must be positive");
    ozgb_status rc = ensure_device(h);
    if (rc) return rc;
    OzConfig cfg;
    cfg.b = bits;
    cfg.s = slices;
    cfg.J = bins > 0 ? bins : slices;
    cfg.rounding = OUT_RN;
    const std::vector<PlanHints> cands = plan_candidates(M, N, K, cfg, max_candidates > 0 ? max_candidates : 64);
    if (cands.empty()) return fail(h, OZGB_ERR_UNSUPPORTED, "no feasible plan for this configuration");
    cudaStream_t st = h->stream;
    if (!h->a.ensure(sizeof(double) * M * K) || !h->b.ensure(sizeof(double) * K * N) ||
        !h->c.ensure(sizeof(double) * M * N) || !h->er.ensure(sizeof(int32_t) * M) || !h->ec.ensure(sizeof(int32_t) * N))
        return fail(h, OZGB_ERR_ALLOC, "autotune buffers");
    const double *dA = static_cast<double *>(h->a.p), *dB = static_cast<double *>(h->b.p);
    launch_fill_random(static_cast<double *>(h->a.p), static_cast<size_t>(M) * K, 1, st);
    launch_fill_random(static_cast<double *>(h->b.p), static_cast<size_t>(K) * N, 2, st);
    cudaMemsetAsync(h->ec.p, 0, sizeof(int32_t) * N, st);
    launch_rowmax(dA, K, M, K, static_cast<int32_t *>(h->er.p), nullptr, st);
    launch_colmax(dB, N, K, N, static_cast<int32_t *>(h->ec.p), nullptr, st);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = 0.0f;
    int best_i = -1;
    Plan best_plan;
    for (size_t i = 0; i < cands.size(); ++i) {
        Plan p;
        std::string why;
        if (!make_plan(M, N, K, cfg, &p, &why, 0, 1 << 30, &cands[i])) continue;
        if (!h->at.ensure(p.a_bytes) || !h->bt.ensure(p.b_bytes)) continue;
        uint16_t *at = static_cast<uint16_t *>(h->at.p), *bt = static_cast<uint16_t *>(h->bt.p);
        launch_split_a(dA, K, M, K, static_cast<int32_t *>(h->er.p), p.cfg.b, p.cfg.s, p.KC, p.n_kc, p.Mp, at, st,
                       false, p.f8);
        launch_split_b(dB, N, K, N, static_cast<int32_t *>(h->ec.p), p.cfg.b, p.cfg.s, p.KC, p.n_kc, p.BN, p.Np, bt, st,
                       false, p.f8);
        GemmArgs g;
        gemm_args_from_plan(&g, p, OUT_RN, static_cast<int *>(h->err.p), h->timeout_ns);
        g.a_tiles = at;
        g.b_tiles = bt;
        g.er = static_cast<int32_t *>(h->er.p);
        g.ec = static_cast<int32_t *>(h->ec.p);
        g.c = static_cast<double *>(h->c.p);
        g.ldc = N;
        g.M = M;
        g.N = N;
        g.n_kc = p.n_kc;
        g.tiles_m = p.tiles_m;
        g.tiles_n = p.tiles_n;
        g.total_tiles = p.tiles_m * p.tiles_n;
        p.fn(g, g.total_tiles, p.smem, st);  // warm-up
        float t[3];
        for (float &ti : t) {
            cudaEventRecord(e0, st);
            p.fn(g, g.total_tiles, p.smem, st);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ti, e0, e1);
        }
        h->launches += 6;
        if ((rc = check_device_error(h, st))) break;
        std::sort(t, t + 3);
        if (best_i < 0 || t[1] < best_ms) {
            best_ms = t[1];
            best_i = static_cast<int>(i);
            best_plan = p;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (best_i < 0) return fail(h, OZGB_ERR_UNSUPPORTED, "no candidate plan ran");
    tune_store(M, N, K, cfg, cands[best_i]);
    if (best) {
        best->bits = best_plan.cfg.b;
        best->slices = best_plan.cfg.s;
        best->bins = best_plan.cfg.J;
        best->rounding = best_plan.cfg.rounding;
        best->tile_n = best_plan.BN;
        best->k_chunk = best_plan.KC;
        best->stages = best_plan.stages;
        best->drain_chunks = best_plan.min_period;
        best->acc_words = best_plan.W;
        best->pairs = best_plan.pairs;
        fill_blocks(best_plan, best);
    }
    return OZGB_OK;
}

int ozgb_grouped_layout_check(const ozgb_problem *probs, int n, int slices, int bins, int *launches_out,
                              long long *units_out) {
    if (!probs || n < 1 || slices < 1) return -1;
    OzConfig cfg;
    cfg.b = 7;
    cfg.s = slices;
    cfg.J = bins > 0 ? bins : slices;
    cfg.rounding = OUT_RN;
    std::vector<Plan> plans(n);
    for (int i = 0; i < n; ++i) {
        std::string why;
        if (probs[i].M < 1 || probs[i].N < 1 || probs[i].K < 1 || probs[i].ldc < probs[i].N) return -2;
        if (!make_plan(probs[i].M, probs[i].N, probs[i].K, cfg, &plans[i], &why)) return -3;
    }
    // stand-in device addresses laid out as enqueue_grouped lays them out
    const uintptr_t slice_base = uintptr_t(1) << 40, exp_base = uintptr_t(1) << 41;
    std::vector<const uint8_t *> a_t(n), b_t(n);
    std::vector<const int32_t *> e_r(n), e_c(n);
    std::vector<uintptr_t> a_lo(n), b_lo(n), er_lo(n), ec_lo(n);
    size_t sl = 0, ex = 0;
    for (int i = 0; i < n; ++i) {
        a_lo[i] = slice_base + sl;
        sl += align256(plans[i].a_bytes);
        b_lo[i] = slice_base + sl;
        sl += align256(plans[i].b_bytes);
        er_lo[i] = exp_base + ex;
        ex += align256(sizeof(int32_t) * probs[i].M);
        ec_lo[i] = exp_base + ex;
        ex += align256(sizeof(int32_t) * probs[i].N);
        a_t[i] = reinterpret_cast<const uint8_t *>(a_lo[i]);
        b_t[i] = reinterpret_cast<const uint8_t *>(b_lo[i]);
        e_r[i] = reinterpret_cast<const int32_t *>(er_lo[i]);
        e_c[i] = reinterpret_cast<const int32_t *>(ec_lo[i]);
    }
    int err_word = 0;
    const std::vector<GroupLaunch> launches =
        build_group_launches(probs, n, plans, a_t, b_t, e_r, e_c, &err_word, 1000000000ull);
    long long units = 0;
    std::map<uintptr_t, int> by_a;
    for (int i = 0; i < n; ++i) by_a[a_lo[i]] = i;
    std::vector<std::vector<char>> seen(n);
    for (int i = 0; i < n; ++i) seen[i].assign(static_cast<size_t>(plans[i].tiles_m) * plans[i].tiles_n, 0);
    for (const GroupLaunch &L : launches) {
        const GemmArgs &g = L.g;
        if (g.total_tiles != static_cast<int>(L.tile_prob.size()) || g.split_parts != 1) return -4;
        for (int u = 0; u < g.total_tiles; ++u) {
            const int pi = L.tile_prob[u];
            if (pi < 0 || pi >= static_cast<int>(L.probs.size())) return -5;
            const GroupProblem &P = L.probs[pi];
            TileRef tr;
            group_tile_ref(L.probs.data(), L.tile_prob.data(), u, g.a_block_bytes, g.b_block_bytes, &tr);
            // which caller problem this is: by its A slice address
            const auto found = by_a.find(reinterpret_cast<uintptr_t>(P.a_tiles));
            if (found == by_a.end()) return -6;
            const int i = found->second;
            const Plan &p = plans[i];
            if (p.fn != L.plan->fn || p.a_block_bytes != g.a_block_bytes || p.b_block_bytes != g.b_block_bytes ||
                p.stage_bytes != g.stage_bytes || p.n_kc != tr.n_kc)
                return -7;
            if (tr.mt < 0 || tr.mt >= p.tiles_m || tr.nt < 0 || tr.nt >= p.tiles_n) return -8;
            char &mark = seen[i][static_cast<size_t>(tr.mt) * p.tiles_n + tr.nt];
            if (mark) return -9;
            mark = 1;
            // the producer's bulk copies: chunks [0, n_kc) of the tile's A and B blocks
            const uintptr_t a0 = reinterpret_cast<uintptr_t>(tr.a_src), b0 = reinterpret_cast<uintptr_t>(tr.b_src);
            if (a0 < a_lo[i] || a0 + static_cast<size_t>(tr.n_kc) * g.a_block_bytes > a_lo[i] + p.a_bytes) return -10;
            if (b0 < b_lo[i] || b0 + static_cast<size_t>(tr.n_kc) * g.b_block_bytes > b_lo[i] + p.b_bytes) return -11;
            if ((a0 | b0) & 15) return -12;
            // the epilogue: rows below M and columns below N of the tile, C and exponents
            if (tr.M != probs[i].M || tr.N != probs[i].N || tr.c != probs[i].C || tr.ldc != probs[i].ldc) return -13;
            if (reinterpret_cast<uintptr_t>(tr.er) != er_lo[i] || reinterpret_cast<uintptr_t>(tr.ec) != ec_lo[i])
                return -14;
            if (tr.mt * BM >= tr.M || tr.nt * p.BN >= tr.N) return -15;  // every tile holds output
            ++units;
        }
    }
    for (int i = 0; i < n; ++i)
        for (char c : seen[i])
            if (!c) return -16;
    if (launches_out) *launches_out = static_cast<int>(launches.size());
    if (units_out) *units_out = units;
    return 0;
}

int ozgb_tuning_entries(void) { return tune_count(); }
void ozgb_tuning_clear(void) { tune_clear(); }

int ozgb_plan_query(int M, int N, int K, int bits, int slices, int bins, ozgb_config *out) {
    OzConfig c;
    c.b = bits;
    c.s = slices;
    c.J = bins;
    Plan p;
    std::string why;
    if (!make_plan(M, N, K, c, &p, &why)) return OZGB_ERR_UNSUPPORTED;
    if (out) {
        out->bits = p.cfg.b;
        out->slices = p.cfg.s;
        out->bins = p.cfg.J;
        out->rounding = p.cfg.rounding;
        out->tile_n = p.BN;
        out->k_chunk = p.KC;
        out->stages = p.stages;
        out->drain_chunks = p.min_period;
        out->acc_words = p.W;
        out->pairs = p.pairs;
        fill_blocks(p, out);
    }
    return OZGB_OK;
}

int ozgb_choose_slices(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N,
                       const double *sa_k, const double *sb_k, int K, int bits, double bound, double *estimate) {
    return ozgb_choose_slices_ex(er, ssr, M, ec, ssc, N, sa_k, sb_k, K, bits, bound, OZGB_CRIT_NORMWISE, 1e-4,
                                 estimate);
}

int ozgb_choose_schedule(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N,
                         const double *sa_k, const double *sb_k, int K, int bits, double bound, int criterion,
                         double tail, int any_pair_set, int sms, int *slices, int *bins, double *estimate) {
    if (!er || !ssr || !ec || !ssc || M < 1 || N < 1 || K < 1 || bits < 1 || bits > 7 || !(bound > 0) || sms < 1)
        return -1;
    if ((criterion != OZGB_CRIT_NORMWISE && criterion != OZGB_CRIT_ELEMENTWISE) || !(tail > 0.0) || !(tail <= 1.0))
        return -1;
    const KnobStats ks = knob_stats_host(er, ssr, M, ec, ssc, N, sa_k, sb_k, K);
    OzConfig base;
    base.b = bits;
    base.rounding = OUT_RN;
    const Schedule sc = choose_schedule(ks, M, N, K, base, bound, 2, 16, criterion, tail, any_pair_set != 0, sms);
    if (slices) *slices = sc.s;
    if (bins) *bins = sc.J;
    if (estimate) *estimate = sc.est;
    return 0;
}

int ozgb_choose_slices_ex(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N,
                          const double *sa_k, const double *sb_k, int K, int bits, double bound, int criterion,
                          double tail, double *estimate) {
    if (!er || !ssr || !ec || !ssc || M < 1 || N < 1 || K < 1 || bits < 1 || !(bound > 0)) return -1;
    if ((criterion != OZGB_CRIT_NORMWISE && criterion != OZGB_CRIT_ELEMENTWISE) || !(tail > 0.0) || !(tail <= 1.0))
        return -1;
    const KnobStats ks = knob_stats_host(er, ssr, M, ec, ssc, N, sa_k, sb_k, K);
    return choose_slices_stats(ks, K, bits, bound, 2, 16, estimate, criterion, tail);
}

}  // extern "C"
