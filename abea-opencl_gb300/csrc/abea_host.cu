// abea_host.cu — host orchestration and the C ABI (include/abea.h).
//
// Mirrors the reference's batch entry align_ocl(core, db) (GPU/align_cuda.c:391-943):
// flatten -> size buffers -> host-to-device copies -> pre/core/post -> device-to-host
// copies, but with one device slab per batch (reused across calls), all copies
// and kernels queued on one CUDA stream per context, per-stage CUDA-event timing,
// and status codes instead of printing and continuing.
#include <cuda_runtime.h>
#include <math.h>
#include <nvtx3/nvToolsExt.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "abea_internal.h"
#include "abea_launch.h"

using namespace abea;

// NVTX range over a host scope (shown by profilers that record NVTX; a no-op otherwise).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ---------------------------------------------------------------- errors
static thread_local std::string g_last_error;

static abea_status_t fail(abea_status_t st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

#define CUDA_TRY(call)                                                                   \
    do {                                                                                 \
        cudaError_t err__ = (call);                                                      \
        if (err__ != cudaSuccess) {                                                      \
            abea_status_t st__ = err__ == cudaErrorMemoryAllocation ? ABEA_ERR_OUT_OF_MEMORY \
                                                                    : ABEA_ERR_CUDA;     \
            return fail(st__, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(err__), \
                        __FILE__, __LINE__);                                             \
        }                                                                                \
    } while (0)

extern "C" const char* abea_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* abea_status_string(abea_status_t s) {
    switch (s) {
    case ABEA_OK: return "ok";
    case ABEA_ERR_INVALID_ARG: return "invalid argument";
    case ABEA_ERR_CAPACITY: return "alignment longer than its output slot";
    case ABEA_ERR_OUT_OF_MEMORY: return "out of memory";
    case ABEA_ERR_CUDA: return "CUDA error";
    case ABEA_ERR_TIMEOUT: return "device wait timed out";
    case ABEA_ERR_NO_DEVICE: return "no usable CUDA device";
    case ABEA_ERR_INTERNAL: return "internal consistency check failed";
    case ABEA_ERR_UNDEFINED: return "reference behaviour undefined for this read";
    }
    return "unknown status";
}

extern "C" const char* abea_version(void) { return "abea-gb300 0.1 (sm_103a)"; }

// ---------------------------------------------------------------- objects
// a batch's input mirror (at 0) and output mirror (at kAuxMirror), in one device block
constexpr size_t kAuxBytes = 64, kAuxMirror = 16;
static_assert(sizeof(InMirror) <= kAuxMirror && kAuxMirror + sizeof(OutMirror) <= kAuxBytes, "aux layout");

struct DevSlab {
    void* base = nullptr;
    size_t bytes = 0;
};

struct abea_batch {
    abea_ctx* ctx = nullptr;
    int32_t n_reads = 0;
    int32_t var_aware = 0;       // emissions use var (ABEA_OPT_VAR_AWARE at creation)
    std::vector<ReadDesc> reads;
    std::vector<int32_t> order;  // longest first
    std::vector<int32_t> dev_order;       // the batched form's order: wide reads, then the rest longest first
    std::vector<int32_t> dev_order_sent;  // the order last copied to the device
    int32_t n_wide = 0;          // leading reads of `order` run on the wide shape
    int32_t n_mid = 0;           // the reads after them run on the medium shape
    // sizes
    int64_t seq_bytes = 0, n_events_total = 0, ev_pad_total = 0, km_pad_total = 0,
            band_pad_total = 0, pair_cap = 0, band_cells = 0;
    int64_t trace_pad_total = 0;  // bands of kept traces
    int64_t ck_floats = 0;        // checkpoint records
    int32_t n_ck = 0;             // checkpointed reads (recompute scratch slots)
    int32_t n_spec = 0;           // block-parallel traceback scratch slots
    // device pointers (sub-ranges of the slab)
    DevSlab slab;
    ReadDesc* d_reads = nullptr;
    char* d_seq = nullptr;
    abea_event_t* d_ev = nullptr;
    abea_model_t* d_model = nullptr;
    float *d_ev_mean = nullptr, *d_km_gm = nullptr, *d_km_sd = nullptr, *d_km_rsd = nullptr,
          *d_km_k1 = nullptr, *d_last_col = nullptr;
    uint8_t* d_trace = nullptr;
    float* d_scores = nullptr;
    float* d_ck = nullptr;           // checkpoint records
    uint8_t* d_ck_scratch = nullptr; // one kCkBands-band trace segment per checkpointed read
    int32_t* d_spec = nullptr;       // cell maps of the wide reads' block-parallel tracebacks
    char* d_aux = nullptr;           // [0]: the InMirror; [kAuxMirror]: the OutMirror
    int32_t* d_band_k0 = nullptr;
    abea_aligned_pair_t* d_pairs = nullptr;
    int32_t* d_n_pairs = nullptr;
    float* d_best = nullptr;
    int32_t* d_status = nullptr;
    unsigned long long* d_slow = nullptr;
    int32_t* d_order = nullptr;
    int32_t* d_queue = nullptr;
    // adjoint
    int32_t *d_path_len = nullptr, *d_path_flags = nullptr, *d_best_event = nullptr, *d_adj_status = nullptr;
    double *d_grad_sc = nullptr, *d_gn = nullptr, *d_path_em = nullptr, *d_grad_model = nullptr;
    bool scores_kept = false;
    bool ran = false;
    abea_timing_t timing{};
    cudaGraphExec_t graph = nullptr;  // batched form: memsets + pre + fused core/post
    std::vector<uint64_t> carve;      // slab base and region sizes: every device pointer follows from them
    std::vector<uint64_t> graph_key;  // what the captured graph's launch arguments were built from
    int graph_launches = 0;           // kernels in the captured graph
    void* d_post = nullptr;           // abea_batch_postalign's outputs (allocated on first use)
    size_t post_bytes = 0;
};

struct abea_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    abea_mode_t mode = ABEA_MODE_PLAIN;
    int64_t store_scores = 0;
    int64_t use_graph = 1;
    int64_t long_read_bands = 0;
    int64_t mid_read_bands = 0;  // medium-shape threshold (0 = the autotuned value, else none)
    int64_t spin_limit = 1 << 22;
    int64_t var_aware = 0;
    int64_t trace_budget = 0;  // bytes of trace a read may keep (0 = every trace)
    int64_t wide_cluster = 0;  // batched form: wide reads on a cluster pair of blocks
    void* db_pin = nullptr;    // pinned staging of abea_align_db
    size_t db_pin_bytes = 0;
    int sm_count = 0;
    cudaEvent_t ev[8] = {};
    cudaEvent_t marker[16] = {};
    void* flush_buf = nullptr;
    size_t flush_bytes = 0;
    abea_batch* scratch = nullptr;  // reused by abea_align_batch / abea_align
    // serving stream: two device batches, their copy stream and events (created on first use)
    abea_batch* sslot[2] = {nullptr, nullptr};
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t sev[2][4] = {};  // per slot: uploaded, compute start, compute end, results copied
    char* h_aux = nullptr;  // pinned: abea_align_batch's mirrors, then its counters and statuses
    size_t h_aux_bytes = 0;
    std::map<uint64_t, int64_t> tuned;      // autotuned wide-shape threshold per workload signature
    std::map<uint64_t, int64_t> tuned_mid;  // autotuned medium-shape threshold per workload signature
};

// ---------------------------------------------------------------- context
extern "C" abea_status_t abea_ctx_create(abea_ctx_t** out, int device, abea_mode_t mode) {
    if (!out) return fail(ABEA_ERR_INVALID_ARG, "abea_ctx_create: null output pointer");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0)
        return fail(ABEA_ERR_NO_DEVICE, "abea_ctx_create: no CUDA device");
    if (device < 0 || device >= n)
        return fail(ABEA_ERR_INVALID_ARG, "abea_ctx_create: device %d out of range", device);
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    if (prop.major * 10 + prop.minor != 103)
        return fail(ABEA_ERR_NO_DEVICE,
                    "abea_ctx_create: device %d is sm_%d%d; this library is built for sm_103a only",
                    device, prop.major, prop.minor);
    abea_ctx* c = new (std::nothrow) abea_ctx();
    if (!c) return fail(ABEA_ERR_OUT_OF_MEMORY, "abea_ctx_create: host allocation failed");
    c->device = device;
    c->mode = mode;
    c->sm_count = prop.multiProcessorCount;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    for (int i = 0; i < 8 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
    for (int i = 0; i < 16 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->marker[i]);
    if (e != cudaSuccess) {
        abea_ctx_destroy(c);
        return fail(ABEA_ERR_CUDA, "abea_ctx_create: %s", cudaGetErrorString(e));
    }
    *out = c;
    return ABEA_OK;
}

static void free_batch_device(abea_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    if (b->slab.base) cudaFree(b->slab.base);
    b->slab = DevSlab{};
    if (b->d_post) cudaFree(b->d_post);
    b->d_post = nullptr;
    b->post_bytes = 0;
}

extern "C" void abea_batch_destroy(abea_batch_t* b) {
    if (!b) return;
    free_batch_device(b);
    delete b;
}

extern "C" void abea_ctx_destroy(abea_ctx_t* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->scratch) abea_batch_destroy(c->scratch);
    for (int i = 0; i < 2; ++i) {
        if (c->sslot[i]) abea_batch_destroy(c->sslot[i]);
        for (int j = 0; j < 4; ++j)
            if (c->sev[i][j]) cudaEventDestroy(c->sev[i][j]);
    }
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->h_aux) cudaFreeHost(c->h_aux);
    for (int i = 0; i < 8; ++i)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (int i = 0; i < 16; ++i)
        if (c->marker[i]) cudaEventDestroy(c->marker[i]);
    if (c->flush_buf) cudaFree(c->flush_buf);
    if (c->db_pin) cudaFreeHost(c->db_pin);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" abea_status_t abea_ctx_set_option(abea_ctx_t* c, abea_option_t opt, int64_t v) {
    if (!c) return fail(ABEA_ERR_INVALID_ARG, "abea_ctx_set_option: null context");
    switch (opt) {
    case ABEA_OPT_MODE:
        if (v != ABEA_MODE_PLAIN && v != ABEA_MODE_BATCHED)
            return fail(ABEA_ERR_INVALID_ARG, "unknown mode %lld", (long long)v);
        c->mode = (abea_mode_t)v;
        return ABEA_OK;
    case ABEA_OPT_STORE_SCORES: c->store_scores = v != 0; return ABEA_OK;
    case ABEA_OPT_USE_GRAPH: c->use_graph = v != 0; return ABEA_OK;
    case ABEA_OPT_LONG_READ_BANDS:
        if (v < 0) return fail(ABEA_ERR_INVALID_ARG, "negative band threshold");
        c->long_read_bands = v;
        return ABEA_OK;
    case ABEA_OPT_SPIN_LIMIT:
        if (v <= 0) return fail(ABEA_ERR_INVALID_ARG, "spin limit must be positive");
        c->spin_limit = v;
        return ABEA_OK;
    case ABEA_OPT_VAR_AWARE: c->var_aware = v != 0; return ABEA_OK;
    case ABEA_OPT_TRACE_BUDGET:
        if (v < 0) return fail(ABEA_ERR_INVALID_ARG, "trace budget must be >= 0");
        c->trace_budget = v;
        return ABEA_OK;
    case ABEA_OPT_WIDE_CLUSTER: c->wide_cluster = v != 0; return ABEA_OK;
    case ABEA_OPT_MEDIUM_READ_BANDS:
        if (v < 0) return fail(ABEA_ERR_INVALID_ARG, "negative band threshold");
        c->mid_read_bands = v;
        return ABEA_OK;
    }
    return fail(ABEA_ERR_INVALID_ARG, "unknown option %d", (int)opt);
}

extern "C" abea_status_t abea_ctx_get_option(abea_ctx_t* c, abea_option_t opt, int64_t* v) {
    if (!c || !v) return fail(ABEA_ERR_INVALID_ARG, "abea_ctx_get_option: null argument");
    switch (opt) {
    case ABEA_OPT_MODE: *v = c->mode; return ABEA_OK;
    case ABEA_OPT_STORE_SCORES: *v = c->store_scores; return ABEA_OK;
    case ABEA_OPT_USE_GRAPH: *v = c->use_graph; return ABEA_OK;
    case ABEA_OPT_LONG_READ_BANDS: *v = c->long_read_bands; return ABEA_OK;
    case ABEA_OPT_SPIN_LIMIT: *v = c->spin_limit; return ABEA_OK;
    case ABEA_OPT_VAR_AWARE: *v = c->var_aware; return ABEA_OK;
    case ABEA_OPT_TRACE_BUDGET: *v = c->trace_budget; return ABEA_OK;
    case ABEA_OPT_WIDE_CLUSTER: *v = c->wide_cluster; return ABEA_OK;
    case ABEA_OPT_MEDIUM_READ_BANDS: *v = c->mid_read_bands; return ABEA_OK;
    }
    return fail(ABEA_ERR_INVALID_ARG, "unknown option %d", (int)opt);
}

extern "C" void* abea_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    return p;
}
extern "C" void abea_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

// ---------------------------------------------------------------- planning
struct Penalties {
    double lp_skip, lp_stay, lp_step, lp_trim;
};

// Transition log-probabilities of a read, computed on the host with the C
// library's log/exp exactly as the reference does (align_swi.cl:233-250).
static Penalties penalties(int32_t n_events, int32_t n_kmers) {
    Penalties p;
    double events_per_kmer = (double)n_events / n_kmers;
    double p_stay = 1 - (1 / (events_per_kmer + 1));
    p.lp_skip = log(1e-10);
    p.lp_stay = log(p_stay);
    p.lp_step = log(1.0 - exp(p.lp_skip) - exp(p.lp_stay));
    p.lp_trim = log(0.01);
    return p;
}

static void split(double v, float& h, float& l) {
    h = (float)v;
    l = (float)(v - (double)h);
}


static GlobalConsts global_consts(int var_aware) {
    GlobalConsts g;
    g.lp_skip = log(1e-10);
    g.lp_trim = log(0.01);
    split(g.lp_skip, g.skip_h, g.skip_l);
    g.trim_f = (float)g.lp_trim;
    g.var_aware = var_aware;
    return g;
}

struct HostInputs {
    int32_t n_reads;
    const char* read;
    const int64_t* read_ptr;
    const int32_t* read_len;
    const abea_event_t* event_table;
    const int64_t* event_ptr;
    const int32_t* n_events;
    const abea_scalings_t* scalings;
    const abea_model_t* model;
};

static abea_status_t validate(const HostInputs& in) {
    if (in.n_reads < 0) return fail(ABEA_ERR_INVALID_ARG, "n_reads < 0");
    if (in.n_reads == 0) return ABEA_OK;
    if (!in.read || !in.read_ptr || !in.read_len || !in.event_ptr || !in.n_events ||
        !in.scalings || !in.model)
        return fail(ABEA_ERR_INVALID_ARG, "null input array");
    for (int32_t i = 0; i < in.n_reads; ++i) {
        if (in.read_len[i] < 0 || in.n_events[i] < 0 || in.read_ptr[i] < 0 || in.event_ptr[i] < 0)
            return fail(ABEA_ERR_INVALID_ARG, "read %d: negative length or offset", i);
        if (in.n_events[i] > 0 && !in.event_table)
            return fail(ABEA_ERR_INVALID_ARG, "null event table");
        if ((int64_t)in.n_events[i] > (1ll << 30) || (int64_t)in.read_len[i] > (1ll << 30))
            return fail(ABEA_ERR_INVALID_ARG, "read %d too long", i);
    }
    return ABEA_OK;
}

// Offsets and per-read constants of a batch.
static abea_status_t plan(abea_batch* b, const HostInputs& in, int var_aware, int64_t trace_budget) {
    b->n_reads = in.n_reads;
    b->var_aware = var_aware;
    b->reads.assign((size_t)in.n_reads, ReadDesc{});
    int64_t seq_end = 0, ev_end = 0, km = 0, ev = 0, bands = 0, cells = 0, tbands = 0, ckf = 0;
    int32_t n_ck = 0;
    for (int32_t i = 0; i < in.n_reads; ++i) {
        ReadDesc& r = b->reads[(size_t)i];
        int32_t len = in.read_len[i], ne = in.n_events[i];
        int32_t nk = len - ABEA_KMER_SIZE + 1;
        r.seq_off = in.read_ptr[i];
        r.ev_src = in.event_ptr[i];
        r.out_off = 2 * in.event_ptr[i];
        r.n_events = ne;
        r.n_kmers = nk;
        r.out_cap = 2 * ne;
        r.scale = in.scalings[i].scale;
        r.shift = in.scalings[i].shift;
        r.var = in.scalings[i].var;
        r.log_var = in.scalings[i].log_var;
        seq_end = std::max(seq_end, in.read_ptr[i] + (int64_t)len);
        ev_end = std::max(ev_end, in.event_ptr[i] + (int64_t)ne);
        r.skip = (nk <= 0 || ne <= 0) ? 1 : 0;
        if (r.skip) {
            r.n_bands = 0;
            r.ev_off = ev;
            r.km_off = km;
            r.band_off = bands;
            r.trace_off = tbands;
            continue;
        }
        r.n_bands = ne + nk + 2;
        Penalties p = penalties(ne, nk);
        r.lp_step = p.lp_step;
        r.lp_stay = p.lp_stay;
        split(p.lp_step, r.step_h, r.step_l);
        split(p.lp_stay, r.stay_h, r.stay_l);
        r.ev_off = ev;
        r.km_off = km;
        r.band_off = bands;
        // a trace over the budget: checkpoints every kCkBands bands instead
        const int64_t trace_bytes = round_up(r.n_bands, 4) * (int64_t)kSlots;
        r.ck = (trace_budget > 0 && trace_bytes > trace_budget) ? 1 : 0;
        r.trace_off = tbands;
        if (r.ck) {
            r.ck_off = ckf;
            r.ck_slot = n_ck++;
            ckf += (int64_t)(r.n_bands / kCkBands + 1) * kCkStride;
        } else {
            tbands += round_up(r.n_bands, 4);
        }
        ev += round_up(ne, kChunk);
        km += round_up(nk, kChunk);
        bands += round_up(r.n_bands, 4);
        cells += (int64_t)r.n_bands * kBand;
    }
    b->seq_bytes = seq_end;
    b->n_events_total = ev_end;
    b->ev_pad_total = ev;
    b->km_pad_total = km;
    b->band_pad_total = bands;
    b->trace_pad_total = tbands;
    b->ck_floats = ckf;
    b->n_ck = n_ck;
    int32_t n_spec = 0;
    for (const ReadDesc& r : b->reads)
        if (!r.skip && !r.ck && r.n_bands >= kSpecMinBands) ++n_spec;
    // one scratch slot per block that starts on a wide read (a block walks one wide read
    // at a time and keeps its slot; the first picks take the longest reads, so at most
    // one slot per qualifying read)
    const int grid = b->ctx ? std::max(batched_blocks_per_sm(false), batched_blocks_per_sm(true)) * b->ctx->sm_count
                            : kSpecMaxSlots;
    b->n_spec = std::min(std::min(n_spec, std::max(grid, 1)), kSpecMaxSlots);
    b->pair_cap = 2 * ev_end;
    b->band_cells = cells;
    // longest first; ties by index
    b->order.resize((size_t)in.n_reads);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int32_t x, int32_t y) {
        return b->reads[(size_t)x].n_bands > b->reads[(size_t)y].n_bands;
    });
    return ABEA_OK;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Carves the device slab; grows it when needed.
static abea_status_t ensure_device(abea_batch* b, bool scores, size_t reserve = 0) {
    size_t n = (size_t)std::max(b->n_reads, 1);
    size_t sizes[33] = {
        sizeof(ReadDesc) * n,                                   // reads
        (size_t)std::max<int64_t>(b->seq_bytes, 1),             // seq
        sizeof(abea_event_t) * (size_t)std::max<int64_t>(b->n_events_total, 1),
        sizeof(abea_model_t) * ABEA_NUM_KMER,
        sizeof(float) * (size_t)std::max<int64_t>(b->ev_pad_total, 16),  // ev_mean
        sizeof(float) * (size_t)std::max<int64_t>(b->km_pad_total, 16),  // gm
        sizeof(float) * (size_t)std::max<int64_t>(b->km_pad_total, 16),  // sd
        sizeof(float) * (size_t)std::max<int64_t>(b->km_pad_total, 16),  // k1
        sizeof(float) * (size_t)std::max<int64_t>(b->ev_pad_total, 16),  // last_col
        sizeof(float) * (size_t)std::max<int64_t>(b->km_pad_total, 16),  // rsd
        (size_t)kSlots * (size_t)std::max<int64_t>(b->trace_pad_total, 4), // trace
        scores ? sizeof(float) * kSlots * (size_t)std::max<int64_t>(b->band_pad_total, 4) : 0,
        sizeof(int32_t) * (size_t)std::max<int64_t>(b->band_pad_total, 4),  // band_k0
        sizeof(abea_aligned_pair_t) * (size_t)std::max<int64_t>(b->pair_cap, 1),
        sizeof(int32_t) * n,   // n_pairs
        sizeof(float) * n,     // best
        sizeof(int32_t) * n,   // status
        sizeof(unsigned long long) * 4,  // slow counter
        sizeof(int32_t) * n,   // order
        sizeof(int32_t) * 8,   // queue counters
        sizeof(int32_t) * n,   // path_len
        sizeof(int32_t) * n,   // path_flags
        sizeof(int32_t) * n,   // best_event
        sizeof(int32_t) * n,   // adj_status
        sizeof(double) * 3 * n,  // grad_sc
        sizeof(double) * 5 * n,  // gn
        sizeof(double) * n,      // path_em
        sizeof(double) * 2 * ABEA_NUM_KMER,  // grad_model
        sizeof(float) * (size_t)std::max<int64_t>(b->ck_floats, 16),  // checkpoints
        (size_t)kCkBands * kSlots * (size_t)std::max<int32_t>(b->n_ck, 0),  // recompute scratch
        sizeof(int32_t) * kSpecRound * kSpecBands * (size_t)b->n_spec,      // traceback cell maps
        kAuxBytes,  // landed counter and output mirror
        0};
    const int n_bufs = 32;
    size_t total = 0;
    for (int i = 0; i < n_bufs; ++i) total += align256(sizes[i]);
    if (total > b->slab.bytes) {
        free_batch_device(b);
        void* p = nullptr;
        const size_t want = std::max(total, reserve);
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(ABEA_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes failed: %s", want,
                        cudaGetErrorString(e));
        }
        b->slab.base = p;
        b->slab.bytes = want;
    }
    char* p = (char*)b->slab.base;
    void* ptrs[33];
    for (int i = 0; i < n_bufs; ++i) {
        ptrs[i] = sizes[i] ? (void*)p : nullptr;
        p += align256(sizes[i]);
    }
    b->d_reads = (ReadDesc*)ptrs[0];
    b->d_seq = (char*)ptrs[1];
    b->d_ev = (abea_event_t*)ptrs[2];
    b->d_model = (abea_model_t*)ptrs[3];
    b->d_ev_mean = (float*)ptrs[4];
    b->d_km_gm = (float*)ptrs[5];
    b->d_km_sd = (float*)ptrs[6];
    b->d_km_k1 = (float*)ptrs[7];
    b->d_last_col = (float*)ptrs[8];
    b->d_km_rsd = (float*)ptrs[9];
    b->d_trace = (uint8_t*)ptrs[10];
    b->d_scores = (float*)ptrs[11];
    b->d_band_k0 = (int32_t*)ptrs[12];
    b->d_pairs = (abea_aligned_pair_t*)ptrs[13];
    b->d_n_pairs = (int32_t*)ptrs[14];
    b->d_best = (float*)ptrs[15];
    b->d_status = (int32_t*)ptrs[16];
    b->d_slow = (unsigned long long*)ptrs[17];
    b->d_order = (int32_t*)ptrs[18];
    b->d_queue = (int32_t*)ptrs[19];
    b->d_path_len = (int32_t*)ptrs[20];
    b->d_path_flags = (int32_t*)ptrs[21];
    b->d_best_event = (int32_t*)ptrs[22];
    b->d_adj_status = (int32_t*)ptrs[23];
    b->d_grad_sc = (double*)ptrs[24];
    b->d_gn = (double*)ptrs[25];
    b->d_path_em = (double*)ptrs[26];
    b->d_grad_model = (double*)ptrs[27];
    b->d_ck = (float*)ptrs[28];
    b->d_ck_scratch = (uint8_t*)ptrs[29];
    b->d_spec = (int32_t*)ptrs[30];
    b->d_aux = (char*)ptrs[31];
    b->scores_kept = scores;
    b->carve.assign(1, (uint64_t)(uintptr_t)b->slab.base);
    for (int i = 0; i < n_bufs; ++i) b->carve.push_back((uint64_t)sizes[i]);
    return ABEA_OK;
}

// Copies a batch to the device.  bases_events = false leaves out the bases and
// the events (the pre stage then reads them from the caller's pinned memory);
// reads_pinned, when given, is a pinned copy of the read descriptors to copy from.
static abea_status_t upload(abea_batch* b, const HostInputs& in, cudaStream_t st, bool bases_events = true,
                            const ReadDesc* reads_pinned = nullptr) {
    if (b->n_reads == 0) return ABEA_OK;
    CUDA_TRY(cudaMemsetAsync(b->d_aux, 0, kAuxBytes, st));  // no input or output mirror
    CUDA_TRY(cudaMemcpyAsync(b->d_reads, reads_pinned ? reads_pinned : b->reads.data(),
                             sizeof(ReadDesc) * b->reads.size(), cudaMemcpyHostToDevice, st));
    if (bases_events && b->seq_bytes > 0)
        CUDA_TRY(cudaMemcpyAsync(b->d_seq, in.read, (size_t)b->seq_bytes, cudaMemcpyHostToDevice, st));
    if (bases_events && b->n_events_total > 0)
        CUDA_TRY(cudaMemcpyAsync(b->d_ev, in.event_table, sizeof(abea_event_t) * (size_t)b->n_events_total,
                                 cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(b->d_model, in.model, sizeof(abea_model_t) * ABEA_NUM_KMER,
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(b->d_order, b->order.data(), sizeof(int32_t) * b->order.size(),
                             cudaMemcpyHostToDevice, st));
    b->dev_order_sent = b->order;
    return ABEA_OK;
}

static int64_t h2d_bytes(const abea_batch* b) {
    return (int64_t)(sizeof(ReadDesc) * b->reads.size()) + b->seq_bytes +
           (int64_t)sizeof(abea_event_t) * b->n_events_total + (int64_t)sizeof(abea_model_t) * ABEA_NUM_KMER +
           (int64_t)sizeof(int32_t) * (int64_t)b->order.size();
}

static int64_t d2h_bytes(const abea_batch* b) {
    return (int64_t)sizeof(abea_aligned_pair_t) * b->pair_cap + (int64_t)sizeof(int32_t) * b->n_reads;
}

// Heuristic wide-shape threshold.  First, the number n of wide reads (the longest
// ones whose trace is kept, at most one per block, the other blocks taking the
// warp-shape reads from the start) that minimises an estimate of the batch's
// makespan, in cycles:
//   the longest wide read on the wide shape, kWideCyc per band;
//   the longest warp-shape read: kWarpFloorCyc per band, or kWarpSmCyc per band
//     times the warps sharing its SM in the first wave (the blocks without a
//     wide read share the other reads round-robin, at most 16 warps each);
//   the warp-shape work spread over those blocks, kWarpSmCyc per band per SM.
// Then every read on the wide shape, the blocks pulling them longest first: the
// longest read at kWideCyc per band, or all the bands over the blocks at
// kWideSmCyc per band per block.  That wins when it is within 2% of the first
// (it cannot be shorter than the longest read, which bounds both) and either the
// longest read bounds it or there are at most 8 reads per block (with more, the
// warp shape's 16 warps per SM hide each other's latency better than the first
// estimate assumes: the serving stream's batches of ~4,000 reads of median 8 kb
// took 1.23 s every read wide against 0.99 s split), except with checkpointed
// reads, which run on the warp shape and would start last.
// Calibrated on GB300 by sweeping the number of wide reads: the f5c batch and the
// 1,024-read batch of 1-10 kb reads are fastest with every read wide (8.46 and
// 18.5 ms, against 8.49-9.10 and 20.8 at the best one-per-block split); the
// 4,096-read adjoint batch with none (35.5 ms; 68.5 with every read wide: at 27
// reads per SM the warp shape's 16 warps issue more per SM).  kWarpFloorCyc
// includes the warp-shape read's traceback, kWideSmCyc the wide reads' tracebacks
// and the blocks' tail.  Ties go to fewer wide reads; the threshold is the band
// count of the n-th wide read (every read: 1; none: INT64_MAX).
constexpr double kWideCyc = 400, kWarpFloorCyc = 1800, kWarpSmCyc = 250, kWideSmCyc = 380;
static int64_t heuristic_threshold(const abea_batch* b, int blocks) {
    const size_t n = b->order.size();
    std::vector<int64_t> wide_ok;  // band counts of the reads that may be wide, longest first
    double rest_bands = 0;
    for (int32_t i : b->order) {
        const ReadDesc& r = b->reads[(size_t)i];
        rest_bands += (double)r.n_bands;
        if (!r.ck) wide_ok.push_back(r.n_bands);
    }
    const double all_bands = rest_bands;
    const bool any_ck = wide_ok.size() < n;
    const int max_wide = (int)std::min<size_t>(wide_ok.size(), (size_t)std::max(0, blocks - 1));
    double best_t = 0;
    int best_n = 0;
    int taken = 0;
    for (int k = 0; k <= max_wide; ++k) {
        if (k > 0) {  // the k-th wide read leaves the warp-shape set
            rest_bands -= (double)wide_ok[(size_t)k - 1];
            ++taken;
        }
        // the longest warp-shape read: skip the wide ones (the longest trace-keeping reads)
        int skip = taken;
        size_t j = 0;
        int64_t longest_warp = 0;
        for (j = 0; j < n; ++j) {
            const ReadDesc& r = b->reads[(size_t)b->order[j]];
            if (!r.ck && skip > 0) {
                --skip;
                continue;
            }
            longest_warp = r.n_bands;
            break;
        }
        const int free_blocks = std::max(1, blocks - k);
        const double warps = std::min(16.0, std::max(1.0, (double)(n - (size_t)k) / free_blocks));
        const double t_wide = k > 0 ? (double)wide_ok[0] * kWideCyc : 0.0;
        const double t_warp = (double)longest_warp * std::max(kWarpFloorCyc, kWarpSmCyc * warps);
        const double t_work = rest_bands * kWarpSmCyc / free_blocks;
        const double t = std::max(t_wide, std::max(t_warp, t_work));
        if (k == 0 || t < best_t * 0.98) {  // a wide read must buy at least 2%
            best_t = t;
            best_n = k;
        }
    }
    if (!any_ck && !wide_ok.empty()) {
        const double t_lat = (double)wide_ok[0] * kWideCyc, t_thr = all_bands * kWideSmCyc / std::max(blocks, 1);
        // at more than 8 reads per block the warp shape's warps hide each other's
        // latency and the split's estimate above is too long: every read wide only
        // where the longest read bounds it anyway, or with few reads per block
        const bool few = (double)n <= 8.0 * blocks;
        if ((t_thr <= t_lat || few) && std::max(t_lat, t_thr) <= best_t * 1.02) return 1;
    }
    return best_n > 0 ? wide_ok[(size_t)best_n - 1] : INT64_MAX;
}

// Reads of the batched form that run on the wide and the medium shapes: the
// longest reads over the wide threshold (the option, the autotuned value, or the
// heuristic above; the blocks take them longest first, one at a time, as many
// each as the queue holds; with the cluster pair at most one per cluster), then
// the longest remaining reads over the medium threshold (none without one; never
// with the cluster pair); never a checkpointed read.  Fills b->dev_order with the wide reads, the
// medium reads, then the rest, each longest first, and sets n_wide and n_mid.
static void choose_shape_reads(abea_batch* b, int sm_count, int64_t threshold, int64_t mid_threshold, bool scores,
                               bool cluster) {
    const int blocks = cluster ? sm_count / 2 : batched_blocks_per_sm(scores) * sm_count;
    if (threshold <= 0) threshold = heuristic_threshold(b, blocks);
    if (mid_threshold <= 0 || cluster) mid_threshold = INT64_MAX;
    std::vector<int32_t> wide, mid, rest;
    for (int32_t i : b->order) {
        const ReadDesc& r = b->reads[(size_t)i];
        if ((!cluster || (int)wide.size() < blocks) && !r.ck && r.n_bands >= threshold)
            wide.push_back(i);
        else if (!r.ck && r.n_bands >= mid_threshold)
            mid.push_back(i);
        else
            rest.push_back(i);
    }
    b->dev_order = wide;
    b->dev_order.insert(b->dev_order.end(), mid.begin(), mid.end());
    b->dev_order.insert(b->dev_order.end(), rest.begin(), rest.end());
    b->n_wide = (int32_t)wide.size();
    b->n_mid = (int32_t)mid.size();
}

// Queues pre, core and post for a batch on the context's stream.
static abea_status_t launch_all(abea_ctx* c, abea_batch* b, int* launches, bool capturing) {
    LaunchArgs la;
    const GlobalConsts g = global_consts(b->var_aware);
    la.pre = PreArgs{b->d_reads, b->n_reads, g, b->d_seq, b->d_ev, b->d_model, b->d_ev_mean, b->d_km_gm,
                     b->d_km_sd, b->d_km_rsd, b->d_km_k1, b->d_last_col, (const InMirror*)b->d_aux};
    la.core = CoreArgs{b->d_reads, b->n_reads, g, b->d_ev_mean, b->d_km_gm, b->d_km_sd, b->d_km_rsd, b->d_km_k1,
                       b->d_last_col, b->d_trace, b->scores_kept ? b->d_scores : nullptr, b->d_band_k0,
                       b->d_slow, b->d_order, b->d_queue, b->n_wide, b->d_ck, b->d_ck_scratch, b->d_spec,
                       b->n_spec,
                       (long long)c->spin_limit, b->n_mid};
    la.post = PostArgs{b->d_reads, b->n_reads, g, b->d_ev_mean, b->d_km_gm, b->d_km_sd, b->d_km_k1, b->d_km_rsd,
                       b->d_last_col, b->d_trace, b->d_band_k0, b->d_pairs, b->d_n_pairs, b->d_best,
                       b->d_status, b->d_path_len, b->d_path_flags, b->d_best_event,
                       (const OutMirror*)(b->d_aux + kAuxMirror)};
    la.sm_count = c->sm_count;
    la.stream = c->stream;
    la.ev_pre = c->ev[1];
    la.ev_core = c->ev[2];
    la.capturing = capturing;
    la.cluster = c->wide_cluster != 0;
    cudaError_t e = c->mode == ABEA_MODE_BATCHED ? launch_batched(la, launches) : launch_plain(la, launches);
    if (e != cudaSuccess) return fail(ABEA_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    return ABEA_OK;
}

static abea_status_t collect_timing(abea_ctx* c, abea_batch* b);

// Workload signature for the autotuner: log2 buckets of the longest read's bands,
// of the read count and of the total bands.
static uint64_t workload_signature(const abea_batch* b) {
    int64_t mx = 0, tot = 0;
    for (const ReadDesc& r : b->reads) {
        mx = std::max<int64_t>(mx, r.n_bands);
        tot += r.n_bands;
    }
    auto lg = [](int64_t v) { int k = 0; while (v > 1) { v >>= 1; ++k; } return (uint64_t)k; };
    return (lg(mx) << 16) | (lg(b->n_reads) << 8) | lg(tot);
}

static abea_status_t queue_work(abea_ctx* c, abea_batch* b, int* launches, bool capturing) {
    CUDA_TRY(cudaMemsetAsync(b->d_slow, 0, sizeof(unsigned long long) * 4, c->stream));
    CUDA_TRY(cudaMemsetAsync(b->d_queue, 0, sizeof(int32_t) * 8, c->stream));
    return launch_all(c, b, launches, capturing);
}

// The batched form's order: wide reads (threshold from the option, else the
// autotuned value of this workload signature, else the heuristic), medium reads
// (threshold from the option, else the autotuned value, else none), then the rest.
static void prepare_order(abea_ctx* c, abea_batch* b) {
    b->n_wide = 0;
    b->n_mid = 0;
    if (c->mode != ABEA_MODE_BATCHED) return;
    const uint64_t sig = workload_signature(b);
    int64_t thr = c->long_read_bands, mid = c->mid_read_bands;
    if (thr == 0) {
        auto it = c->tuned.find(sig);
        if (it != c->tuned.end()) thr = it->second;
    }
    if (mid == 0) {
        auto it = c->tuned_mid.find(sig);
        if (it != c->tuned_mid.end()) mid = it->second;
    }
    choose_shape_reads(b, c->sm_count, thr, mid, b->scores_kept, c->wide_cluster != 0);
}

static abea_status_t run_batch(abea_ctx* c, abea_batch* b) {
    NvtxRange nv("abea run");
    CUDA_TRY(cudaSetDevice(c->device));
    b->timing = abea_timing_t{};
    if (b->n_reads == 0) {
        b->ran = true;
        return ABEA_OK;
    }
    // wide shape for the longest reads in the batched form
    prepare_order(c, b);
    if (c->mode == ABEA_MODE_BATCHED) {
        if (b->dev_order != b->dev_order_sent) {
            CUDA_TRY(cudaMemcpyAsync(b->d_order, b->dev_order.data(), sizeof(int32_t) * b->dev_order.size(),
                                     cudaMemcpyHostToDevice, c->stream));
            CUDA_TRY(cudaStreamSynchronize(c->stream));  // the host vector may change before the copy runs
            b->dev_order_sent = b->dev_order;
        }
    }
    int launches = 0;
    if (c->mode == ABEA_MODE_BATCHED && c->use_graph) {
        // the whole run as one CUDA graph, re-captured when its parameters change
        // the kernels' arguments (device pointers, counts, constants) follow from
        // the slab layout and these; any change re-captures
        std::vector<uint64_t> key = b->carve;
        key.push_back((uint64_t)b->n_reads);
        key.push_back((uint64_t)b->n_wide);
        key.push_back((uint64_t)b->n_mid);
        key.push_back((uint64_t)(b->scores_kept ? 1 : 0) | ((uint64_t)b->var_aware << 1) |
                      ((uint64_t)(c->wide_cluster != 0) << 2));
        if (!b->graph || key != b->graph_key) {
            if (b->graph) cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            abea_status_t st = queue_work(c, b, &launches, true);
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (st) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (e != cudaSuccess) return fail(ABEA_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                b->graph = nullptr;
                return fail(ABEA_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
            }
            b->graph_key = key;
            b->graph_launches = launches;
        }
        launches = b->graph_launches;
        CUDA_TRY(cudaEventRecord(c->ev[0], c->stream));
        CUDA_TRY(cudaGraphLaunch(b->graph, c->stream));
        CUDA_TRY(cudaEventRecord(c->ev[3], c->stream));
    } else {
        CUDA_TRY(cudaEventRecord(c->ev[0], c->stream));
        abea_status_t st = queue_work(c, b, &launches, false);
        if (st) return st;
        CUDA_TRY(cudaEventRecord(c->ev[3], c->stream));
    }
    b->timing.kernel_launches = launches;
    b->ran = true;
    return ABEA_OK;
}

// Autotuner: times the batched form on `b` with candidate thresholds for the
// wide shape — none, the heuristic, the band counts of the reads ranked at 1, 2,
// 3, 4, 6, 8, 12 and 16 sixteenths of the resident blocks and at 3/2, 2, 3, 4 and
// 6 times their number (every read when the batch has fewer), and 15, 20, 45 and
// 60% of the longest read — keeps the fastest for
// this workload signature (longest read, read count and total bands, log2
// buckets) and returns it.
extern "C" abea_status_t abea_autotune(abea_ctx_t* c, abea_batch_t* b, int64_t* best_threshold, float* best_ms) {
    NvtxRange nv("abea autotune");
    if (!c || !b) return fail(ABEA_ERR_INVALID_ARG, "abea_autotune: null argument");
    if (b->n_reads == 0) return ABEA_OK;
    const abea_mode_t mode0 = c->mode;
    const int64_t thr0 = c->long_read_bands, mid0 = c->mid_read_bands;
    c->mode = ABEA_MODE_BATCHED;
    // the wide stage runs without medium reads: neither the option nor a medium
    // threshold tuned earlier for this signature may shape its timings
    c->mid_read_bands = INT64_MAX;
    const int blocks = batched_blocks_per_sm(b->scores_kept) * c->sm_count;
    int64_t longest = 0;
    for (const ReadDesc& r : b->reads) longest = std::max<int64_t>(longest, r.n_bands);
    std::vector<int64_t> cands = {INT64_MAX, heuristic_threshold(b, blocks)};
    if (c->wide_cluster == 0 && std::find(cands.begin(), cands.end(), (int64_t)1) == cands.end())
        cands.push_back(1);  // every read wide
    for (int num : {1, 2, 3, 4, 6, 8, 12, 16}) {  // the longest num/16 of the resident blocks
        size_t k = std::min<size_t>(b->order.size(), (size_t)std::max(1, blocks * num / 16)) - 1;
        const int64_t c = std::max<int64_t>(1, b->reads[(size_t)b->order[k]].n_bands);
        if (std::find(cands.begin(), cands.end(), c) == cands.end()) cands.push_back(c);
    }
    for (int pct : {15, 20, 45, 60}) {  // fractions of the longest read
        const int64_t c = std::max<int64_t>(1, longest * pct / 100);
        if (std::find(cands.begin(), cands.end(), c) == cands.end()) cands.push_back(c);
    }
    if (c->wide_cluster == 0)
        for (int mul : {3, 4, 6, 8, 12}) {  // more wide reads than blocks: 3/2 .. 6 per block, then every read
            const size_t k = std::min<size_t>(b->order.size(), (size_t)blocks * mul / 2);
            const int64_t v = k < b->order.size() ? std::max<int64_t>(1, b->reads[(size_t)b->order[k - 1]].n_bands) : 1;
            if (std::find(cands.begin(), cands.end(), v) == cands.end()) cands.push_back(v);
        }
    int64_t best = 0;
    float best_t = 1e30f;
    abea_status_t st = ABEA_OK;
    for (int64_t cand : cands) {
        c->long_read_bands = cand;
        float t_min = 1e30f;
        for (int rep = 0; rep < 3 && !st; ++rep) {
            if ((st = run_batch(c, b))) break;
            if ((st = collect_timing(c, b))) break;
            if (rep > 0) t_min = std::min(t_min, b->timing.total_ms);
        }
        if (st) break;
        if (t_min < best_t) {
            best_t = t_min;
            best = cand;
        }
    }
    // then the medium shape with that wide threshold: none, or the band count of
    // the reads that leave k of the remaining reads for it (k from a quarter of the
    // block halves to four per half) or at fractions of the longest remaining read
    int64_t best_mid = INT64_MAX;
    if (!st && c->wide_cluster == 0) {
        c->long_read_bands = best;
        std::vector<int64_t> rest;  // band counts of the reads left after the wide ones, longest first
        int n_wide_best = 0;
        for (int32_t i : b->order) {
            const ReadDesc& r = b->reads[(size_t)i];
            if (n_wide_best < blocks && !r.ck && r.n_bands >= best) {
                ++n_wide_best;
                continue;
            }
            if (!r.ck) rest.push_back(r.n_bands);
        }
        std::vector<int64_t> mids;
        for (int num : {1, 2, 4, 8, 16}) {  // num/2 medium reads per block half
            const size_t k = (size_t)std::max(1, blocks * 2 * num / 4);
            if (k <= rest.size()) {
                const int64_t v = std::max<int64_t>(1, rest[k - 1]);
                if (std::find(mids.begin(), mids.end(), v) == mids.end()) mids.push_back(v);
            }
        }
        if (!rest.empty())
            for (int pct : {25, 50, 75}) {
                const int64_t v = std::max<int64_t>(1, rest[0] * pct / 100);
                if (std::find(mids.begin(), mids.end(), v) == mids.end()) mids.push_back(v);
            }
        for (int64_t cand : mids) {
            c->mid_read_bands = cand;
            float t_min = 1e30f;
            for (int rep = 0; rep < 3 && !st; ++rep) {
                if ((st = run_batch(c, b))) break;
                if ((st = collect_timing(c, b))) break;
                if (rep > 0) t_min = std::min(t_min, b->timing.total_ms);
            }
            if (st) break;
            if (t_min < best_t * 0.98f) {  // the medium shape must buy 2%
                best_t = t_min;
                best_mid = cand;
            }
        }
    }
    c->mode = mode0;
    c->long_read_bands = thr0;
    c->mid_read_bands = mid0;
    if (st) return st;
    c->tuned[workload_signature(b)] = best;
    c->tuned_mid[workload_signature(b)] = best_mid;
    if (best_threshold) *best_threshold = best;
    if (best_ms) *best_ms = best_t;
    return ABEA_OK;
}

// Autotuner cache: "abea-autotune 2 sm_count <n>" then "<signature> <wide threshold>
// <medium threshold>" lines (INT64_MAX = none).  Version 1 files (no medium
// threshold) are read too.
extern "C" abea_status_t abea_autotune_save(abea_ctx_t* c, const char* path, int32_t* n_entries) {
    if (!c || !path) return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_save: null argument");
    FILE* f = fopen(path, "w");
    if (!f) return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_save: cannot open %s", path);
    fprintf(f, "abea-autotune 2 sm_count %d\n", c->sm_count);
    for (const auto& kv : c->tuned) {
        auto m = c->tuned_mid.find(kv.first);
        fprintf(f, "%llu %lld %lld\n", (unsigned long long)kv.first, (long long)kv.second,
                (long long)(m == c->tuned_mid.end() ? INT64_MAX : m->second));
    }
    const bool ok = fclose(f) == 0;
    if (!ok) return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_save: write to %s failed", path);
    if (n_entries) *n_entries = (int32_t)c->tuned.size();
    return ABEA_OK;
}

extern "C" abea_status_t abea_autotune_load(abea_ctx_t* c, const char* path, int32_t* n_entries) {
    if (!c || !path) return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_load: null argument");
    FILE* f = fopen(path, "r");
    if (!f) return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_load: cannot open %s", path);
    int version = 0, sm = 0;
    if (fscanf(f, "abea-autotune %d sm_count %d", &version, &sm) != 2 || (version != 1 && version != 2)) {
        fclose(f);
        return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_load: %s is not an autotuner cache", path);
    }
    if (sm != c->sm_count) {
        fclose(f);
        return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_load: %s was tuned on %d SMs, this device has %d", path,
                    sm, c->sm_count);
    }
    std::map<uint64_t, std::pair<int64_t, int64_t>> got;
    unsigned long long sig = 0;
    long long thr = 0, mid = INT64_MAX;
    const int fields = version == 1 ? 2 : 3;
    int r;
    while ((r = version == 1 ? fscanf(f, "%llu %lld", &sig, &thr) : fscanf(f, "%llu %lld %lld", &sig, &thr, &mid)) ==
           fields) {
        if (thr < 1 || mid < 1) {
            fclose(f);
            return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_load: bad threshold in %s", path);
        }
        got[(uint64_t)sig] = {(int64_t)thr, (int64_t)mid};
    }
    const bool at_end = r == EOF;
    fclose(f);
    if (!at_end) return fail(ABEA_ERR_INVALID_ARG, "abea_autotune_load: malformed line in %s", path);
    for (const auto& kv : got) {
        c->tuned[kv.first] = kv.second.first;
        c->tuned_mid[kv.first] = kv.second.second;
    }
    if (n_entries) *n_entries = (int32_t)got.size();
    return ABEA_OK;
}

static abea_status_t collect_timing(abea_ctx* c, abea_batch* b) {
    if (b->n_reads == 0) return ABEA_OK;
    CUDA_TRY(cudaEventSynchronize(c->ev[3]));
    float t = 0;
    CUDA_TRY(cudaEventElapsedTime(&t, c->ev[0], c->ev[1]));
    b->timing.pre_ms = t;
    CUDA_TRY(cudaEventElapsedTime(&t, c->ev[1], c->ev[2]));
    b->timing.core_ms = t;
    CUDA_TRY(cudaEventElapsedTime(&t, c->ev[2], c->ev[3]));
    b->timing.post_ms = t;
    CUDA_TRY(cudaEventElapsedTime(&t, c->ev[0], c->ev[3]));
    b->timing.total_ms = t;
    return ABEA_OK;
}

static abea_status_t download(abea_ctx* c, abea_batch* b, abea_aligned_pair_t* pairs, int32_t* n_pairs) {
    if (b->n_reads == 0) return ABEA_OK;
    if (pairs && b->pair_cap > 0)
        CUDA_TRY(cudaMemcpyAsync(pairs, b->d_pairs, sizeof(abea_aligned_pair_t) * (size_t)b->pair_cap,
                                 cudaMemcpyDeviceToHost, c->stream));
    if (n_pairs)
        CUDA_TRY(cudaMemcpyAsync(n_pairs, b->d_n_pairs, sizeof(int32_t) * (size_t)b->n_reads,
                                 cudaMemcpyDeviceToHost, c->stream));
    return ABEA_OK;
}

// The batch's device-side counters and per-read statuses as a status: from
// `host` (counters, then statuses, already copied by the caller after a
// synchronize) or copied here.
static abea_status_t check_status(abea_ctx* c, abea_batch* b, const void* host = nullptr) {
    if (b->n_reads == 0) return ABEA_OK;
    std::vector<char> buf;
    if (!host) {
        buf.resize(sizeof(unsigned long long) * 4 + sizeof(int32_t) * (size_t)b->n_reads);
        CUDA_TRY(cudaMemcpyAsync(buf.data(), b->d_slow, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost,
                                 c->stream));
        CUDA_TRY(cudaMemcpyAsync(buf.data() + sizeof(unsigned long long) * 4, b->d_status,
                                 sizeof(int32_t) * (size_t)b->n_reads, cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        host = buf.data();
    }
    unsigned long long cnt[4];
    memcpy(cnt, host, sizeof(cnt));
    if (cnt[2]) return fail(ABEA_ERR_TIMEOUT, "%llu device-side waits ran out of polls (ABEA_OPT_SPIN_LIMIT)", cnt[2]);
    if (cnt[3]) return fail(ABEA_ERR_INTERNAL, "%llu device-side stores out of their region (bounds-checked build)", cnt[3]);
    const int32_t* st = (const int32_t*)((const char*)host + sizeof(cnt));
    for (int32_t i = 0; i < b->n_reads; ++i)
        if (st[i] != 0) return fail((abea_status_t)st[i], "read %d: %s", i, abea_status_string((abea_status_t)st[i]));
    return ABEA_OK;
}

// ---------------------------------------------------------------- batch API
static HostInputs inputs(int32_t n, const char* read, const int64_t* read_ptr, const int32_t* read_len,
                         const abea_event_t* ev, const int64_t* event_ptr, const int32_t* n_events,
                         const abea_scalings_t* sc, const abea_model_t* model) {
    HostInputs in{n, read, read_ptr, read_len, ev, event_ptr, n_events, sc, model};
    return in;
}

extern "C" abea_status_t abea_batch_create(abea_ctx_t* c, int32_t n_reads, const char* read,
                                           const int64_t* read_ptr, const int32_t* read_len,
                                           const abea_event_t* event_table, const int64_t* event_ptr,
                                           const int32_t* n_events, const abea_scalings_t* scalings,
                                           const abea_model_t* model, abea_batch_t** out) {
    if (!c || !out) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_create: null argument");
    *out = nullptr;
    HostInputs in = inputs(n_reads, read, read_ptr, read_len, event_table, event_ptr, n_events, scalings, model);
    abea_status_t st = validate(in);
    if (st) return st;
    CUDA_TRY(cudaSetDevice(c->device));
    abea_batch* b = new (std::nothrow) abea_batch();
    if (!b) return fail(ABEA_ERR_OUT_OF_MEMORY, "host allocation failed");
    b->ctx = c;
    if ((st = plan(b, in, (int)c->var_aware, c->trace_budget)) || (st = ensure_device(b, c->store_scores != 0)) || (st = upload(b, in, c->stream))) {
        abea_batch_destroy(b);
        return st;
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        abea_batch_destroy(b);
        return fail(ABEA_ERR_CUDA, "upload failed: %s", cudaGetErrorString(e));
    }
    *out = b;
    return ABEA_OK;
}

extern "C" abea_status_t abea_batch_run(abea_ctx_t* c, abea_batch_t* b) {
    if (!c || !b) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_run: null argument");
    if (b->ctx != c) return fail(ABEA_ERR_INVALID_ARG, "batch belongs to another context");
    return run_batch(c, b);
}

extern "C" abea_status_t abea_batch_sync(abea_ctx_t* c) {
    if (!c) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_sync: null context");
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return ABEA_OK;
}

extern "C" abea_status_t abea_batch_results(abea_ctx_t* c, abea_batch_t* b, abea_aligned_pair_t* pairs,
                                            int32_t* n_pairs) {
    if (!c || !b) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_results: null argument");
    if (!b->ran) return fail(ABEA_ERR_INVALID_ARG, "batch has not been run");
    abea_status_t st = download(c, b, pairs, n_pairs);
    if (st) return st;
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return check_status(c, b);
}

extern "C" abea_status_t abea_batch_timing(abea_ctx_t* c, abea_batch_t* b, abea_timing_t* t) {
    if (!c || !b || !t) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_timing: null argument");
    abea_status_t st = collect_timing(c, b);
    if (st) return st;
    *t = b->timing;
    return ABEA_OK;
}

extern "C" abea_status_t abea_batch_best_scores(abea_ctx_t* c, abea_batch_t* b, float* best) {
    if (!c || !b || !best) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_best_scores: null argument");
    if (b->n_reads == 0) return ABEA_OK;
    CUDA_TRY(cudaMemcpyAsync(best, b->d_best, sizeof(float) * (size_t)b->n_reads, cudaMemcpyDeviceToHost,
                             c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return ABEA_OK;
}

extern "C" abea_status_t abea_batch_slow_cells(abea_ctx_t* c, abea_batch_t* b, int64_t* count) {
    if (!c || !b || !count) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_slow_cells: null argument");
    unsigned long long v = 0;
    if (b->n_reads) {
        CUDA_TRY(cudaMemcpyAsync(&v, b->d_slow, sizeof(v), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    *count = (int64_t)v;
    return ABEA_OK;
}

extern "C" abea_status_t abea_batch_read_bands(abea_ctx_t* c, abea_batch_t* b, int32_t ri, float* bands,
                                               uint8_t* trace, abea_event_kmer_pair_t* bll) {
    if (!c || !b) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_read_bands: null argument");
    if (ri < 0 || ri >= b->n_reads) return fail(ABEA_ERR_INVALID_ARG, "read index out of range");
    if (bands && !b->scores_kept)
        return fail(ABEA_ERR_INVALID_ARG, "scores were not kept (ABEA_OPT_STORE_SCORES)");
    const ReadDesc& r = b->reads[(size_t)ri];
    if (r.skip) return ABEA_OK;
    if (r.ck && trace) return fail(ABEA_ERR_INVALID_ARG, "read %d keeps checkpoints, not its trace (ABEA_OPT_TRACE_BUDGET)", ri);
    int64_t nb = r.n_bands, nbp = round_up(nb, 4);
    std::vector<uint8_t> tr((size_t)(nbp * kSlots));
    std::vector<int32_t> k0((size_t)nbp);
    std::vector<float> sc;
    if (!r.ck)
        CUDA_TRY(cudaMemcpyAsync(tr.data(), b->d_trace + r.trace_off * kSlots, tr.size(), cudaMemcpyDeviceToHost,
                                 c->stream));
    CUDA_TRY(cudaMemcpyAsync(k0.data(), b->d_band_k0 + r.band_off, sizeof(int32_t) * k0.size(),
                             cudaMemcpyDeviceToHost, c->stream));
    if (bands) {
        sc.resize((size_t)(nbp * kSlots));
        CUDA_TRY(cudaMemcpyAsync(sc.data(), b->d_scores + r.band_off * kSlots, sizeof(float) * sc.size(),
                                 cudaMemcpyDeviceToHost, c->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    // slot layout -> reference layout: offset o of band b is k-mer k0+o, slot (k0+o)&127
    for (int64_t bi = 0; bi < nb; ++bi) {
        int32_t kk = k0[(size_t)bi];
        if (bll) {
            bll[bi].kmer_idx = kk;
            bll[bi].event_idx = (int32_t)(bi - 2 - kk);
        }
        for (int o = 0; o < kBand; ++o) {
            int slot = (kk + o) & 127;
            if (trace) trace[bi * kBand + o] = tr[(size_t)trace_index(bi, slot)];
            if (bands) bands[bi * kBand + o] = sc[(size_t)(bi * kSlots + slot)];
        }
    }
    return ABEA_OK;
}

// ---------------------------------------------------------------- adjoint
// Queues the backward kernel over the stored paths of the last run.
static abea_status_t queue_backward(abea_ctx* c, abea_batch* b, bool model_grad) {
    if (model_grad)
        CUDA_TRY(cudaMemsetAsync(b->d_grad_model, 0, sizeof(double) * 2 * ABEA_NUM_KMER, c->stream));
    AdjArgs a{b->d_reads, b->n_reads, b->var_aware, b->d_seq, b->d_model, b->d_ev_mean, b->d_pairs,
              b->d_path_len, b->d_path_flags, b->d_grad_sc, b->d_gn, b->d_path_em,
              model_grad ? b->d_grad_model : nullptr, b->d_adj_status};
    cudaError_t e = launch_adjoint(a, c->stream);
    if (e != cudaSuccess) return fail(ABEA_ERR_CUDA, "adjoint launch failed: %s", cudaGetErrorString(e));
    return ABEA_OK;
}

extern "C" abea_status_t abea_batch_backward(abea_ctx_t* c, abea_batch_t* b, double* grad_scalings,
                                             double* grad_model, double* path_emission, int32_t* read_status) {
    NvtxRange nv("abea backward");
    if (!c || !b) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_backward: null argument");
    if (b->ctx != c) return fail(ABEA_ERR_INVALID_ARG, "batch belongs to another context");
    if (!b->ran) return fail(ABEA_ERR_INVALID_ARG, "batch has not been run");
    CUDA_TRY(cudaSetDevice(c->device));
    if (b->n_reads == 0) {
        if (grad_model) memset(grad_model, 0, sizeof(double) * 2 * ABEA_NUM_KMER);
        return ABEA_OK;
    }
    abea_status_t st = queue_backward(c, b, grad_model != nullptr);
    if (st) return st;
    const size_t n = (size_t)b->n_reads;
    if (grad_scalings)
        CUDA_TRY(cudaMemcpyAsync(grad_scalings, b->d_grad_sc, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost,
                                 c->stream));
    if (grad_model)
        CUDA_TRY(cudaMemcpyAsync(grad_model, b->d_grad_model, sizeof(double) * 2 * ABEA_NUM_KMER,
                                 cudaMemcpyDeviceToHost, c->stream));
    if (path_emission)
        CUDA_TRY(cudaMemcpyAsync(path_emission, b->d_path_em, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                 c->stream));
    if (read_status)
        CUDA_TRY(cudaMemcpyAsync(read_status, b->d_adj_status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                 c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return ABEA_OK;
}

extern "C" abea_status_t abea_backward_batch(abea_ctx_t* c, abea_batch_t* b, double* grad_scalings,
                                             double* grad_model, double* path_emission, int32_t* read_status) {
    return abea_batch_backward(c, b, grad_scalings, grad_model, path_emission, read_status);
}

// Host copy of the per-read scalings -> descriptors (and their shortcut flag).
static void apply_scalings(abea_batch* b, const abea_scalings_t* sc) {
    for (int32_t i = 0; i < b->n_reads; ++i) {
        ReadDesc& r = b->reads[(size_t)i];
        r.scale = sc[i].scale;
        r.shift = sc[i].shift;
        r.var = sc[i].var;
        r.log_var = sc[i].log_var;
    }
}

static abea_status_t upload_reads(abea_ctx* c, abea_batch* b) {
    if (b->n_reads == 0) return ABEA_OK;
    CUDA_TRY(cudaMemcpyAsync(b->d_reads, b->reads.data(), sizeof(ReadDesc) * b->reads.size(),
                             cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));  // the host descriptors may change next
    return ABEA_OK;
}

extern "C" abea_status_t abea_batch_set_scalings(abea_ctx_t* c, abea_batch_t* b, const abea_scalings_t* sc) {
    if (!c || !b || (!sc && b->n_reads > 0)) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_set_scalings: null argument");
    if (b->ctx != c) return fail(ABEA_ERR_INVALID_ARG, "batch belongs to another context");
    CUDA_TRY(cudaSetDevice(c->device));
    apply_scalings(b, sc);
    return upload_reads(c, b);
}

// One Gauss-Newton step of every read's (shift, scale) from the fixed-path
// normal equations gn[5*i] = {h00, h01, h11, t0, t1} of the adjoint kernel.
static void gn_step(const abea_batch* b, const double* gn, const int32_t* ast, abea_scalings_t* sc) {
    for (size_t i = 0; i < (size_t)b->n_reads; ++i) {
        if (ast[i] != 0 || b->reads[i].skip) continue;
        const double* h = &gn[5 * i];
        const double det = h[0] * h[2] - h[1] * h[1];
        if (!(det > 1e-12 * h[0] * h[2])) continue;  // fewer than two distinct levels on the path
        // [h0 h1; h1 h2] (d_shift, d_scale) = -(t1, t2)
        const double ds = (-h[3] * h[2] + h[4] * h[1]) / det;
        const double dk = (-h[4] * h[0] + h[3] * h[1]) / det;
        const double ns = (double)sc[i].shift + ds, nk = (double)sc[i].scale + dk;
        if (!std::isfinite(ns) || !std::isfinite(nk) || !(nk > 0.0)) continue;
        sc[i].shift = (float)ns;
        sc[i].scale = (float)nk;
    }
}

// Gauss-Newton on (shift, scale): the residuals (x - scale*mu - shift)/sd of the
// emitting cells of the fixed path are linear in (shift, scale), so one step
// solves the weighted least-squares problem on that path exactly; re-aligning
// with the new scalings moves the path, hence the iterations.  Far from the
// truth the first paths are partly misaligned and bias the fit, so iteration
// `it` of `n` aligns with every emission stdv multiplied by
// T = first_temperature^((n-1-it)/(n-1)) (the last one with T = 1).  A common
// factor on every sd of a read leaves its GN solution unchanged, so the normal
// equations are taken from the tempered run as they are.
extern "C" abea_status_t abea_batch_recalibrate(abea_ctx_t* c, abea_batch_t* b, int32_t iterations,
                                                double first_temperature, abea_scalings_t* out) {
    NvtxRange nv("abea recalibrate");
    if (!c || !b) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_recalibrate: null argument");
    if (b->ctx != c) return fail(ABEA_ERR_INVALID_ARG, "batch belongs to another context");
    if (iterations < 0) return fail(ABEA_ERR_INVALID_ARG, "iterations < 0");
    if (!(first_temperature > 0.0) || !std::isfinite(first_temperature))
        return fail(ABEA_ERR_INVALID_ARG, "first_temperature must be positive");
    CUDA_TRY(cudaSetDevice(c->device));
    const size_t n = (size_t)b->n_reads;
    std::vector<abea_scalings_t> sc(n), run_sc(n);
    for (size_t i = 0; i < n; ++i) {
        const ReadDesc& r = b->reads[i];
        sc[i] = abea_scalings_t{r.scale, r.shift, r.var, r.log_var};
    }
    std::vector<double> gn(5 * n);
    std::vector<int32_t> ast(n);
    const int32_t va0 = b->var_aware;
    abea_status_t st = ABEA_OK;
    for (int32_t it = 0; it < iterations && n > 0 && !st; ++it) {
        const double T = iterations > 1 && first_temperature != 1.0
                             ? pow(first_temperature, (double)(iterations - 1 - it) / (double)(iterations - 1))
                             : 1.0;
        b->var_aware = (va0 || T != 1.0) ? 1 : 0;
        for (size_t i = 0; i < n; ++i) {
            run_sc[i] = sc[i];
            if (T != 1.0) {
                run_sc[i].var = va0 ? (float)((double)sc[i].var * T) : (float)T;
                run_sc[i].log_var = va0 ? (float)((double)sc[i].log_var + log(T)) : (float)log(T);
            }
        }
        apply_scalings(b, run_sc.data());
        if ((st = upload_reads(c, b)) || (st = run_batch(c, b)) || (st = queue_backward(c, b, false))) break;
        cudaError_t e = cudaMemcpyAsync(gn.data(), b->d_gn, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ast.data(), b->d_adj_status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            st = fail(ABEA_ERR_CUDA, "recalibration: %s", cudaGetErrorString(e));
            break;
        }
        gn_step(b, gn.data(), ast.data(), sc.data());
    }
    // the batch keeps its own emission mode and the final scalings
    b->var_aware = va0;
    apply_scalings(b, sc.data());
    if (st) return st;
    if (n > 0 && iterations > 0) {
        if ((st = upload_reads(c, b)) || (st = run_batch(c, b))) return st;
        CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    if (out)
        for (size_t i = 0; i < n; ++i) out[i] = sc[i];
    return ABEA_OK;
}

// ---------------------------------------------------------------- one-call batch
// The caller's host buffer of `bytes` bytes as the device sees it: pinned memory
// is mapped into every device's address space under unified addressing.  Both
// ends must be pinned and mapped contiguously; otherwise (pageable memory)
// nullptr.
static void* device_view(void* p, size_t bytes) {
    if (!p || bytes == 0) return nullptr;
    auto view = [](void* q) -> char* {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return at.type == cudaMemoryTypeHost ? (char*)at.devicePointer : nullptr;
    };
    char* first = view(p);
    char* last = view((char*)p + bytes - 1);
    return first && last == first + bytes - 1 ? first : nullptr;
}

static abea_status_t align_batch_impl(abea_ctx* c, const HostInputs& in, abea_aligned_pair_t* pairs,
                                      int32_t* n_pairs) {
    NvtxRange nv("abea align_batch");
    abea_status_t st = validate(in);
    if (st) return st;
    CUDA_TRY(cudaSetDevice(c->device));
    if (!c->scratch) {
        c->scratch = new (std::nothrow) abea_batch();
        if (!c->scratch) return fail(ABEA_ERR_OUT_OF_MEMORY, "host allocation failed");
        c->scratch->ctx = c;
    }
    abea_batch* b = c->scratch;
    if ((st = plan(b, in, (int)c->var_aware, c->trace_budget)) || (st = ensure_device(b, c->store_scores != 0))) return st;
    // Pinned buffers of the caller are used in place: the pre stage reads each
    // read's bases and events from host memory (no input copy precedes the
    // kernel), and each read's pairs and count go into the caller's buffers as
    // the read finishes (no result copy follows it).  Pageable buffers are copied.
    InMirror im{nullptr, nullptr};
    OutMirror om{nullptr, nullptr};
    if (b->n_reads > 0) {
        if (b->seq_bytes > 0 && b->n_events_total > 0)
            im = InMirror{(const char*)device_view((void*)in.read, (size_t)b->seq_bytes),
                          (const abea_event_t*)device_view((void*)in.event_table,
                                                           sizeof(abea_event_t) * (size_t)b->n_events_total)};
        if (!im.seq || !im.ev) im = InMirror{nullptr, nullptr};
        om = OutMirror{(abea_aligned_pair_t*)device_view(pairs, sizeof(abea_aligned_pair_t) * (size_t)b->pair_cap),
                       (int32_t*)device_view(n_pairs, sizeof(int32_t) * (size_t)b->n_reads)};
    }
    const bool mirror = im.seq || om.pairs || om.n_pairs;
    // pinned: the mirrors as copied to the device, then the batch's counters and
    // statuses as copied back (read before the call returns, after one synchronize),
    // then the read descriptors as copied to the device
    const size_t desc_at = (kAuxBytes + sizeof(unsigned long long) * 4 + sizeof(int32_t) * (size_t)b->n_reads + 15) &
                           ~(size_t)15;
    const size_t aux_bytes = desc_at + sizeof(ReadDesc) * (size_t)b->n_reads;
    if (c->h_aux_bytes < aux_bytes) {
        if (c->h_aux) cudaFreeHost(c->h_aux);
        c->h_aux = nullptr;
        c->h_aux_bytes = 0;
        if (cudaHostAlloc((void**)&c->h_aux, aux_bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            c->h_aux = nullptr;
            return fail(ABEA_ERR_OUT_OF_MEMORY, "pinned host allocation failed");
        }
        c->h_aux_bytes = aux_bytes;
    }
    if (im.seq && c->mode == ABEA_MODE_BATCHED && c->wide_cluster == 0) {
        // The first reads the kernel starts are copied to HBM before it (up to 4
        // reads, 1.5 MB): otherwise they share the CPU-GPU link with every other
        // read's first loads, and the first is the longest.
        prepare_order(c, b);
        int64_t bytes = 0;
        for (size_t q = 0; q < b->dev_order.size() && q < 4; ++q) {
            ReadDesc& r = b->reads[(size_t)b->dev_order[q]];
            const int64_t rb = (int64_t)r.n_kmers + ABEA_KMER_SIZE - 1 + (int64_t)sizeof(abea_event_t) * r.n_events;
            if (r.skip || bytes + rb > ((int64_t)3 << 19)) break;
            r.in_hbm = 1;
            bytes += rb;
        }
    }
    ReadDesc* desc = (ReadDesc*)(c->h_aux + desc_at);
    if (b->n_reads > 0) memcpy(desc, b->reads.data(), sizeof(ReadDesc) * (size_t)b->n_reads);
    CUDA_TRY(cudaEventRecord(c->ev[4], c->stream));
    if ((st = upload(b, in, c->stream, im.seq == nullptr, desc))) return st;
    if (im.seq)
        for (const ReadDesc& r : b->reads) {
            if (!r.in_hbm) continue;
            CUDA_TRY(cudaMemcpyAsync(b->d_seq + r.seq_off, in.read + r.seq_off,
                                     (size_t)r.n_kmers + ABEA_KMER_SIZE - 1, cudaMemcpyHostToDevice, c->stream));
            CUDA_TRY(cudaMemcpyAsync(b->d_ev + r.ev_src, in.event_table + r.ev_src,
                                     sizeof(abea_event_t) * (size_t)r.n_events, cudaMemcpyHostToDevice, c->stream));
        }
    if (mirror) {
        memset(c->h_aux, 0, kAuxBytes);
        memcpy(c->h_aux, &im, sizeof(im));
        memcpy(c->h_aux + kAuxMirror, &om, sizeof(om));
        CUDA_TRY(cudaMemcpyAsync(b->d_aux, c->h_aux, kAuxBytes, cudaMemcpyHostToDevice, c->stream));
    }
    CUDA_TRY(cudaEventRecord(c->ev[5], c->stream));
    if ((st = run_batch(c, b))) return st;
    CUDA_TRY(cudaEventRecord(c->ev[6], c->stream));
    if ((st = download(c, b, om.pairs ? nullptr : pairs, om.n_pairs ? nullptr : n_pairs))) return st;
    char* hst = c->h_aux + kAuxBytes;
    if (b->n_reads > 0) {
        CUDA_TRY(cudaMemcpyAsync(hst, b->d_slow, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaMemcpyAsync(hst + sizeof(unsigned long long) * 4, b->d_status, sizeof(int32_t) * (size_t)b->n_reads,
                                 cudaMemcpyDeviceToHost, c->stream));
    }
    CUDA_TRY(cudaEventRecord(c->ev[7], c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if ((st = collect_timing(c, b))) return st;
    float t = 0;
    CUDA_TRY(cudaEventElapsedTime(&t, c->ev[4], c->ev[5]));
    b->timing.h2d_ms = t;
    CUDA_TRY(cudaEventElapsedTime(&t, c->ev[6], c->ev[7]));
    b->timing.d2h_ms = t;
    return check_status(c, b, hst);
}

extern "C" abea_status_t abea_align_batch(abea_ctx_t* c, int32_t n_reads, const char* read,
                                          const int64_t* read_ptr, const int32_t* read_len,
                                          const abea_event_t* event_table, const int64_t* event_ptr,
                                          const int32_t* n_events, const abea_scalings_t* scalings,
                                          const abea_model_t* model, abea_aligned_pair_t* event_align_pairs,
                                          int32_t* n_event_align_pairs) {
    if (!c) return fail(ABEA_ERR_INVALID_ARG, "abea_align_batch: null context");
    if (n_reads > 0 && (!event_align_pairs || !n_event_align_pairs))
        return fail(ABEA_ERR_INVALID_ARG, "abea_align_batch: null output");
    HostInputs in = inputs(n_reads, read, read_ptr, read_len, event_table, event_ptr, n_events, scalings, model);
    return align_batch_impl(c, in, event_align_pairs, n_event_align_pairs);
}

extern "C" abea_status_t abea_align_batch_persistent(abea_ctx_t* c, int32_t n_reads, const char* read,
                                                     const int64_t* read_ptr, const int32_t* read_len,
                                                     const abea_event_t* event_table, const int64_t* event_ptr,
                                                     const int32_t* n_events, const abea_scalings_t* scalings,
                                                     const abea_model_t* model,
                                                     abea_aligned_pair_t* event_align_pairs,
                                                     int32_t* n_event_align_pairs) {
    if (!c) return fail(ABEA_ERR_INVALID_ARG, "abea_align_batch_persistent: null context");
    const abea_mode_t mode0 = c->mode;
    c->mode = ABEA_MODE_BATCHED;
    const abea_status_t st = abea_align_batch(c, n_reads, read, read_ptr, read_len, event_table, event_ptr, n_events,
                                              scalings, model, event_align_pairs, n_event_align_pairs);
    c->mode = mode0;
    return st;
}

// f5c's db_t arrays: flatten into pinned staging (GPU/align_cuda.c:432-497's layout),
// align, unflatten.
// Runs fn(lo, hi) over contiguous ranges of [0, n) of about equal weight
// (weight(i) bytes per item, `total` in all), one range per host thread: up to
// kHostThreads, or `threads` when positive; one call on the calling thread below
// kHostMinBytes.  A thread that cannot be started leaves its range to the caller.
constexpr int kHostThreads = 8;
constexpr int64_t kHostMinBytes = 8 << 20;
template <class Weight, class Fn>
static void for_ranges(size_t n, int64_t total, int threads, Weight weight, Fn fn) {
    int t = threads;
    if (t <= 0) {
        const unsigned hw = std::max(std::thread::hardware_concurrency(), 1u);
        t = total < kHostMinBytes ? 1 : (int)std::min<unsigned>((unsigned)kHostThreads, hw);
    }
    if (t <= 1 || n < 2 || total <= 0) {
        fn((size_t)0, n);
        return;
    }
    // range k holds items [cut[k], cut[k+1]): cut[j] is the first item after the
    // weight prefix reaches j/t of the total
    std::vector<size_t> cut((size_t)t + 1, n);
    cut[0] = 0;
    int64_t acc = 0;
    int j = 1;
    for (size_t i = 0; i < n && j < t; ++i) {
        acc += weight(i);
        while (j < t && acc * t >= total * j) cut[(size_t)j++] = i + 1;
    }
    std::vector<std::thread> th;
    int started = 1;
    try {
        th.reserve((size_t)t - 1);
        for (; started < t; ++started) th.emplace_back(fn, cut[(size_t)started], cut[(size_t)started + 1]);
    } catch (...) {
        // no more threads: the calling thread takes the ranges not started
    }
    fn(cut[0], cut[1]);
    for (int k = started; k < t; ++k) fn(cut[(size_t)k], cut[(size_t)k + 1]);
    for (auto& x : th) x.join();
}

// Copies f5c's per-read arrays into the flattened layout: reads NUL separated
// from read_ptr[i], events from event_ptr[i].
static void stage_db(size_t n, char* const* read, const int32_t* read_len, const abea_event_table_t* et,
                     const int64_t* read_ptr, const int64_t* event_ptr, char* seq, abea_event_t* ev,
                     int64_t total_bytes, int threads) {
    for_ranges(
        n, total_bytes, threads,
        [=](size_t i) { return (int64_t)read_len[i] + 1 + (int64_t)sizeof(abea_event_t) * (int64_t)et[i].n; },
        [=](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; ++i) {
                if (read_len[i] > 0) memcpy(seq + read_ptr[i], read[i], (size_t)read_len[i]);
                seq[read_ptr[i] + read_len[i]] = 0;
                if (et[i].n > 0) memcpy(ev + event_ptr[i], et[i].event, sizeof(abea_event_t) * et[i].n);
            }
        });
}

// The staging of abea_align_db on its own (no device), for tests: writes the
// flattened reads and events to seq / ev; returns 0, or -1 on a bad argument.
extern "C" int32_t abea_internal_stage_db(int32_t n_reads, char* const* read, const int32_t* read_len,
                                          const abea_event_table_t* et, char* seq, abea_event_t* ev,
                                          int32_t threads) {
    if (n_reads < 0 || (n_reads > 0 && (!read || !read_len || !et || !seq || !ev))) return -1;
    const size_t n = (size_t)n_reads;
    std::vector<int64_t> read_ptr(n), event_ptr(n);
    int64_t seq_bytes = 0, events = 0;
    for (size_t i = 0; i < n; ++i) {  // the same per-read checks as abea_align_db
        if (read_len[i] < 0 || (read_len[i] > 0 && !read[i]) || (et[i].n > 0 && !et[i].event)) return -1;
        read_ptr[i] = seq_bytes;
        seq_bytes += read_len[i] + 1;
        event_ptr[i] = events;
        events += (int64_t)et[i].n;
    }
    stage_db(n, read, read_len, et, read_ptr.data(), event_ptr.data(), seq, ev,
             seq_bytes + (int64_t)sizeof(abea_event_t) * events, threads);
    return 0;
}

extern "C" abea_status_t abea_align_db(abea_ctx_t* c, int32_t n_reads, char* const* read, const int32_t* read_len,
                                       const abea_event_table_t* et, const abea_scalings_t* scalings,
                                       const abea_model_t* model, abea_aligned_pair_t* const* pairs,
                                       int32_t* n_pairs) {
    if (!c) return fail(ABEA_ERR_INVALID_ARG, "abea_align_db: null context");
    if (n_reads < 0) return fail(ABEA_ERR_INVALID_ARG, "n_reads < 0");
    if (n_reads == 0) return ABEA_OK;
    if (!read || !read_len || !et || !scalings || !model || !pairs || !n_pairs)
        return fail(ABEA_ERR_INVALID_ARG, "abea_align_db: null argument");
    const size_t n = (size_t)n_reads;
    std::vector<int64_t> read_ptr(n), event_ptr(n);
    std::vector<int32_t> n_ev(n);
    int64_t seq_bytes = 0, events = 0;
    for (size_t i = 0; i < n; ++i) {
        if (read_len[i] < 0 || (read_len[i] > 0 && !read[i]) || (et[i].n > 0 && !et[i].event) ||
            et[i].n > (size_t)(1u << 30) || !pairs[i])
            return fail(ABEA_ERR_INVALID_ARG, "abea_align_db: read %zu: bad input", i);
        read_ptr[i] = seq_bytes;
        seq_bytes += read_len[i] + 1;  // NUL separated
        event_ptr[i] = events;
        n_ev[i] = (int32_t)et[i].n;
        events += (int64_t)et[i].n;
    }
    const size_t seq_sz = align256((size_t)seq_bytes), ev_sz = align256(sizeof(abea_event_t) * (size_t)events);
    const size_t pair_sz = align256(sizeof(abea_aligned_pair_t) * (size_t)std::max<int64_t>(2 * events, 1));
    const size_t need = seq_sz + ev_sz + pair_sz;
    if (need > c->db_pin_bytes) {
        if (c->db_pin) cudaFreeHost(c->db_pin);
        c->db_pin = nullptr;
        c->db_pin_bytes = 0;
        CUDA_TRY(cudaSetDevice(c->device));
        if (cudaHostAlloc(&c->db_pin, need, cudaHostAllocDefault) != cudaSuccess) {
            c->db_pin = nullptr;
            cudaGetLastError();
            return fail(ABEA_ERR_OUT_OF_MEMORY, "pinned staging of %zu bytes failed", need);
        }
        c->db_pin_bytes = need;
    }
    char* seq = (char*)c->db_pin;
    abea_event_t* ev = (abea_event_t*)(seq + seq_sz);
    abea_aligned_pair_t* out = (abea_aligned_pair_t*)((char*)ev + ev_sz);
    stage_db(n, read, read_len, et, read_ptr.data(), event_ptr.data(), seq, ev,
             seq_bytes + (int64_t)sizeof(abea_event_t) * events, 0);
    HostInputs in = inputs(n_reads, seq, read_ptr.data(), read_len, ev, event_ptr.data(), n_ev.data(), scalings, model);
    const abea_status_t st = align_batch_impl(c, in, out, n_pairs);
    // per-read statuses (capacity, undefined) leave the other reads' results valid
    if (st != ABEA_OK && st != ABEA_ERR_CAPACITY && st != ABEA_ERR_UNDEFINED) return st;
    int64_t out_bytes = 0;
    for (size_t i = 0; i < n; ++i) out_bytes += (int64_t)sizeof(abea_aligned_pair_t) * std::max(n_pairs[i], 0);
    const int64_t* ep = event_ptr.data();
    for_ranges(
        n, out_bytes, 0, [=](size_t i) { return (int64_t)sizeof(abea_aligned_pair_t) * std::max(n_pairs[i], 0); },
        [=](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; ++i)
                if (n_pairs[i] > 0)
                    memcpy(pairs[i], out + 2 * ep[i], sizeof(abea_aligned_pair_t) * (size_t)n_pairs[i]);
        });
    return st;
}

// Method-of-moments scalings of a device-resident batch.
extern "C" abea_status_t abea_batch_estimate_scalings(abea_ctx_t* c, abea_batch_t* b, abea_scalings_t* out,
                                                      int32_t apply) {
    if (!c || !b) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_estimate_scalings: null argument");
    if (b->ctx != c) return fail(ABEA_ERR_INVALID_ARG, "batch belongs to another context");
    if (b->n_reads == 0) return ABEA_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    const size_t n = (size_t)b->n_reads;
    MomArgs m{b->d_reads, b->n_reads, b->d_seq, b->d_ev, b->d_model, b->d_gn};  // d_gn: [n][5] scratch
    cudaError_t e = launch_mom(m, c->stream);
    if (e != cudaSuccess) return fail(ABEA_ERR_CUDA, "moment kernel launch failed: %s", cudaGetErrorString(e));
    std::vector<double> v(2 * n);
    CUDA_TRY(cudaMemcpyAsync(v.data(), b->d_gn, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    std::vector<abea_scalings_t> sc(n);
    for (size_t i = 0; i < n; ++i) sc[i] = abea_scalings_t{(float)v[2 * i], (float)v[2 * i + 1], 1.0f, 0.0f};
    if (out) memcpy(out, sc.data(), sizeof(abea_scalings_t) * n);
    if (apply) {
        apply_scalings(b, sc.data());
        return upload_reads(c, b);
    }
    return ABEA_OK;
}

// f5c's postalign for every read of a run batch, on the AlignedPairs in HBM.
extern "C" abea_status_t abea_batch_postalign(abea_ctx_t* c, abea_batch_t* b, abea_event_alignment_t* alignment,
                                              abea_index_pair_t* base_to_event_map, double* events_per_base,
                                              int32_t* n_alignment) {
    if (!c || !b) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_postalign: null argument");
    if (b->ctx != c) return fail(ABEA_ERR_INVALID_ARG, "batch belongs to another context");
    if (!b->ran) return fail(ABEA_ERR_INVALID_ARG, "batch has not been run");
    if (b->n_reads == 0) return ABEA_OK;
    NvtxRange nv("abea postalign");
    CUDA_TRY(cudaSetDevice(c->device));
    const size_t n = (size_t)b->n_reads;
    const size_t n_rec = (size_t)std::max<int64_t>(b->n_events_total, 1);
    const size_t n_map = (size_t)std::max<int64_t>(b->seq_bytes, 1);
    const size_t rec_bytes = sizeof(abea_event_alignment_t) * n_rec, map_bytes = sizeof(abea_index_pair_t) * n_map;
    const size_t off_map = (size_t)round_up((int64_t)rec_bytes, 256);
    const size_t off_epb = off_map + (size_t)round_up((int64_t)map_bytes, 256);
    const size_t off_cnt = off_epb + (size_t)round_up((int64_t)(sizeof(double) * n), 256);
    const size_t need = off_cnt + sizeof(int32_t) * n;
    if (b->post_bytes < need) {
        if (b->d_post) cudaFree(b->d_post);
        b->d_post = nullptr;
        b->post_bytes = 0;
        if (cudaMalloc(&b->d_post, need) != cudaSuccess) {
            cudaGetLastError();
            b->d_post = nullptr;
            return fail(ABEA_ERR_OUT_OF_MEMORY, "postalign outputs: cannot allocate %zu bytes", need);
        }
        b->post_bytes = need;
    }
    char* base = (char*)b->d_post;
    PostalignArgs pa{b->d_reads,
                     b->n_reads,
                     b->d_seq,
                     b->d_pairs,
                     b->d_n_pairs,
                     (abea_index_pair_t*)(base + off_map),
                     (abea_event_alignment_t*)base,
                     (double*)(base + off_epb),
                     (int32_t*)(base + off_cnt)};
    CUDA_TRY(cudaMemsetAsync(pa.rec, 0, rec_bytes, c->stream));
    CUDA_TRY(cudaMemsetAsync(pa.map, 0xff, map_bytes, c->stream));  // {-1, -1}
    cudaError_t e = launch_postalign(pa, c->stream);
    if (e != cudaSuccess) return fail(ABEA_ERR_CUDA, "postalign kernel launch failed: %s", cudaGetErrorString(e));
    std::vector<int32_t> cnt(n);
    if (alignment)
        CUDA_TRY(cudaMemcpyAsync(alignment, pa.rec, sizeof(abea_event_alignment_t) * (size_t)b->n_events_total,
                                 cudaMemcpyDeviceToHost, c->stream));
    if (base_to_event_map)
        CUDA_TRY(cudaMemcpyAsync(base_to_event_map, pa.map, sizeof(abea_index_pair_t) * (size_t)b->seq_bytes,
                                 cudaMemcpyDeviceToHost, c->stream));
    if (events_per_base)
        CUDA_TRY(cudaMemcpyAsync(events_per_base, pa.epb, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaMemcpyAsync(cnt.data(), pa.count, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (n_alignment) memcpy(n_alignment, cnt.data(), sizeof(int32_t) * n);
    for (size_t i = 0; i < n; ++i)
        if (cnt[i] < 0) return fail(ABEA_ERR_INTERNAL, "read %zu: its AlignedPairs are not a path of unit steps", i);
    return ABEA_OK;
}

// ---------------------------------------------------------------- serving stream
// Device bytes one read adds to a batch's slab (the per-read terms of
// ensure_device), and the slab's fixed part (model, model gradient, counters,
// alignment padding).
static int64_t read_device_bytes(int32_t len, int32_t ne, int64_t trace_budget, bool scores) {
    const int64_t nk = (int64_t)len - ABEA_KMER_SIZE + 1;
    int64_t bytes = (int64_t)sizeof(ReadDesc) + len + 1 + (int64_t)sizeof(abea_event_t) * ne +
                    (int64_t)sizeof(abea_aligned_pair_t) * 2 * ne +
                    8 * (int64_t)sizeof(int32_t) + 9 * (int64_t)sizeof(double);
    if (nk > 0 && ne > 0) {
        const int64_t nb = ne + nk + 2, nb4 = round_up(nb, 4);
        bytes += 2 * 4 * round_up(ne, kChunk) + 4 * 4 * round_up(nk, kChunk) + 4 * nb4;
        const int64_t trace = nb4 * kSlots;
        if (trace_budget > 0 && trace > trace_budget)
            bytes += 4 * (nb / kCkBands + 1) * kCkStride + (int64_t)kCkBands * kSlots;
        else
            bytes += trace;
        if (scores) bytes += 4 * (int64_t)kSlots * nb4;
    }
    return bytes;
}

static int64_t slab_fixed_bytes() {
    return (int64_t)sizeof(abea_model_t) * ABEA_NUM_KMER + 2 * (int64_t)sizeof(double) * ABEA_NUM_KMER +
           32 * 256 + 16 * 1024;
}

// Traceback cell maps of a batch holding n reads of at least kSpecMinBands bands.
static int64_t spec_bytes(int64_t n) {
    return (int64_t)sizeof(int32_t) * kSpecRound * kSpecBands * std::min<int64_t>(n, kSpecMaxSlots);
}

static void CUDART_CB stamp_now(void* p) {
    *(std::chrono::steady_clock::time_point*)p = std::chrono::steady_clock::now();
}

namespace {
// One of the two device batches of a stream: its inputs rebased to the batch.
struct StreamSlot {
    abea_batch* b = nullptr;
    cudaEvent_t* ev = nullptr;  // uploaded, compute start, compute end, results copied
    std::vector<int64_t> rp, ep;
    int32_t r0 = 0, r1 = 0;
    int64_t ev_base = 0;
    bool busy = false;  // work of its last batch is queued
};
}  // namespace

extern "C" abea_status_t abea_align_stream(abea_ctx_t* c, const abea_stream_config_t* cfg, int32_t n_reads,
                                           const char* read, const int64_t* read_ptr, const int32_t* read_len,
                                           const abea_event_t* event_table, const int64_t* event_ptr,
                                           const int32_t* n_events, const abea_scalings_t* scalings,
                                           const abea_model_t* model, abea_aligned_pair_t* pairs,
                                           int32_t* n_pairs, abea_scalings_t* scalings_out, double* latency_ms,
                                           abea_stream_stats_t* stats) {
    NvtxRange nv("abea align_stream");
    using clock = std::chrono::steady_clock;
    const clock::time_point t_call = clock::now();
    if (!c) return fail(ABEA_ERR_INVALID_ARG, "abea_align_stream: null context");
    if (n_reads > 0 && (!pairs || !n_pairs)) return fail(ABEA_ERR_INVALID_ARG, "abea_align_stream: null output");
    const abea_stream_config_t conf = cfg ? *cfg : abea_stream_config_t{0, 0, 0};
    if (conf.batch_bytes < 0 || conf.recalibrate < 0 || conf.recalibrate > 1 || conf.reserved != 0)
        return fail(ABEA_ERR_INVALID_ARG, "abea_align_stream: bad configuration");
    const HostInputs all = inputs(n_reads, read, read_ptr, read_len, event_table, event_ptr, n_events, scalings, model);
    abea_status_t st = validate(all);
    if (st) return st;
    for (int32_t i = 0; i + 1 < n_reads; ++i)
        if (event_ptr[i] + n_events[i] > event_ptr[i + 1])
            return fail(ABEA_ERR_INVALID_ARG, "abea_align_stream: event ranges of reads %d and %d overlap or are out of order",
                        i, i + 1);
    if (stats) *stats = abea_stream_stats_t{};
    if (n_reads == 0) return ABEA_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    int64_t budget = conf.batch_bytes;
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        CUDA_TRY(cudaMemGetInfo(&fr, &tot));
        budget = std::min<int64_t>(16ll << 30, (int64_t)(0.4 * (double)fr));
    }
    // admission in input order by device footprint
    const bool scores = c->store_scores != 0;
    std::vector<int32_t> cut = {0};
    std::vector<int64_t> cut_bytes;
    int64_t acc = slab_fixed_bytes(), max_bytes = 0, cells = 0, n_long = 0;
    for (int32_t i = 0; i < n_reads; ++i) {
        const int64_t rb = read_device_bytes(read_len[i], n_events[i], c->trace_budget, scores);
        const int64_t nk = (int64_t)read_len[i] - ABEA_KMER_SIZE + 1;
        const int64_t nb = nk > 0 && n_events[i] > 0 ? n_events[i] + nk + 2 : 0;
        const bool trace_kept = c->trace_budget <= 0 || round_up(nb, 4) * kSlots <= c->trace_budget;
        const int64_t lg = nb >= kSpecMinBands && trace_kept ? 1 : 0;  // a traceback map slot
        if (i > cut.back() && acc + rb + spec_bytes(n_long + lg) > budget) {
            cut.push_back(i);
            cut_bytes.push_back(acc + spec_bytes(n_long));
            max_bytes = std::max(max_bytes, acc + spec_bytes(n_long));
            acc = slab_fixed_bytes();
            n_long = 0;
        }
        acc += rb;
        n_long += lg;
        cells += nb * (int64_t)kBand;
    }
    cut.push_back(n_reads);
    cut_bytes.push_back(acc + spec_bytes(n_long));
    max_bytes = std::max(max_bytes, acc + spec_bytes(n_long));
    const int nb = (int)cut.size() - 1;
    // resources kept by the context
    if (!c->copy_stream) CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        if (!c->sslot[i]) {
            c->sslot[i] = new (std::nothrow) abea_batch();
            if (!c->sslot[i]) return fail(ABEA_ERR_OUT_OF_MEMORY, "host allocation failed");
            c->sslot[i]->ctx = c;
        }
        for (int j = 0; j < 4; ++j)
            if (!c->sev[i][j]) CUDA_TRY(cudaEventCreate(&c->sev[i][j]));
    }
    int32_t* status = nullptr;
    if (cudaHostAlloc((void**)&status, sizeof(int32_t) * (size_t)n_reads, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return fail(ABEA_ERR_OUT_OF_MEMORY, "pinned status array failed");
    }
    StreamSlot slot[2];
    for (int i = 0; i < 2; ++i) {
        slot[i].b = c->sslot[i];
        slot[i].ev = c->sev[i];
    }
    std::vector<clock::time_point> admit((size_t)nb), done((size_t)nb);
    cudaStream_t cs = c->copy_stream;
    double compute_ms = 0;
    int32_t max_reads = 0;
    std::vector<abea_scalings_t> sc;
    std::vector<double> gn;
    std::vector<int32_t> ast;

    auto harvest = [&](StreamSlot& S) -> abea_status_t {  // the slot's last batch is done
        if (!S.busy) return ABEA_OK;
        CUDA_TRY(cudaEventSynchronize(S.ev[3]));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, S.ev[1], S.ev[2]));
        compute_ms += ms;
        S.busy = false;
        return ABEA_OK;
    };
    auto prepare = [&](int k) -> abea_status_t {  // admit batch k: plan and copy to the device
        StreamSlot& S = slot[k & 1];
        abea_status_t s2 = harvest(S);
        if (s2) return s2;
        S.r0 = cut[(size_t)k];
        S.r1 = cut[(size_t)k + 1];
        const int32_t n = S.r1 - S.r0;
        max_reads = std::max(max_reads, n);
        int64_t rbase = read_ptr[S.r0];
        for (int32_t i = S.r0; i < S.r1; ++i) rbase = std::min(rbase, read_ptr[i]);
        S.ev_base = event_ptr[S.r0];
        S.rp.resize((size_t)n);
        S.ep.resize((size_t)n);
        for (int32_t i = 0; i < n; ++i) {
            S.rp[(size_t)i] = read_ptr[S.r0 + i] - rbase;
            S.ep[(size_t)i] = event_ptr[S.r0 + i] - S.ev_base;
        }
        HostInputs in = inputs(n, read + rbase, S.rp.data(), read_len + S.r0,
                               event_table ? event_table + S.ev_base : nullptr, S.ep.data(), n_events + S.r0,
                               scalings + S.r0, model);
        if ((s2 = plan(S.b, in, (int)c->var_aware, c->trace_budget)) ||
            (s2 = ensure_device(S.b, scores, (size_t)max_bytes)))
            return s2;
        prepare_order(c, S.b);
        admit[(size_t)k] = clock::now();
        if ((s2 = upload(S.b, in, cs))) return s2;
        if (c->mode == ABEA_MODE_BATCHED) {  // the batched form's order, so that the run needs no copy
            CUDA_TRY(cudaMemcpyAsync(S.b->d_order, S.b->dev_order.data(), sizeof(int32_t) * S.b->dev_order.size(),
                                     cudaMemcpyHostToDevice, cs));
            S.b->dev_order_sent = S.b->dev_order;
        }
        CUDA_TRY(cudaEventRecord(S.ev[0], cs));
        S.busy = true;
        return ABEA_OK;
    };
    auto start = [&](int k) -> abea_status_t {  // align batch k
        StreamSlot& S = slot[k & 1];
        CUDA_TRY(cudaStreamWaitEvent(c->stream, S.ev[0], 0));
        CUDA_TRY(cudaEventRecord(S.ev[1], c->stream));
        return run_batch(c, S.b);
    };
    auto finish = [&](int k) -> abea_status_t {  // recalibrate, re-align, copy the results back
        StreamSlot& S = slot[k & 1];
        abea_batch* b = S.b;
        const size_t n = (size_t)b->n_reads;
        abea_status_t s2;
        if (conf.recalibrate) {
            if ((s2 = queue_backward(c, b, false))) return s2;
            gn.resize(5 * n);
            ast.resize(n);
            CUDA_TRY(cudaMemcpyAsync(gn.data(), b->d_gn, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost, c->stream));
            CUDA_TRY(cudaMemcpyAsync(ast.data(), b->d_adj_status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                     c->stream));
            CUDA_TRY(cudaStreamSynchronize(c->stream));
            sc.resize(n);
            for (size_t i = 0; i < n; ++i) {
                const ReadDesc& r = b->reads[i];
                sc[i] = abea_scalings_t{r.scale, r.shift, r.var, r.log_var};
            }
            gn_step(b, gn.data(), ast.data(), sc.data());
            apply_scalings(b, sc.data());
            if ((s2 = upload_reads(c, b)) || (s2 = run_batch(c, b))) return s2;
        }
        if (scalings_out)
            for (size_t i = 0; i < n; ++i) {
                const ReadDesc& r = b->reads[i];
                scalings_out[S.r0 + i] = abea_scalings_t{r.scale, r.shift, r.var, r.log_var};
            }
        CUDA_TRY(cudaEventRecord(S.ev[2], c->stream));
        CUDA_TRY(cudaStreamWaitEvent(cs, S.ev[2], 0));
        if (b->pair_cap > 0)
            CUDA_TRY(cudaMemcpyAsync(pairs + 2 * S.ev_base, b->d_pairs, sizeof(abea_aligned_pair_t) * (size_t)b->pair_cap,
                                     cudaMemcpyDeviceToHost, cs));
        CUDA_TRY(cudaMemcpyAsync(n_pairs + S.r0, b->d_n_pairs, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, cs));
        CUDA_TRY(cudaMemcpyAsync(status + S.r0, b->d_status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, cs));
        CUDA_TRY(cudaEventRecord(S.ev[3], cs));
        CUDA_TRY(cudaLaunchHostFunc(cs, stamp_now, &done[(size_t)k]));
        return ABEA_OK;
    };

    st = prepare(0);
    for (int k = 0; k < nb && !st; ++k) {
        if ((st = start(k))) break;
        if (k + 1 < nb && (st = prepare(k + 1))) break;  // overlaps batch k's alignment
        st = finish(k);
    }
    // drain both streams before returning (copies into the caller's buffers)
    const cudaError_t e1 = cudaStreamSynchronize(c->stream), e2 = cudaStreamSynchronize(cs);
    if (!st && e1 != cudaSuccess) st = fail(ABEA_ERR_CUDA, "stream: %s", cudaGetErrorString(e1));
    if (!st && e2 != cudaSuccess) st = fail(ABEA_ERR_CUDA, "stream: %s", cudaGetErrorString(e2));
    for (int i = 0; i < 2 && !st; ++i) st = harvest(slot[i]);
    for (int i = 0; i < 2; ++i) slot[i].busy = false;
    if (!st) {
        for (int32_t i = 0; i < n_reads; ++i)
            if (status[i] != 0) {
                st = fail((abea_status_t)status[i], "read %d: %s", i, abea_status_string((abea_status_t)status[i]));
                break;
            }
    }
    cudaFreeHost(status);
    if (st) return st;
    clock::time_point last = t_call;
    for (int k = 0; k < nb; ++k) {
        last = std::max(last, done[(size_t)k]);
        if (latency_ms) {
            const double ms = std::chrono::duration<double, std::milli>(done[(size_t)k] - admit[(size_t)k]).count();
            for (int32_t i = cut[(size_t)k]; i < cut[(size_t)k + 1]; ++i) latency_ms[i] = ms;
        }
    }
    if (stats) {
        stats->n_batches = nb;
        stats->max_batch_reads = max_reads;
        stats->max_batch_bytes = max_bytes;
        stats->band_cells = cells;
        stats->wall_ms = std::chrono::duration<double, std::milli>(last - t_call).count();
        stats->compute_ms = compute_ms;
    }
    return ABEA_OK;
}

extern "C" abea_status_t abea_ctx_last_timing(abea_ctx_t* c, abea_timing_t* t, int64_t* h2d, int64_t* d2h) {
    if (!c || !t) return fail(ABEA_ERR_INVALID_ARG, "abea_ctx_last_timing: null argument");
    if (!c->scratch) return fail(ABEA_ERR_INVALID_ARG, "no batch has run on this context");
    *t = c->scratch->timing;
    if (h2d) *h2d = h2d_bytes(c->scratch);
    if (d2h) *d2h = d2h_bytes(c->scratch);
    return ABEA_OK;
}

extern "C" abea_status_t abea_batch_io_bytes(abea_batch_t* b, int64_t* h2d, int64_t* d2h, int64_t* band_cells) {
    if (!b) return fail(ABEA_ERR_INVALID_ARG, "abea_batch_io_bytes: null batch");
    if (h2d) *h2d = h2d_bytes(b);
    if (d2h) *d2h = d2h_bytes(b);
    if (band_cells) *band_cells = b->band_cells;
    return ABEA_OK;
}

// ---------------------------------------------------------------- f5c align()
// One context per calling thread: f5c calls align() from its worker threads
// (GPU/f5c.h:57-59), so each thread queues on its own stream.
struct ThreadCtx {
    abea_ctx* ctx = nullptr;
    ~ThreadCtx() {
        if (ctx) abea_ctx_destroy(ctx);
    }
};
static thread_local ThreadCtx t_ctx;

extern "C" int32_t abea_align_cap(abea_aligned_pair_t* out_2, int32_t out_capacity, const char* sequence,
                                  int32_t sequence_len, const abea_event_t* events, int32_t n_events,
                                  const abea_model_t* models, abea_scalings_t scaling) {
    if (!out_2 || !sequence || !models || out_capacity < 0 || sequence_len < 0 || n_events < 0 ||
        (n_events > 0 && !events))
        return fail(ABEA_ERR_INVALID_ARG, "abea_align: invalid argument");
    if (!t_ctx.ctx) {
        // The batched form puts a lone read on the wide shape (about 380 cycles per
        // band, against 1,150 for one warp); every call has its own layout, so
        // there is no graph to replay.
        int dev = 0;
        cudaGetDevice(&dev);
        abea_status_t st = abea_ctx_create(&t_ctx.ctx, dev, ABEA_MODE_BATCHED);
        if (st) return st;
        abea_ctx_set_option(t_ctx.ctx, ABEA_OPT_USE_GRAPH, 0);
    }
    abea_ctx* c = t_ctx.ctx;
    int64_t read_ptr = 0, event_ptr = 0;
    int32_t npairs = 0;
    // the batch output has room for 2*n_events pairs; stage it when the caller's
    // slot is smaller
    std::vector<abea_aligned_pair_t> tmp((size_t)std::max(2 * n_events, 1));
    HostInputs in = inputs(1, sequence, &read_ptr, &sequence_len, events, &event_ptr, &n_events, &scaling, models);
    abea_status_t st = align_batch_impl(c, in, tmp.data(), &npairs);
    if (st) return st;
    if (npairs < 0) return npairs;
    if (npairs > out_capacity) return fail(ABEA_ERR_CAPACITY, "abea_align: %d pairs exceed capacity %d", npairs, out_capacity);
    memcpy(out_2, tmp.data(), sizeof(abea_aligned_pair_t) * (size_t)npairs);
    return npairs;
}

extern "C" int32_t abea_align(abea_aligned_pair_t* out_2, char* sequence, int32_t sequence_len,
                              abea_event_table_t events, abea_model_t* models, abea_scalings_t scaling,
                              float sample_rate) {
    (void)sample_rate;  // unused by the algorithm, as in the reference
    if (events.n > (size_t)0x3fffffff) return fail(ABEA_ERR_INVALID_ARG, "abea_align: too many events");
    int32_t ne = (int32_t)events.n;
    return abea_align_cap(out_2, 2 * ne, sequence, sequence_len, events.event, ne, models, scaling);
}

// f5c's own symbol: a weak alias, so that an f5c build that drops its CPU
// align.c links this library in its place while a build that keeps it wins.
extern "C" int32_t align(abea_aligned_pair_t* out_2, char* sequence, int32_t sequence_len,
                         abea_event_table_t events, abea_model_t* models, abea_scalings_t scaling,
                         float sample_rate) __attribute__((weak, alias("abea_align")));

// ---------------------------------------------------------------- timing helpers
extern "C" abea_status_t abea_ctx_mark(abea_ctx_t* c, int i) {
    if (!c || i < 0 || i >= 16) return fail(ABEA_ERR_INVALID_ARG, "abea_ctx_mark: bad argument");
    CUDA_TRY(cudaEventRecord(c->marker[i], c->stream));
    return ABEA_OK;
}

extern "C" abea_status_t abea_ctx_elapsed(abea_ctx_t* c, int i, int j, float* ms) {
    if (!c || !ms || i < 0 || i >= 16 || j < 0 || j >= 16)
        return fail(ABEA_ERR_INVALID_ARG, "abea_ctx_elapsed: bad argument");
    CUDA_TRY(cudaEventSynchronize(c->marker[j]));
    CUDA_TRY(cudaEventElapsedTime(ms, c->marker[i], c->marker[j]));
    return ABEA_OK;
}

extern "C" abea_status_t abea_ctx_flush_l2(abea_ctx_t* c) {
    if (!c) return fail(ABEA_ERR_INVALID_ARG, "abea_ctx_flush_l2: null context");
    CUDA_TRY(cudaSetDevice(c->device));
    if (!c->flush_buf) {
        int l2 = 0;
        CUDA_TRY(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->device));
        size_t bytes = std::max<size_t>((size_t)l2 * 2, (size_t)256 << 20);
        CUDA_TRY(cudaMalloc(&c->flush_buf, bytes));
        c->flush_bytes = bytes;
    }
    static int flip = 0;
    CUDA_TRY(cudaMemsetAsync(c->flush_buf, (flip++) & 0xff, c->flush_bytes, c->stream));
    return ABEA_OK;
}

// ---------------------------------------------------------------- single-read description
// ReadDesc of one read whose scratch regions all start at offset 0 (used by the
// no-allocation entry point, which lays the regions out itself).
namespace abea {
ReadDesc describe_single_read(int32_t sequence_len, int32_t n_events, abea_scalings_t sc, int32_t out_capacity) {
    ReadDesc r{};
    const int32_t nk = sequence_len - ABEA_KMER_SIZE + 1;
    r.n_events = n_events;
    r.n_kmers = nk;
    r.out_cap = out_capacity;
    r.scale = sc.scale;
    r.shift = sc.shift;
    r.var = sc.var;
    r.log_var = sc.log_var;
    r.skip = (nk <= 0 || n_events <= 0) ? 1 : 0;
    if (r.skip) return r;
    r.n_bands = n_events + nk + 2;
    Penalties p = penalties(n_events, nk);
    r.lp_step = p.lp_step;
    r.lp_stay = p.lp_stay;
    split(p.lp_step, r.step_h, r.step_l);
    split(p.lp_stay, r.stay_h, r.stay_l);
    return r;
}
GlobalConsts parity_consts() { return global_consts(0); }
}  // namespace abea

extern "C" const char* abea_internal_set_error(const char* msg) {
    g_last_error = msg;
    return g_last_error.c_str();
}

// The batched form's heuristic wide-shape threshold for a batch of reads with
// these band counts on `blocks` resident blocks (no device needed): for tests
// and for callers who size batches.  INT64_MAX = no wide read; -1 = bad input.
// The heuristic on band counts alone (host code, for tests); ck (optional) marks
// the reads whose trace is not kept (checkpointed), which stay on the warp shape.
extern "C" int64_t abea_internal_wide_threshold_ck(const int64_t* n_bands, const int32_t* ck, int32_t n_reads,
                                                   int32_t blocks) {
    if (n_reads < 0 || blocks < 1 || (n_reads > 0 && !n_bands)) return -1;
    abea_batch b;
    b.n_reads = n_reads;
    b.reads.assign((size_t)n_reads, ReadDesc{});
    for (int32_t i = 0; i < n_reads; ++i) {
        if (n_bands[i] < 0) return -1;
        b.reads[(size_t)i].n_bands = (int32_t)std::min<int64_t>(n_bands[i], INT32_MAX);
        b.reads[(size_t)i].ck = ck && ck[i] ? 1 : 0;
    }
    b.order.resize((size_t)n_reads);
    std::iota(b.order.begin(), b.order.end(), 0);
    std::stable_sort(b.order.begin(), b.order.end(), [&](int32_t x, int32_t y) {
        return b.reads[(size_t)x].n_bands > b.reads[(size_t)y].n_bands;
    });
    return heuristic_threshold(&b, blocks);
}

extern "C" int64_t abea_internal_wide_threshold(const int64_t* n_bands, int32_t n_reads, int32_t blocks) {
    return abea_internal_wide_threshold_ck(n_bands, nullptr, n_reads, blocks);
}
