// C-ABI layer: the reference's include/orth.h entry points on one GB300, and the
// device-pointer extension declared in include/orth_gb300.h.
//
// Each variant's driver below issues, per block step, exactly the reference's
// sequence of operations (cited per line), with MPI_Allreduce replaced by one
// deterministic device-wide reduction and every small s x s step kept on the
// device, so a whole QR is enqueued on one stream with no host round trip.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <climits>
#include <deque>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/orth.h"
#include "../../include/orth_gb300.h"
#include "common.cuh"
#include "kernels.h"
#include "host_stage.h"
#include "split.h"

namespace bcgs {

std::atomic<long long> g_launch_count{0};
std::atomic<long long> g_reduce_count{0};

static inline bool is_split(int precision) {
    return precision == ORTH_GB300_SPLIT_BF16 || precision == ORTH_GB300_SPLIT_BF16_FAST;
}
static inline int split_digits_of(int precision) { return precision == ORTH_GB300_SPLIT_BF16_FAST ? 6 : 7; }

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t want) {
        if (want <= bytes) return 0;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) return (int)e;
        bytes = want;
        return 0;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

// Cached workspace (grow-only). The reference is not thread-safe either (it uses
// MPI_COMM_WORLD collectives); calls are serialized by a mutex here.
// Per-call scratch of the drivers. Slot 0 serves every entry point; split-precision
// batches use up to kSlots slots, one per concurrent stream.
constexpr int kSlots = 16;
struct Scratch {
    DevBuf part, small, status, tsqr, split;
};
Scratch g_scratch[kSlots];
thread_local int g_slot = 0;
inline Scratch& scr() { return g_scratch[g_slot]; }

struct Context {
    DevBuf gram, hostX, hostR, metric;
    cudaStream_t slot_stream[kSlots] = {};
    double* hostR_stage = nullptr;
    size_t hostR_stage_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;   // host-path column transfers
    // Host-path timeline: call start, last H2D chunk landed, the QR's kernels done,
    // last D2H chunk landed.
    cudaEvent_t host_ev[4] = {};
    int num_sms = kNumSMsDefault;
    bool init = false;
};

Context g_ctx;
std::mutex g_mu;

// Optional per-kernel-class timing with CUDA events recorded on the launching
// stream around each launch group. Classes: 0 tall Gram (incl. its reduction),
// 1 tall update, 2 small s x s kernels, 3 TSQR, 4 digit slicing (split modes).
// Algorithmic flops are FP64-equivalent (2 per multiply-add of the FP64 product).
// Algorithmic bytes are FP64-equivalent too: 8 bytes per element of every
// operand column the product must read once and every column it writes, in any
// precision. Traffic bytes are what the kernels as built move at least: the
// same for the FP64 form; BF16 digit planes (2 bytes x digits per element) for
// the operands the split forms read.
constexpr int kProfClasses = 5;
struct ProfPending { int cls; cudaEvent_t a, b; };
struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    std::vector<ProfPending> pending;
    double ms[kProfClasses] = {0, 0, 0, 0, 0};
    long long launches[kProfClasses] = {0, 0, 0, 0, 0};
    double flops[kProfClasses] = {0, 0, 0, 0, 0};
    double bytes[kProfClasses] = {0, 0, 0, 0, 0};
    double traffic[kProfClasses] = {0, 0, 0, 0, 0};
    long long calls[kProfClasses] = {0, 0, 0, 0, 0};
    cudaEvent_t get() {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
};
Prof g_prof;

struct ProfScope {
    int cls;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    long long l0;
    ProfScope(int c, cudaStream_t s, double flops, double bytes, double traffic = -1.0)
        : cls(c), st(s), l0(g_launch_count - g_aux_launch_count) {
        if (!g_prof.on) return;
        a = g_prof.get();
        cudaEventRecord(a, st);
        g_prof.flops[cls] += flops;
        g_prof.bytes[cls] += bytes;
        g_prof.traffic[cls] += traffic < 0.0 ? bytes : traffic;
        g_prof.calls[cls] += 1;
    }
    ~ProfScope() {
        if (!g_prof.on) return;
        cudaEvent_t b = g_prof.get();
        cudaEventRecord(b, st);
        g_prof.pending.push_back({cls, a, b});
        g_prof.launches[cls] += g_launch_count - g_aux_launch_count - l0;
    }
};
thread_local orth_gb300_status g_last_status = {0, 0, 0, 0};
// Timeline of this thread's last host-buffer run (ms from its first device
// operation): X resident, compute done, Q and R back; then the call's wall time.
thread_local double g_last_host_timing[4] = {0, 0, 0, 0};

// Precision of the orth.h host entry points: FP64 (the reference's arithmetic)
// unless set through orth_gb300_set_host_precision or ORTH_GB300_PRECISION
// ("fp64", "split", "split_fast") at first use.
int g_host_precision = -1;
int host_precision() {
    if (g_host_precision < 0) {
        g_host_precision = ORTH_GB300_FP64;
        const char* e = getenv("ORTH_GB300_PRECISION");
        if (e && strcmp(e, "split") == 0) g_host_precision = ORTH_GB300_SPLIT_BF16;
        if (e && strcmp(e, "split_fast") == 0) g_host_precision = ORTH_GB300_SPLIT_BF16_FAST;
    }
    return g_host_precision;
}
// IntraOrtho of the panels the reference hands to TSQR (block 1 of every
// variant; each step's panels in bcgsi2 and bcgsi2P2s): the TSQR tree (the
// reference's choice, default) or CholQR2, set through orth_gb300_set_intra_ortho
// or ORTH_GB300_INTRA ("tsqr", "cholqr2") at first use.
int g_intra_mode = -1;
int intra_mode() {
    if (g_intra_mode < 0) {
        g_intra_mode = ORTH_GB300_INTRA_TSQR;
        const char* e = getenv("ORTH_GB300_INTRA");
        if (e && strcmp(e, "cholqr2") == 0) g_intra_mode = ORTH_GB300_INTRA_CHOLQR2;
    }
    return g_intra_mode;
}
std::atomic<long long> g_last_launches{0};
thread_local long long g_last_reductions = 0;

int init_ctx() {
    if (g_ctx.init) return 0;
    int dev = 0;
    BCGS_CUDA_TRY(cudaGetDevice(&dev));
    BCGS_CUDA_TRY(cudaDeviceGetAttribute(&g_ctx.num_sms, cudaDevAttrMultiProcessorCount, dev));
    BCGS_CUDA_TRY(cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking));
    BCGS_CUDA_TRY(cudaStreamCreateWithFlags(&g_ctx.copy_in, cudaStreamNonBlocking));
    BCGS_CUDA_TRY(cudaStreamCreateWithFlags(&g_ctx.copy_out, cudaStreamNonBlocking));
    for (cudaEvent_t& e : g_ctx.host_ev) BCGS_CUDA_TRY(cudaEventCreate(&e));
    g_ctx.init = true;
    return 0;
}

// Largest Gram-partial buffer any step needs (doubles).
i64 part_doubles(i64 m, int n, int s, int num_sms) {
    i64 best = 0;
    const int na_max = n + s, nb_max = 2 * s;
    for (int na = 1; na <= na_max; ++na) {
        for (int nb = 1; nb <= nb_max; ++nb) {
            i64 v = gram_chunks_fp64(m, na, nb, num_sms) * (i64)na * nb;
            if (v > best) best = v;
        }
    }
    return best + 1024;
}

// Small buffers carved from one allocation (doubles).
struct Small {
    double* G1;    // (n+s) x 2s reduced Gram
    double* G2;    // (n+s) x 2s second reduced Gram (two-sync variants)
    double* Scol;  // n x s
    double* S0;    // s x s first-step coefficients
    double* Sd;    // s x s
    double* Yd;    // s x s
    double* Cq;    // 3 s x s: CholQR2's panel Gram, R1 and R2
};

i64 small_doubles(int n, int s) {
    return 2LL * (n + s) * 2 * s + (i64)n * s + 6LL * s * s + 64;
}

Small carve_small(double* base, int n, int s) {
    Small w;
    w.G1 = base;
    w.G2 = w.G1 + (i64)(n + s) * 2 * s;
    w.Scol = w.G2 + (i64)(n + s) * 2 * s;
    w.S0 = w.Scol + (i64)n * s;
    w.Sd = w.S0 + (i64)s * s;
    w.Yd = w.Sd + (i64)s * s;
    w.Cq = w.Yd + (i64)s * s;
    return w;
}

int reserve(i64 m, int n, int s, int precision) {
    int rc = init_ctx();
    if (rc) return rc;
    rc = scr().part.ensure((size_t)part_doubles(m, n, s, g_ctx.num_sms) * sizeof(double));
    if (rc) return rc;
    rc = scr().small.ensure((size_t)small_doubles(n, s) * sizeof(double));
    if (rc) return rc;
    rc = scr().status.ensure(kStatusWords * sizeof(int));
    if (rc) return rc;
    rc = scr().tsqr.ensure((size_t)tsqr_workspace_doubles(m, s) * sizeof(double));
    if (rc) return rc;
    if (is_split(precision)) {
        rc = scr().split.ensure((size_t)split_workspace_bytes(m, n, s, g_ctx.num_sms));
        if (rc) return rc;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Host-buffer runs (the orth.h entry points): X arrives in column chunks on one
// copy stream and Q leaves on another while the QR runs; the two directions
// overlap on the link. The compute stream waits only for the chunks a primitive
// reads (need). Every update or TSQR that writes from column c0 marks columns
// [0, c0) final (final). No variant writes a column left of the block it is
// working on, so those columns can be copied back at once.
//
// Page-locked host buffers take asynchronous copies issued from the calling
// thread. A copy to or from pageable memory returns only once the driver has
// taken the data (to the device) or delivered it (to the host), so issued from
// the calling thread it would hold back the launches behind it: the QR would
// wait for each chunk of Q to reach the host. For a pageable X the copies are
// issued by two worker threads instead (uploader, downloader) on the same copy
// streams; need() then waits on the host until the uploader has issued the
// chunk's copy and recorded its event, and final() hands the downloader an
// event recorded on the compute stream.
// ---------------------------------------------------------------------------
struct HostLink {
    double* hX = nullptr;   // caller's X (host), ld ldh
    i64 ldh = 0, m = 0;
    int n = 0, chunk = 1;
    double* dX = nullptr;   // device copy, ld m
    cudaStream_t cin = nullptr, cout = nullptr;
    bool pageable = false;           // hX is not page-locked: copies go through the worker threads
    cudaEvent_t x_done = nullptr;    // recorded on cin after the last chunk of X (if set)
    std::vector<cudaEvent_t> ev_in;  // one per chunk of X, recorded on cin after its copy
    std::vector<cudaEvent_t> ev_out; // final() events (pageable path)
    cudaEvent_t ev_fin = nullptr;
    int waited = 0, out_done = 0;
    std::atomic<int> err{0};
    int dev = 0;

    // Page-locked staging slots for a pageable X (null: the driver's own path).
    HostStage* stage = nullptr;
    std::vector<cudaEvent_t> up_ev, dn_ev;   // slot i's last copy engine transfer
    std::vector<char> up_used;
    int up_next = 0;

    // Worker threads (pageable path).
    struct Req { cudaEvent_t ev; int c0, c1; };
    std::thread up, down;
    std::mutex mu;
    std::condition_variable cv;
    int issued_in = 0;               // chunks whose copy is issued and event recorded
    std::vector<Req> reqs;           // final() requests not yet taken by the downloader
    bool closing = false;

    cudaError_t copy(double* dst, i64 ldd, const double* src, i64 lds, int c0, int nc, cudaMemcpyKind kind,
                     cudaStream_t s) {
        const size_t w = (size_t)m * sizeof(double);
        if (ldd == m && lds == m)
            return cudaMemcpyAsync(dst + (i64)c0 * ldd, src + (i64)c0 * lds, w * nc, kind, s);
        return cudaMemcpy2DAsync(dst + (i64)c0 * ldd, (size_t)ldd * sizeof(double), src + (i64)c0 * lds,
                                 (size_t)lds * sizeof(double), w, (size_t)nc, kind, s);
    }
    void fail(int e) {
        int z = 0;
        err.compare_exchange_strong(z, e);
    }
    // Contiguous pieces of columns [c0, c0 + nc) of X, at most one slot each:
    // f(host pointer, device pointer, bytes) in column order.
    template <class F>
    int for_pieces(int c0, int nc, size_t max_bytes, F f) {
        const size_t col = (size_t)m * sizeof(double);
        auto split = [&](char* h, char* d, size_t bytes) -> int {
            for (size_t off = 0; off < bytes; off += max_bytes) {
                const int e = f(h + off, d + off, std::min(max_bytes, bytes - off));
                if (e) return e;
            }
            return 0;
        };
        if (ldh == m)
            return split(reinterpret_cast<char*>(hX + (i64)c0 * m), reinterpret_cast<char*>(dX + (i64)c0 * m),
                         col * (size_t)nc);
        for (int c = c0; c < c0 + nc; ++c) {
            const int e = split(reinterpret_cast<char*>(hX + (i64)c * ldh), reinterpret_cast<char*>(dX + (i64)c * m),
                                col);
            if (e) return e;
        }
        return 0;
    }
    // Issue chunk k of X and record its event (either thread). Through the
    // staging slots: host threads copy a piece into a free slot while the copy
    // engine moves the previous ones.
    int put_chunk(int k) {
        const int c0 = k * chunk;
        const int nc = n - c0 < chunk ? n - c0 : chunk;
        int e = 0;
        if (stage) {
            e = for_pieces(c0, nc, stage->slot_bytes, [&](char* h, char* d, size_t bytes) -> int {
                const int sl = up_next++ % (int)stage->up.size();
                if (up_used[sl]) {
                    const int ee = (int)cudaEventSynchronize(up_ev[sl]);
                    if (ee) return ee;
                }
                stage->pool->copy(stage->up[sl], h, bytes);
                int ee = (int)cudaMemcpyAsync(d, stage->up[sl], bytes, cudaMemcpyHostToDevice, cin);
                if (!ee) ee = (int)cudaEventRecord(up_ev[sl], cin);
                up_used[sl] = 1;
                return ee;
            });
        } else {
            e = (int)copy(dX, m, hX, ldh, c0, nc, cudaMemcpyHostToDevice, cin);
        }
        if (!e) e = (int)cudaEventRecord(ev_in[k], cin);
        return e;
    }
    // Q columns [c0, c1) to the host through the download slots, after event ev on
    // the compute stream. In flight: (slot, host destination, bytes) whose copy
    // engine transfer is issued; the host copy out of a slot waits for it.
    struct Pending { int slot; char* h; size_t bytes; };
    std::deque<Pending> dn_fifo;
    int dn_next = 0;
    int drain_one() {
        const Pending q = dn_fifo.front();
        dn_fifo.pop_front();
        const int e = (int)cudaEventSynchronize(dn_ev[q.slot]);
        if (!e && !err) stage->pool->copy(q.h, stage->down[q.slot], q.bytes);
        return e;
    }
    int get_cols_staged(const Req& r) {
        int e = (int)cudaStreamWaitEvent(cout, r.ev, 0);
        if (e) return e;
        return for_pieces(r.c0, r.c1 - r.c0, stage->slot_bytes, [&](char* h, char* d, size_t bytes) -> int {
            const int sl = dn_next++ % (int)stage->down.size();
            if ((int)dn_fifo.size() == (int)stage->down.size()) {   // the oldest holds this slot
                const int ee = drain_one();
                if (ee) return ee;
            }
            int ee = (int)cudaMemcpyAsync(stage->down[sl], d, bytes, cudaMemcpyDeviceToHost, cout);
            if (!ee) ee = (int)cudaEventRecord(dn_ev[sl], cout);
            if (!ee) dn_fifo.push_back(Pending{sl, h, bytes});
            return ee;
        });
    }
    // Enqueue every H2D chunk on cin (after `st` reaches this point).
    void start(cudaStream_t st) {
        (void)cudaGetDevice(&dev);
        cudaEvent_t e0 = nullptr;
        int e = (int)cudaEventCreateWithFlags(&e0, cudaEventDisableTiming);
        if (e) { fail(e); return; }
        cudaEventRecord(e0, st);
        cudaStreamWaitEvent(cin, e0, 0);
        cudaStreamWaitEvent(cout, e0, 0);
        cudaEventDestroy(e0);
        if ((e = (int)cudaEventCreateWithFlags(&ev_fin, cudaEventDisableTiming))) { fail(e); return; }
        const int nchunks = (n + chunk - 1) / chunk;
        for (int k = 0; k < nchunks; ++k) {
            cudaEvent_t ek = nullptr;
            if ((e = (int)cudaEventCreateWithFlags(&ek, cudaEventDisableTiming))) { fail(e); return; }
            ev_in.push_back(ek);
        }
        if (pageable) stage = host_stage();
        if (stage) {
            for (size_t i = 0; i < stage->up.size() + stage->down.size(); ++i) {
                cudaEvent_t ek = nullptr;
                if ((e = (int)cudaEventCreateWithFlags(&ek, cudaEventDisableTiming))) { fail(e); return; }
                (i < stage->up.size() ? up_ev : dn_ev).push_back(ek);
            }
            up_used.assign(stage->up.size(), 0);
        }
        if (!pageable) {
            for (int k = 0; k < nchunks && !err; ++k)
                if ((e = put_chunk(k))) fail(e);
            if (!err && x_done && (e = (int)cudaEventRecord(x_done, cin))) fail(e);
            issued_in = nchunks;
            return;
        }
        up = std::thread([this, nchunks] {
            int e = (int)cudaSetDevice(dev);
            for (int k = 0; k < nchunks; ++k) {
                if (!e && !err) e = put_chunk(k);
                if (e) fail(e);
                std::lock_guard<std::mutex> lock(mu);
                issued_in = k + 1;
                cv.notify_all();
            }
            if (!err && x_done && (e = (int)cudaEventRecord(x_done, cin))) fail(e);
        });
    }
    void need(cudaStream_t st, int c_end) {
        while (!err && waited < c_end && waited < n) {
            const int k = waited / chunk;
            if (pageable) {
                std::unique_lock<std::mutex> lock(mu);
                cv.wait(lock, [&] { return issued_in > k || err != 0; });
                if (err) break;
            }
            const int e = (int)cudaStreamWaitEvent(st, ev_in[k], 0);
            if (e) fail(e);
            waited = (k + 1) * chunk;
        }
    }
    void final(cudaStream_t st, int c_end) {
        if (err || c_end <= out_done) return;
        if (c_end > n) c_end = n;
        int e = 0;
        if (!pageable) {
            e = (int)cudaEventRecord(ev_fin, st);
            if (!e) e = (int)cudaStreamWaitEvent(cout, ev_fin, 0);
            if (!e) e = (int)copy(hX, ldh, dX, m, out_done, c_end - out_done, cudaMemcpyDeviceToHost, cout);
            if (e) fail(e);
            out_done = c_end;
            return;
        }
        cudaEvent_t ev = nullptr;
        e = (int)cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (!e) e = (int)cudaEventRecord(ev, st);
        if (e) {
            if (ev) cudaEventDestroy(ev);
            fail(e);
            return;
        }
        {
            std::lock_guard<std::mutex> lock(mu);
            ev_out.push_back(ev);
            reqs.push_back(Req{ev, out_done, c_end});
            cv.notify_all();
        }
        out_done = c_end;
        if (!down.joinable()) {
            down = std::thread([this] {
                int e = (int)cudaSetDevice(dev);
                if (e) fail(e);
                for (;;) {
                    Req r;
                    {
                        std::unique_lock<std::mutex> lock(mu);
                        if (reqs.empty() && !closing && stage && !dn_fifo.empty()) {
                            // Nothing new to issue: move landed columns out meanwhile.
                            lock.unlock();
                            const int e2 = drain_one();
                            if (e2) fail(e2);
                            continue;
                        }
                        cv.wait(lock, [&] { return !reqs.empty() || closing; });
                        if (reqs.empty()) {   // closing: the last columns out of the slots
                            lock.unlock();
                            while (stage && !dn_fifo.empty()) {
                                const int e2 = drain_one();
                                if (e2) fail(e2);
                            }
                            return;
                        }
                        r = reqs.front();
                        reqs.erase(reqs.begin());
                    }
                    if (err) continue;   // drain the queue without copying
                    if (stage) {
                        e = get_cols_staged(r);
                    } else {
                        e = (int)cudaStreamWaitEvent(cout, r.ev, 0);
                        if (!e) e = (int)copy(hX, ldh, dX, m, r.c0, r.c1 - r.c0, cudaMemcpyDeviceToHost, cout);
                    }
                    if (e) fail(e);
                }
            });
        }
    }
    // The last columns of Q and all of R, enqueued before the caller reads the run's
    // status, so that they do not wait for that read. R goes to the staging buffer
    // hR (page-locked) on the compute stream; done (if set) is recorded there when
    // the QR's kernels have finished, before R's copy.
    double* hR = nullptr;
    const double* dR = nullptr;
    size_t rbytes = 0;
    cudaEvent_t done = nullptr;
    bool finished = false;
    void finish(cudaStream_t st) {
        final(st, n);
        int e = 0;
        if (!err && done && (e = (int)cudaEventRecord(done, st))) fail(e);
        if (!err && (e = (int)cudaMemcpyAsync(hR, dR, rbytes, cudaMemcpyDeviceToHost, st))) fail(e);
        finished = !err;
    }
    // Waits for the worker threads: after it returns every copy of this run is
    // issued (and, for pageable memory, complete).
    void join() {
        {
            std::lock_guard<std::mutex> lock(mu);
            closing = true;
            cv.notify_all();
        }
        if (up.joinable()) up.join();
        if (down.joinable()) down.join();
    }
    void release() {
        join();
        for (cudaEvent_t e : ev_in) cudaEventDestroy(e);
        ev_in.clear();
        for (cudaEvent_t e : ev_out) cudaEventDestroy(e);
        ev_out.clear();
        for (cudaEvent_t e : up_ev) cudaEventDestroy(e);
        up_ev.clear();
        for (cudaEvent_t e : dn_ev) cudaEventDestroy(e);
        dn_ev.clear();
        if (ev_fin) cudaEventDestroy(ev_fin);
        ev_fin = nullptr;
    }
    ~HostLink() { join(); }
};

// ---------------------------------------------------------------------------
// Row-sharded runs: this rank holds rows [row0, row0 + msub) of X. The Gram's
// partial sums are taken over chunks of kShardRows rows, aligned globally; every
// rank gathers all ranks' chunk partials (in rank order, padded to maxc chunks
// with zeros) and sums them in global chunk order, so every rank gets the Gram a
// one-rank run of the same chunking gets, bit for bit. TSQR gathers its leaf
// level's R factors the same way (TsqrShard).
// ---------------------------------------------------------------------------
constexpr i64 kShardRows = ORTH_GB300_SHARD_ROWS;

struct Shard {
    const orth_gb300_comm* comm = nullptr;
    int rank = 0, size = 1;
    i64 row0 = 0, msub = 0, m = 0;
    i64 maxc = 0;                    // most Gram chunks on any rank
    std::vector<i64> t0, nt;         // TSQR leaf tiles of each rank
    i64 T = 0, maxt = 0;
    DevBuf part, all, tmine, tall;   // exchange buffers
};

// The reference's 1-D block-row partition (SRC/orth.c:69-76, TESTS/test_orth.c:
// 24-32) applied to chunks of kShardRows rows: size ranks share ceil(m / rows)
// chunks, each rank m/size of them and the last (m mod size) ranks one more.
void shard_chunks(i64 m, int size, int rank, i64* c_begin, i64* c_count) {
    const i64 nch = ceil_div(m, kShardRows);
    const i64 cpr = nch / size, res = nch - cpr * size;
    if (res >= size - rank) {
        *c_begin = rank * cpr + res - size + rank;
        *c_count = cpr + 1;
    } else {
        *c_begin = rank * cpr;
        *c_count = cpr;
    }
}

void shard_rows(i64 m, int size, int rank, i64* row0, i64* msub) {
    i64 cb = 0, cc = 0;
    shard_chunks(m, size, rank, &cb, &cc);
    *row0 = cb * kShardRows;
    const i64 end = (cb + cc) * kShardRows < m ? (cb + cc) * kShardRows : m;
    *msub = end > *row0 ? end - *row0 : 0;
}

int comm_gather(void* ctx, const double* mine, double* all, long long count, cudaStream_t st) {
    const orth_gb300_comm* c = static_cast<const orth_gb300_comm*>(ctx);
    return c->allgather(c->ctx, mine, all, count, (void*)st) ? (int)cudaErrorUnknown : 0;
}

// ---------------------------------------------------------------------------
// Per-call engine: the primitives every variant is written in.
// ---------------------------------------------------------------------------
struct Engine {
    double* X;
    i64 ld;
    i64 m;
    int n, s;
    double* R;
    int ldR;
    int precision;
    cudaStream_t st;
    Small w;
    int* status;
    int err = 0;
    HostLink* link = nullptr;   // host-buffer runs only
    Shard* shard = nullptr;     // row-sharded runs only (FP64)

    // C (na x nb, ldc) = X[:, a0:a0+na]^T X[:, b0:b0+nb] in FP64: one deterministic
    // reduction, over all ranks in a row-sharded run.
    void gram_fp64(int a0, int na, int b0, int nb, double* C, int ldc) {
        if (err) return;
        if (!shard) {
            const int chunks = gram_chunks_fp64(m, na, nb, g_ctx.num_sms);
            err = launch_gram_fp64(X, ld, m, a0, na, b0, nb, C, ldc, scr().part.as<double>(), chunks, st);
            return;
        }
        Shard& sh = *shard;
        const i64 blk = (i64)na * nb;
        const i64 mine = ceil_div(m, kShardRows);
        double* part = sh.part.as<double>();
        err = launch_gram_partials_fp64(X, ld, m, a0, na, b0, nb, part, kShardRows, st);
        if (!err && mine < sh.maxc) err = zero_async(part + mine * blk, (size_t)((sh.maxc - mine) * blk) * sizeof(double), st);
        if (!err) err = comm_gather((void*)sh.comm, part, sh.all.as<double>(), sh.maxc * blk, st);
        if (!err) err = launch_gram_reduce(sh.all.as<double>(), (int)(sh.size * sh.maxc), na, nb, C, ldc, st);
    }

    // X columns [0, c_end) must be on the device; columns [0, c_fin) are final.
    void host_sync(int c_end, int c_fin) {
        if (!link || err) return;
        link->need(st, c_end);
        if (c_fin >= 0) link->final(st, c_fin);
        if (link->err) err = link->err;
    }

    // C (na x nb, ld na) = X[:, 0:na]^T X[:, b0:b0+nb]: one synchronization.
    void gram(int na, int b0, int nb, double* C) {
        if (err || na <= 0 || nb <= 0) return;
        host_sync(na > b0 + nb ? na : b0 + nb, -1);
        if (is_split(precision)) {
            ProfScope pslice(4, st, 0.0, 0.0);
            err = split_prepare(na > b0 + nb ? na : b0 + nb, st);
            if (err) return;
        }
        const double eb = is_split(precision) ? 2.0 * split_digits() : 8.0;
        ProfScope ps(0, st, 2.0 * m * na * nb, 8.0 * m * (na + nb), eb * m * (na + nb));
        if (is_split(precision)) {
            err = launch_gram_split(X, ld, m, na, b0, nb, C, na, scr().split.as<char>(),
                                    scr().split.bytes, g_ctx.num_sms, st);
            return;
        }
        gram_fp64(0, na, b0, nb, C, na);
    }
    // X[:, c0:c0+nc] = (X[:, c0:c0+nc] - X[:, 0:K] S) T^{-1}
    void update(int K, int c0, int nc, const double* S, int lds, const double* T, int ldt) {
        if (err || nc <= 0) return;
        host_sync(K > c0 + nc ? K : c0 + nc, c0);
        if (is_split(precision)) {
            ProfScope pslice(4, st, 0.0, 0.0);
            err = split_prepare(K + nc, st);
            if (err) return;
        }
        const double traffic = is_split(precision) ? 2.0 * split_digits() * m * (K + nc) + 8.0 * m * nc
                                                   : 8.0 * m * (K + 2.0 * nc);
        ProfScope ps(1, st, 2.0 * m * K * nc + (T ? (double)m * nc * nc : 0.0), 8.0 * m * (K + 2.0 * nc), traffic);
        if (is_split(precision)) {
            err = launch_update_split(X, ld, m, K, c0, nc, S, lds, T, ldt, scr().split.as<char>(),
                                      scr().split.bytes, g_ctx.num_sms, st);
            return;
        }
        err = launch_update_fp64(X, ld, m, 0, K, c0, nc, S, lds, T, ldt, st);
    }
    // Split modes: Q_k and U_{k+1} of the lagged variants in one tensor-core pass.
    void fused_update(int K, int nz, const double* G, int ldg, const double* Ty, const double* Sp,
                      const double* Ts) {
        if (err) return;
        host_sync(K + s + nz, K);
        {
            ProfScope pslice(4, st, 0.0, 0.0);
            err = split_prepare(K + s + nz, st);
            if (err) return;
        }
        const double traffic = 2.0 * split_digits() * m * (K + s + nz) + 8.0 * m * (s + nz);
        ProfScope ps(1, st, 2.0 * m * K * (s + nz) + (double)m * (s * s + nz * nz),
                     8.0 * m * (K + s + nz) + 8.0 * m * (s + nz), traffic);
        err = launch_fused_update_split(X, ld, m, K, s, nz, G, ldg, Ty, Sp, K + s, Ts, g_ctx.num_sms, st);
    }
    void pyth_chol(const double* Om, int ldom, const double* A, int lda, int k, int nz, double* T,
                   int step) {
        if (err) return;
        ProfScope ps(2, st, 0.0, 0.0);
        err = launch_pyth_chol(Om, ldom, A, lda, k, nz, T, nz, status, step, st);
    }
    void scol(const double* G, int ldg, int mZ, int nZ, const double* Yd, double* Scol) {
        if (err) return;
        ProfScope ps(2, st, 0.0, 0.0);
        err = launch_scol(G, ldg, mZ, s, nZ, Yd, s, Scol, mZ + s, st);
    }
    void rblock(int c0, int K, int ny, const double* A, int lda, const double* B, int ldb,
                const double* Sd, const double* Yd, int mode) {
        if (err) return;
        ProfScope ps(2, st, 0.0, 0.0);
        err = launch_rblock(R, ldR, c0, K, ny, A, lda, B, ldb, Sd, ny, Yd, ny, mode, st);
    }
    // Explicit TSQR of X[:, c0:c0+nc]; R into (Rout, ldr).
    void tsqr(int c0, int nc, double* Rout, int ldr) {
        if (err) return;
        host_sync(c0 + nc, c0);
        ProfScope ps(3, st, 6.0 * m * nc * nc, 8.0 * m * nc * 3.0);
        if (shard) {
            TsqrShard ts;
            ts.rank = shard->rank; ts.size = shard->size; ts.T = shard->T; ts.maxt = shard->maxt;
            ts.t0 = shard->t0.data(); ts.nt = shard->nt.data();
            ts.mine = shard->tmine.as<double>(); ts.all = shard->tall.as<double>();
            ts.gather = comm_gather; ts.ctx = (void*)shard->comm;
            err = launch_tsqr_sharded(X, ld, m, c0, nc, Rout, ldr, scr().tsqr.as<double>(), ts, st);
            return;
        }
        err = launch_tsqr(X, ld, m, c0, nc, Rout, ldr, scr().tsqr.as<double>(), st);
        if (is_split(precision)) split_mark_stale(c0, nc);
    }
    // CholQR2 of X[:, c0:c0+nc] (FP64 in every precision): twice G = V^T V (one
    // deterministic reduction), T = chol(G), V = V T^{-1}; then R = R2 R1 into
    // (Rout, ldr). A Cholesky breakdown is recorded as block step `step`.
    void cholqr2(int c0, int nc, double* Rout, int ldr, int step) {
        if (err) return;
        host_sync(c0 + nc, c0);
        ProfScope ps(3, st, 2.0 * (2.0 * m * nc * nc + (double)m * nc * nc), 8.0 * m * nc * 6.0);
        double* G = w.Cq;
        double* R1 = G + (i64)s * s;
        double* R2 = R1 + (i64)s * s;
        for (int pass = 0; pass < 2 && !err; ++pass) {
            double* T = pass ? R2 : R1;
            gram_fp64(c0, nc, c0, nc, G, nc);
            if (!err) err = launch_pyth_chol(G, nc, nullptr, 0, 0, nc, T, nc, status, step, st);
            if (!err) err = launch_update_fp64(X, ld, m, 0, 0, c0, nc, nullptr, 0, T, nc, st);
        }
        if (!err) err = launch_rblock(Rout, ldr, 0, 0, nc, nullptr, 0, nullptr, 0, R1, nc, R2, nc, 0, st);
        if (is_split(precision)) split_mark_stale(c0, nc);
    }
    // IntraOrtho of the panel X[:, c0:c0+nc] (where the reference calls TSQR).
    void intra(int c0, int nc, double* Rout, int ldr, int step) {
        if (intra_mode() == ORTH_GB300_INTRA_CHOLQR2) cholqr2(c0, nc, Rout, ldr, step);
        else tsqr(c0, nc, Rout, ldr);
    }
};

int nblocks_after_first(int n, int s) { return (n - s + s - 1) / s; }  // p = ceil((n-s0)/s)

// --------------------------- C1 bcgsi2P1s ----------------------------------
// SRC/orth.c:48-222. One synchronization per block step.
void run_p1s(Engine& e) {
    const int s = e.s, n = e.n, s0 = s;
    const int p = nblocks_after_first(n, s);
    Small& w = e.w;
    e.intra(0, s0, e.R, e.ldR, 1);                                   // :105-107
    // First step (:110-147).
    double* W = w.G2;                                                // 2s x s, ld 2s
    e.gram(2 * s, s0, s, W);                                         // :111-114
    e.pyth_chol(W + s0, 2 * s, W, 2 * s, s0, s, w.Sd, 1);            // :115-119
    e.update(s0, s0, s, W, 2 * s, w.Sd, s);                          // :121-124  U2
    int nZ = n - s - s0 < s ? n - s - s0 : s;                        // :125
    int na = 2 * s + nZ, nb = s + nZ;
    double* G = w.G1;
    e.gram(na, s0, nb, G);                                           // :127-133
    e.pyth_chol(G + s0, na, G, na, s0, s, w.Yd, 1);                  // :134-137
    e.update(s0, s0, s, G, na, w.Yd, s);                             // :139-142  Q2
    e.rblock(s0, s0, s, W, 2 * s, G, na, w.Sd, w.Yd, 0);             // :144-147
    int ldg = na;
    int mZ = s0;
    for (int i = 1; i < p; ++i) {                                    // :152-218
        const int mScol = mZ + s;
        e.scol(G, ldg, mZ, nZ, w.Yd, w.Scol);                        // :155-159
        // Omega_k = X_k^T X_k from the last synchronization (:160-163).
        e.pyth_chol(G + mScol + (i64)s * ldg, ldg, w.Scol, mScol, mScol, nZ, w.Sd, i + 1);  // :160-171
        e.update(mScol, mScol, nZ, w.Scol, mScol, w.Sd, nZ);         // :173-176  U_k
        int nY, nZn;
        if (i < p - 1) {                                             // :177-190
            nZn = n - (i + 1) * s - s0 < s ? n - (i + 1) * s - s0 : s;
            na = mScol + s + nZn;
            nb = s + nZn;
            nY = s;
        } else {                                                     // :191-199
            nZn = nZ;
            na = mScol + nZ;
            nb = nZ;
            nY = nZ;
        }
        e.gram(na, mScol, nb, G);                                    // the one sync
        ldg = na;
        e.pyth_chol(G + mScol, ldg, G, ldg, mScol, nY, w.Yd, i + 1); // :200-204
        e.update(mScol, mScol, nY, G, ldg, w.Yd, nY);                // :206-209  Q_k
        e.rblock(mScol, mScol, nY, w.Scol, mScol, G, ldg, w.Sd, w.Yd, 0);  // :211-215
        mZ += s;
        nZ = nZn;
    }
}

// Split-precision form of C1/C2: the same operations in the same order, except
// that the finalization of Q_k (after the step's single synchronization) and the
// first pass of block k+1 run as one tensor-core pass over Q (Engine::fused_update),
// so Q is read once per block step. pyth = true: BCGSI+P-1S (scaled first pass,
// SRC/orth.c:152-218); false: BCGSI+A-1S (unscaled first pass, SRC/orth.c:307-363).
void run_lagged_fused(Engine& e, bool pyth) {
    const int s = e.s, n = e.n, s0 = s;
    const int p = nblocks_after_first(n, s);
    Small& w = e.w;
    const int mode = pyth ? 0 : 1;
    e.intra(0, s0, e.R, e.ldR, 1);
    double* W = w.G2;
    int nZ = n - s - s0 < s ? n - s - s0 : s;
    int na, nb;
    double* G = w.G1;
    if (pyth) {
        e.gram(2 * s, s0, s, W);                                     // :111-114
        e.pyth_chol(W + s0, 2 * s, W, 2 * s, s0, s, w.Sd, 1);        // :115-119
        e.update(s0, s0, s, W, 2 * s, w.Sd, s);                      // :121-124
    } else {
        e.gram(s0, s0, s, w.S0);                                     // :275-278
        e.update(s0, s0, s, w.S0, s0, nullptr, 0);                   // :280-281
    }
    na = 2 * s + (pyth ? nZ : 0);
    nb = s + nZ;
    e.gram(pyth ? na : 2 * s, s0, nb, G);                            // :127-133 / :284-287
    int ldg = pyth ? na : 2 * s;
    e.pyth_chol(G + s0, ldg, G, ldg, s0, s, w.Yd, 1);                // :134-137 / :288-291
    if (pyth) e.rblock(s0, s0, s, W, 2 * s, G, ldg, w.Sd, w.Yd, 0);  // :144-147
    else e.rblock(s0, s0, s, w.S0, s0, G, ldg, nullptr, w.Yd, 1);    // :298-302
    if (p <= 1) {
        e.update(s0, s0, s, G, ldg, w.Yd, s);                        // Q_2 alone
        return;
    }
    int mZ = s0;
    {
        const int mScolN = mZ + s;
        e.scol(G, ldg, mZ, nZ, w.Yd, w.Scol);                        // :155-159
        if (pyth) e.pyth_chol(G + mScolN + (i64)s * ldg, ldg, w.Scol, mScolN, mScolN, nZ, w.Sd, 2);
        e.fused_update(s0, nZ, G, ldg, w.Yd, w.Scol, pyth ? w.Sd : nullptr);
    }
    for (int i = 1; i < p; ++i) {
        const int mScol = mZ + s;
        int nY, nZn;
        if (i < p - 1) {
            nZn = n - (i + 1) * s - s0 < s ? n - (i + 1) * s - s0 : s;
            na = mScol + s + (pyth ? nZn : 0);
            nb = s + nZn;
            nY = s;
        } else {
            nZn = nZ;
            na = mScol + nZ;
            nb = nZ;
            nY = nZ;
        }
        e.gram(na, mScol, nb, G);                                    // the one synchronization
        ldg = na;
        e.pyth_chol(G + mScol, ldg, G, ldg, mScol, nY, w.Yd, i + 1);
        e.rblock(mScol, mScol, nY, w.Scol, mScol, G, ldg, pyth ? w.Sd : nullptr, w.Yd, mode);
        if (i < p - 1) {
            const int mZn = mZ + s, mScolN = mZn + s;
            e.scol(G, ldg, mZn, nZn, w.Yd, w.Scol);
            if (pyth) e.pyth_chol(G + mScolN + (i64)s * ldg, ldg, w.Scol, mScolN, mScolN, nZn, w.Sd, i + 2);
            e.fused_update(mScol, nZn, G, ldg, w.Yd, w.Scol, pyth ? w.Sd : nullptr);
        } else {
            e.update(mScol, mScol, nY, G, ldg, w.Yd, nY);            // last Q_k
        }
        mZ += s;
        nZ = nZn;
    }
}

// --------------------------- C2 bcgsi21s -----------------------------------
// SRC/orth.c:224-367. One synchronization per block step; the first pass is an
// unnormalized projection.
void run_21s(Engine& e) {
    const int s = e.s, n = e.n, s0 = s;
    const int p = nblocks_after_first(n, s);
    Small& w = e.w;
    e.intra(0, s0, e.R, e.ldR, 1);                                   // :269-271
    e.gram(s0, s0, s, w.S0);                                         // :275-278
    e.update(s0, s0, s, w.S0, s0, nullptr, 0);                       // :280-281
    int nZ = n - s - s0 < s ? n - s - s0 : s;                        // :282
    int na = 2 * s, nb = s + nZ;
    double* G = w.G1;
    e.gram(na, s0, nb, G);                                           // :284-287
    e.pyth_chol(G + s0, na, G, na, s0, s, w.Yd, 1);                  // :288-291
    e.update(s0, s0, s, G, na, w.Yd, s);                             // :293-296
    e.rblock(s0, s0, s, w.S0, s0, G, na, nullptr, w.Yd, 1);          // :298-302
    int ldg = na, mZ = s0;
    for (int i = 1; i < p; ++i) {
        const int mScol = mZ + s;
        e.scol(G, ldg, mZ, nZ, w.Yd, w.Scol);                        // :310-314
        e.update(mScol, mScol, nZ, w.Scol, mScol, nullptr, 0);       // :323-324
        int nY, nZn;
        if (i < p - 1) {                                             // :325-335
            nZn = n - (i + 1) * s - s0 < s ? n - (i + 1) * s - s0 : s;
            na = mScol + s;
            nb = s + nZn;
            nY = s;
        } else {                                                     // :336-344
            nZn = nZ;
            na = mScol + nZ;
            nb = nZ;
            nY = nZ;
        }
        e.gram(na, mScol, nb, G);
        ldg = na;
        e.pyth_chol(G + mScol, ldg, G, ldg, mScol, nY, w.Yd, i + 1); // :345-349
        e.update(mScol, mScol, nY, G, ldg, w.Yd, nY);                // :351-354
        e.rblock(mScol, mScol, nY, w.Scol, mScol, G, ldg, nullptr, w.Yd, 1);  // :356-360
        mZ += s;
        nZ = nZn;
    }
}

// --------------------------- C3 bcgspipi2 ----------------------------------
// SRC/orth.c:369-462. Two synchronizations per block step.
void run_pipi(Engine& e) {
    const int s = e.s, n = e.n, s0 = s;
    const int p = nblocks_after_first(n, s);
    Small& w = e.w;
    e.intra(0, s0, e.R, e.ldR, 1);                                   // :411-413
    int mScol = s0;
    for (int i = 0; i < p; ++i) {
        const int nZ = n - i * s - s0 < s ? n - i * s - s0 : s;       // :419
        const int na = mScol + nZ;
        e.gram(na, mScol, nZ, w.G1);                                 // :421-424
        e.pyth_chol(w.G1 + mScol, na, w.G1, na, mScol, nZ, w.Sd, i + 1);  // :425-429
        e.update(mScol, mScol, nZ, w.G1, na, w.Sd, nZ);              // :431-434
        e.gram(na, mScol, nZ, w.G2);                                 // :435-438
        e.pyth_chol(w.G2 + mScol, na, w.G2, na, mScol, nZ, w.Yd, i + 1);  // :440-444
        e.update(mScol, mScol, nZ, w.G2, na, w.Yd, nZ);              // :446-449
        e.rblock(mScol, mScol, nZ, w.G1, na, w.G2, na, w.Sd, w.Yd, 0);    // :451-455
        mScol += s;
    }
}

// --------------------------- C4 bcgsi2 -------------------------------------
// SRC/orth.c:464-548. Two synchronizations and two TSQRs per block step.
void run_bcgsi2(Engine& e) {
    const int s = e.s, n = e.n, s0 = s;
    const int p = nblocks_after_first(n, s);
    Small& w = e.w;
    e.intra(0, s0, e.R, e.ldR, 1);                                   // :503-505
    int mScol = s0;
    for (int i = 0; i < p; ++i) {
        const int nZ = n - i * s - s0 < s ? n - i * s - s0 : s;       // :511
        e.gram(mScol, mScol, nZ, w.G1);                              // :512-515
        e.update(mScol, mScol, nZ, w.G1, mScol, nullptr, 0);         // :518-519
        e.intra(mScol, nZ, w.Sd, nZ, i + 1);                         // :520-523
        e.gram(mScol, mScol, nZ, w.G2);                              // :524-527
        e.update(mScol, mScol, nZ, w.G2, mScol, nullptr, 0);         // :530-531
        e.intra(mScol, nZ, w.Yd, nZ, i + 1);                         // :532-535
        e.rblock(mScol, mScol, nZ, w.G1, mScol, w.G2, mScol, w.Sd, w.Yd, 0);  // :537-541
        mScol += s;
    }
}

// --------------------------- C5 bcgsi2P2s ----------------------------------
// SRC/orth.c:550-697. TSQR first pass, one Pythagorean synchronization.
void run_p2s(Engine& e) {
    const int s = e.s, n = e.n, s0 = s;
    const int p = nblocks_after_first(n, s);
    Small& w = e.w;
    e.intra(0, s0, e.R, e.ldR, 1);                                   // :599-601
    e.gram(s0, s0, s, w.S0);                                         // :605-608
    e.update(s0, s0, s, w.S0, s0, nullptr, 0);                       // :610-611
    e.intra(s0, s, w.Sd, s, 1);                                      // :612-614
    int nZ = n - s - s0 < s ? n - s - s0 : s;                        // :615
    int na = 2 * s, nb = s + nZ;
    double* G = w.G1;
    e.gram(na, s0, nb, G);                                           // :617-620
    e.pyth_chol(G + s0, na, G, na, s0, s, w.Yd, 1);                  // :621-624
    e.update(s0, s0, s, G, na, w.Yd, s);                             // :625-628
    e.rblock(s0, s0, s, w.S0, s0, G, na, w.Sd, w.Yd, 0);             // :609,:630-633
    int ldg = na, mZ = s0;
    for (int i = 1; i < p; ++i) {
        const int mScol = mZ + s;
        e.scol(G, ldg, mZ, nZ, w.Yd, w.Scol);                        // :641-645
        e.update(mScol, mScol, nZ, w.Scol, mScol, nullptr, 0);       // :647-648
        e.intra(mScol, nZ, w.Sd, nZ, i + 1);                         // :649-652
        int nY, nZn;
        if (i < p - 1) {                                             // :653-666
            nZn = n - (i + 1) * s - s0 < s ? n - (i + 1) * s - s0 : s;
            na = mScol + s;          // X_{k+1}^T X_{k+1} (:660-662) is never used; skipped
            nb = s + nZn;
            nY = s;
        } else {                                                     // :667-675
            nZn = nZ;
            na = mScol + nZ;
            nb = nZ;
            nY = nZ;
        }
        e.gram(na, mScol, nb, G);
        ldg = na;
        e.pyth_chol(G + mScol, ldg, G, ldg, mScol, nY, w.Yd, i + 1); // :676-680
        e.update(mScol, mScol, nY, G, ldg, w.Yd, nY);                // :681-684
        e.rblock(mScol, mScol, nY, w.Scol, mScol, G, ldg, w.Sd, w.Yd, 0);  // :686-690
        mZ += s;
        nZ = nZn;
    }
}

bool valid_args(int m, int n, int s, long long ldX, int ldR) {
    return m >= 1 && s >= 1 && s <= 64 && n >= 2 * s && ldX >= m && ldR >= n && (i64)m >= n;
}

int run_device(int variant, int m, int n, int s, double* dX, i64 ldX, double* dR, int ldR,
               int precision, cudaStream_t st, orth_gb300_status* out, HostLink* link = nullptr) {
    if (!valid_args(m, n, s, ldX, ldR)) return 2;
    if (variant < 0 || variant > 4) return 2;
    if (precision != ORTH_GB300_FP64 && !is_split(precision)) return 4;
    if (is_split(precision) && !split_supported(m, n, s)) return 4;
    int rc = reserve(m, n, s, precision);
    if (rc) {
        if (out) { std::memset(out, 0, sizeof(*out)); out->cuda_error = rc; }
        return 3;
    }
    const long long launches0 = g_launch_count;
    const long long reductions0 = g_reduce_count;
    Engine e{dX, (i64)ldX, (i64)m, n, s, dR, ldR, precision, st,
             carve_small(scr().small.as<double>(), n, s), scr().status.as<int>()};
    e.link = link;
    cudaError_t ce = (cudaError_t)zero_async(e.status, kStatusWords * sizeof(int), st);
    if (ce != cudaSuccess) e.err = (int)ce;
    if (!e.err && is_split(precision))
        e.err = split_begin(dX, ldX, m, n, s, split_digits_of(precision), scr().split.as<char>(), scr().split.bytes, g_ctx.num_sms, st);
    switch (variant) {
        case ORTH_GB300_BCGSI2P1S:
            if (is_split(precision)) run_lagged_fused(e, true); else run_p1s(e);
            break;
        case ORTH_GB300_BCGSI21S:
            if (is_split(precision)) run_lagged_fused(e, false); else run_21s(e);
            break;
        case ORTH_GB300_BCGSPIPI2: run_pipi(e); break;
        case ORTH_GB300_BCGSI2: run_bcgsi2(e); break;
        default: run_p2s(e); break;
    }
    g_last_launches = g_launch_count - launches0;
    g_last_reductions = g_reduce_count - reductions0;
    if (link && !e.err) {
        link->finish(st);
        if (link->err) e.err = link->err;
    }
    if (out) {
        std::memset(out, 0, sizeof(*out));
        int h[kStatusWords] = {0, 0, 0, 0};
        if (!e.err) {
            ce = cudaMemcpyAsync(h, e.status, sizeof(h), cudaMemcpyDeviceToHost, st);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
            if (ce != cudaSuccess) e.err = (int)ce;
        }
        out->breakdown_step = h[0];
        out->breakdown_info = h[1];
        out->timeout = h[2];
        if (!e.err && is_split(precision)) {
            int w = 0;
            int rc2 = split_error_word(&w, st);
            if (rc2) e.err = rc2;
            if (w) { out->timeout = w; e.err = (int)cudaErrorLaunchTimeout; }
        }
        out->cuda_error = e.err;
    }
    return e.err ? 3 : 0;
}

// Row-sharded run of one rank (FP64): this rank's rows of X (msub x n, ld ldX)
// and a full R (written on every rank, as the reference writes R on every rank).
int run_sharded(int variant, i64 m, int n, int s, double* dX, i64 ldX, double* dR, int ldR, cudaStream_t st,
                const orth_gb300_comm* comm, orth_gb300_status* out) {
    if (out) std::memset(out, 0, sizeof(*out));
    if (!comm || !comm->allgather || comm->size < 1 || comm->rank < 0 || comm->rank >= comm->size) return 2;
    if (variant < 0 || variant > 4 || s < 1 || s > 64 || n < 2 * s || ldR < n || m < n || !dX || !dR) return 2;
    if (ceil_div(m, kShardRows) < comm->size) return 2;   // every rank holds at least one chunk
    Shard sh;
    sh.comm = comm; sh.rank = comm->rank; sh.size = comm->size; sh.m = m;
    shard_rows(m, sh.size, sh.rank, &sh.row0, &sh.msub);
    if (ldX < sh.msub) return 2;
    const int TR = tsqr_tile_rows(s);
    sh.t0.resize(sh.size); sh.nt.resize(sh.size);
    for (int r = 0; r < sh.size; ++r) {
        i64 r0 = 0, ms = 0, cb = 0, cc = 0;
        shard_rows(m, sh.size, r, &r0, &ms);
        shard_chunks(m, sh.size, r, &cb, &cc);
        sh.t0[r] = r0 / TR;
        sh.nt[r] = ceil_div(ms, TR);
        if (cc > sh.maxc) sh.maxc = cc;
        if (sh.nt[r] > sh.maxt) sh.maxt = sh.nt[r];
    }
    sh.T = ceil_div(m, TR);
    int rc = init_ctx();
    if (!rc) rc = reserve(sh.msub, n, s, ORTH_GB300_FP64);
    const i64 blk = (i64)(n + s) * 2 * s;
    if (!rc) rc = sh.part.ensure((size_t)(sh.maxc * blk) * sizeof(double));
    if (!rc) rc = sh.all.ensure((size_t)(sh.size * sh.maxc * blk) * sizeof(double));
    if (!rc) rc = sh.tmine.ensure((size_t)(sh.maxt * s * s) * sizeof(double));
    if (!rc) rc = sh.tall.ensure((size_t)(sh.size * sh.maxt * s * s) * sizeof(double));
    if (!rc) rc = scr().tsqr.ensure((size_t)tsqr_workspace_doubles(m, s) * sizeof(double));
    if (rc) {
        if (out) out->cuda_error = rc;
        return 3;
    }
    const long long reductions0 = g_reduce_count;
    Engine e{dX, ldX, sh.msub, n, s, dR, ldR, ORTH_GB300_FP64, st,
             carve_small(scr().small.as<double>(), n, s), scr().status.as<int>()};
    e.shard = &sh;
    e.err = zero_async(e.status, kStatusWords * sizeof(int), st);
    switch (variant) {
        case ORTH_GB300_BCGSI2P1S: run_p1s(e); break;
        case ORTH_GB300_BCGSI21S: run_21s(e); break;
        case ORTH_GB300_BCGSPIPI2: run_pipi(e); break;
        case ORTH_GB300_BCGSI2: run_bcgsi2(e); break;
        default: run_p2s(e); break;
    }
    g_last_reductions = g_reduce_count - reductions0;
    int h[kStatusWords] = {0, 0, 0, 0};
    if (!e.err) {
        cudaError_t ce = cudaMemcpyAsync(h, e.status, sizeof(h), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) e.err = (int)ce;
    }
    if (out) {
        out->breakdown_step = h[0];
        out->breakdown_info = h[1];
        out->timeout = h[2];
        out->cuda_error = e.err;
    }
    // The exchange buffers are this call's: wait for the stream before they go.
    cudaStreamSynchronize(st);
    sh.part.release(); sh.all.release(); sh.tmine.release(); sh.tall.release();
    return e.err ? 3 : 0;
}

// Whether p is memory the GPU can address directly (device or managed memory).
bool is_device_pointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked host memory (cudaHostAlloc, cudaHostRegister, orth_gb300_host_alloc).
bool is_page_locked(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Copies what the reference writes into R (SRC/orth.c): for column j of block b,
// rows [0, end of block b); bcgsi21s writes only the upper triangle of its
// diagonal blocks after the first (SRC/orth.c:302,360 use dlacpy 'U').
cudaError_t write_back_r(int variant, int n, int s, const double* src, int lds, double* dst, int ldd,
                         cudaMemcpyKind kind) {
    for (int j = 0; j < n; ++j) {
        const int b = j / s;
        int rows = (b + 1) * s < n ? (b + 1) * s : n;
        if (variant == ORTH_GB300_BCGSI21S && b >= 1) rows = j + 1;
        cudaError_t ce = cudaMemcpy(dst + (size_t)j * ldd, src + (size_t)j * lds, (size_t)rows * sizeof(double), kind);
        if (ce != cudaSuccess) return ce;
    }
    return cudaSuccess;
}

// orth.h entry point called with X in device (or managed) memory: the QR runs in
// place on the caller's buffer, with no staging. R is written in place when it is
// device memory too (the kernels write exactly the reference's part of R), else
// through a device copy and the write-back rule. Synchronous, like the reference.
int run_on_device_buffers(int variant, int m, int n, int s, double* dX, int ldX, double* R, int ldR, bool r_dev,
                          int precision) {
    cudaStream_t st = g_ctx.stream;
    orth_gb300_status stt;
    std::memset(&stt, 0, sizeof(stt));
    double* dR = R;
    int ldr = ldR;
    if (!r_dev) {
        if (g_ctx.hostR.ensure((size_t)n * n * sizeof(double))) return 3;
        dR = g_ctx.hostR.as<double>();
        ldr = n;
        if (zero_async(dR, (size_t)n * n * sizeof(double), st)) return 3;
    }
    int rc = run_device(variant, m, n, s, dX, ldX, dR, ldr, precision, st, &stt);
    if (!rc && !r_dev) {
        cudaError_t ce = cudaStreamSynchronize(st);
        if (ce == cudaSuccess) ce = write_back_r(variant, n, s, dR, n, R, ldR, cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) {
            stt.cuda_error = (int)ce;
            rc = 3;
        }
    }
    g_last_status = stt;
    return rc;
}

// Host-buffer form (the orth.h ABI).
int run_host(int variant, int m, int n, int s, double* Xsub, int ldXsub, double* R, int ldR,
             double* work, int lwork, int precision) {
    (void)work;
    // lwork rule of the reference (SRC/orth.c:82,255,397,489,584), in 64 bits and
    // capped at INT_MAX so that sizes the reference cannot index are still usable.
    const i64 msub = m;
    i64 need = 5LL * n * s + 9LL * s * s + (variant == ORTH_GB300_BCGSI2 ? msub * s : msub * n);
    if (need > INT_MAX) need = INT_MAX;
    if ((i64)lwork < need) {
        printf("%% Work space is too small. It should be larger than 6*n*s + 8*s*s.\n");
        fflush(stdout);
        return 1;
    }
    if (!valid_args(m, n, s, ldXsub, ldR) || Xsub == nullptr || R == nullptr) return 2;
    std::lock_guard<std::mutex> lock(g_mu);
    int rc = init_ctx();
    if (rc) return 3;
    cudaStream_t st = g_ctx.stream;
    const bool x_dev = is_device_pointer(Xsub), r_dev = is_device_pointer(R);
    if (x_dev) return run_on_device_buffers(variant, m, n, s, Xsub, ldXsub, R, ldR, r_dev, precision);
    const size_t xbytes = (size_t)m * n * sizeof(double);
    const size_t rbytes = (size_t)n * n * sizeof(double);
    if (g_ctx.hostX.ensure(xbytes) || g_ctx.hostR.ensure(rbytes)) return 3;
    if (g_ctx.hostR_stage_bytes < rbytes) {
        if (g_ctx.hostR_stage) cudaFreeHost(g_ctx.hostR_stage);
        g_ctx.hostR_stage = nullptr;
        g_ctx.hostR_stage_bytes = 0;
        if (cudaMallocHost(&g_ctx.hostR_stage, rbytes) != cudaSuccess) return 3;
        g_ctx.hostR_stage_bytes = rbytes;
    }
    double* dX = g_ctx.hostX.as<double>();
    double* dR = g_ctx.hostR.as<double>();
    orth_gb300_status stt;
    std::memset(&stt, 0, sizeof(stt));
    // X goes up in column chunks of at least one block and about 64 MB on a copy
    // stream; Q comes back on another as its columns become final (HostLink).
    HostLink link;
    link.hX = Xsub; link.ldh = ldXsub; link.m = m; link.n = n; link.dX = dX;
    link.cin = g_ctx.copy_in; link.cout = g_ctx.copy_out;
    link.hR = g_ctx.hostR_stage; link.dR = dR; link.rbytes = rbytes;
    link.pageable = !is_page_locked(Xsub);
    {
        const i64 per64mb = ((i64)64 << 20) / ((i64)m * (i64)sizeof(double));
        link.chunk = (int)(per64mb > s ? (per64mb < n ? per64mb : n) : s);
    }
    const auto wall0 = std::chrono::steady_clock::now();
    cudaEvent_t* tev = g_ctx.host_ev;
    bool timed = false;
    cudaError_t ce = cudaEventRecord(tev[0], st);
    if (ce == cudaSuccess) ce = (cudaError_t)zero_async(dR, rbytes, st);
    link.x_done = tev[1];
    if (ce == cudaSuccess) {
        link.start(st);
        ce = (cudaError_t)link.err.load();
    }
    link.done = tev[2];
    if (ce == cudaSuccess) {
        rc = run_device(variant, m, n, s, dX, m, dR, n, precision, st, &stt, &link);
        link.join();   // every copy issued (pageable: complete)
        if (!rc) {
            ce = link.finished ? (cudaError_t)link.err.load() : cudaErrorUnknown;
            if (ce == cudaSuccess) ce = cudaEventRecord(tev[3], g_ctx.copy_out);
            timed = ce == cudaSuccess;
        }
    }
    // The caller's buffer is in use until both copy streams are done, on every path.
    cudaError_t c1 = cudaStreamSynchronize(g_ctx.copy_in);
    cudaError_t c2 = cudaStreamSynchronize(g_ctx.copy_out);
    cudaError_t c3 = cudaStreamSynchronize(st);
    link.release();
    if (timed && c1 == cudaSuccess && c2 == cudaSuccess && c3 == cudaSuccess) {
        for (int k = 1; k < 4; ++k) {
            float ms = 0.f;
            g_last_host_timing[k - 1] = cudaEventElapsedTime(&ms, tev[0], tev[k]) == cudaSuccess ? ms : -1.0;
        }
        g_last_host_timing[3] =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    }
    if (ce == cudaSuccess) ce = c1 != cudaSuccess ? c1 : (c2 != cudaSuccess ? c2 : c3);
    if (rc) {
        g_last_status = stt;
        return rc;
    }
    if (ce != cudaSuccess) {
        stt.cuda_error = (int)ce;
        g_last_status = stt;
        return 3;
    }
    // Write back what the reference writes: for column j of block b, rows
    // [0, end of block b); bcgsi21s writes only the upper triangle of its
    // diagonal blocks after the first (SRC/orth.c:302,360 use dlacpy 'U').
    const double* hs = g_ctx.hostR_stage;
    if (r_dev) {
        ce = write_back_r(variant, n, s, hs, n, R, ldR, cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) {
            stt.cuda_error = (int)ce;
            g_last_status = stt;
            return 3;
        }
        g_last_status = stt;
        return 0;
    }
    for (int j = 0; j < n; ++j) {
        const int b = j / s;
        int rows = (b + 1) * s < n ? (b + 1) * s : n;
        if (variant == ORTH_GB300_BCGSI21S && b >= 1) rows = j + 1;
        std::memcpy(R + (size_t)j * ldR, hs + (size_t)j * n, (size_t)rows * sizeof(double));
    }
    g_last_status = stt;
    return 0;
}

}  // namespace

// Schedule of a split-precision batch (host arithmetic only): the number of
// scratch slots S and each matrix's slot. A slot's scratch is sized for its
// largest matrix, and the longest-first assignment gives each slot one of the S
// largest, so S is the most slots whose S largest workspaces fit in half of
// free_bytes (at least one; free_bytes < 0: no memory limit), at most kSlots,
// count and max_slots (if >= 1). Jobs (weight m n^2) go longest first, each to the
// least loaded slot; `order` receives that sequence.
int split_batch_plan(int count, const int* m, const int* n, const int* s, int num_sms, long long free_bytes,
                     int max_slots, std::vector<int>& order, std::vector<int>& slot_of) {
    order.assign((size_t)(count > 0 ? count : 0), 0);
    slot_of.assign(order.size(), 0);
    if (count < 1) return 0;
    int S = count < kSlots ? count : kSlots;
    if (max_slots >= 1 && S > max_slots) S = max_slots;
    if (free_bytes >= 0) {
        std::vector<double> wsz(count);
        for (int b = 0; b < count; ++b)
            wsz[b] = (double)split_workspace_bytes(m[b], n[b], s[b], num_sms) +
                     8.0 * ((double)part_doubles(m[b], n[b], s[b], num_sms) + (double)tsqr_workspace_doubles(m[b], s[b]));
        std::sort(wsz.begin(), wsz.end(), [](double a, double b) { return a > b; });
        double acc = 0.0;
        int fit = 0;
        for (int k = 0; k < S; ++k) {
            acc += wsz[k];
            if (acc > 0.5 * (double)free_bytes) break;
            fit = k + 1;
        }
        S = fit > 1 ? fit : 1;
    }
    for (int b = 0; b < count; ++b) order[b] = b;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        const double wa = (double)m[a] * n[a] * n[a], wb = (double)m[b] * n[b] * n[b];
        return wa > wb || (wa == wb && a < b);
    });
    std::vector<double> load(S, 0.0);
    for (int b : order) {
        int k = 0;
        for (int q = 1; q < S; ++q)
            if (load[q] < load[k]) k = q;
        slot_of[b] = k;
        load[k] += (double)m[b] * n[b] * n[b];
    }
    return S;
}

// Split-precision batches: the matrices one after another on `st` through the
// single-matrix driver (its digit store is 14 bytes per element, so a whole
// batch's stores at once would not fit). Workspaces are grown for the largest
// shapes first, so no allocation happens between matrices. After each matrix its
// status words (4 ints) and the split kernels' error word go to dstatus[8 b ..]
// on the device; nothing waits on the host.
int split_batch_enqueue(int variant, int count, const int* m, const int* n, const int* s, double* const* dX,
                        const long long* ldX, double* const* dR, const int* ldR, int precision, cudaStream_t st,
                        int* dstatus, int max_slots) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (init_ctx()) return 3;
    size_t free_b = 0, total_b = 0;
    const long long fb = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess ? (long long)free_b : -1;
    std::vector<int> order, slot_of;
    const int S = split_batch_plan(count, m, n, s, g_ctx.num_sms, fb, max_slots, order, slot_of);
    int rc = 0;
    for (int k = 0; k < S && !rc; ++k)
        if (!g_ctx.slot_stream[k] &&
            cudaStreamCreateWithFlags(&g_ctx.slot_stream[k], cudaStreamNonBlocking) != cudaSuccess)
            rc = 3;
    // Grow every slot's scratch for its largest shapes before anything is enqueued.
    for (int i = 0; i < count && !rc; ++i) {
        const int b = order[i];
        g_slot = slot_of[b];
        if (reserve(m[b], n[b], s[b], precision)) rc = 3;
    }
    cudaEvent_t fork = nullptr;
    if (!rc && cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) rc = 3;
    if (!rc && cudaEventRecord(fork, st) != cudaSuccess) rc = 3;
    for (int k = 0; k < S && !rc; ++k)
        if (cudaStreamWaitEvent(g_ctx.slot_stream[k], fork, 0) != cudaSuccess) rc = 3;
    for (int i = 0; i < count && !rc; ++i) {
        const int b = order[i], k = slot_of[b];
        g_slot = k;
        split_select_slot(k);
        cudaStream_t ss = g_ctx.slot_stream[k];
        rc = run_device(variant, m[b], n[b], s[b], dX[b], ldX[b], dR[b], ldR[b], precision, ss, nullptr);
        if (rc) break;
        cudaError_t ce = cudaMemcpyAsync(dstatus + 8 * (i64)b, scr().status.as<int>(), kStatusWords * sizeof(int),
                                         cudaMemcpyDeviceToDevice, ss);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(dstatus + 8 * (i64)b + 4, split_error_ptr(), sizeof(int), cudaMemcpyDeviceToDevice, ss);
        if (ce != cudaSuccess) rc = 3;
    }
    g_slot = 0;
    split_select_slot(0);
    // Join: the caller's stream waits for every slot stream.
    for (int k = 0; k < S; ++k) {
        cudaEvent_t j = nullptr;
        if (cudaEventCreateWithFlags(&j, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(j, g_ctx.slot_stream[k]);
            cudaStreamWaitEvent(st, j, 0);
            cudaEventDestroy(j);
        }
    }
    if (fork) cudaEventDestroy(fork);
    return rc;
}

}  // namespace bcgs

using namespace bcgs;

extern "C" {

int bcgsi2P1s(int m, int n, int s, double* Xsub, int ldXsub, double* R, int ldR, double* work,
              int lwork) {
    return run_host(ORTH_GB300_BCGSI2P1S, m, n, s, Xsub, ldXsub, R, ldR, work, lwork, host_precision());
}
int bcgsi21s(int m, int n, int s, double* Xsub, int ldXsub, double* R, int ldR, double* work,
             int lwork) {
    return run_host(ORTH_GB300_BCGSI21S, m, n, s, Xsub, ldXsub, R, ldR, work, lwork, host_precision());
}
int bcgspipi2(int m, int n, int s, double* Xsub, int ldXsub, double* R, int ldR, double* work,
              int lwork) {
    return run_host(ORTH_GB300_BCGSPIPI2, m, n, s, Xsub, ldXsub, R, ldR, work, lwork, host_precision());
}
int bcgsi2(int m, int n, int s, double* Xsub, int ldXsub, double* R, int ldR, double* work,
           int lwork) {
    return run_host(ORTH_GB300_BCGSI2, m, n, s, Xsub, ldXsub, R, ldR, work, lwork, host_precision());
}
int bcgsi2P2s(int m, int n, int s, double* Xsub, int ldXsub, double* R, int ldR, double* work,
              int lwork) {
    return run_host(ORTH_GB300_BCGSI2P2S, m, n, s, Xsub, ldXsub, R, ldR, work, lwork, host_precision());
}

int orth_gb300_run_dev(int variant, int m, int n, int s, double* dX, long long ldX, double* dR,
                       int ldR, int precision, void* stream, orth_gb300_status* status) {
    std::lock_guard<std::mutex> lock(g_mu);
    return run_device(variant, m, n, s, dX, ldX, dR, ldR, precision, (cudaStream_t)stream, status);
}

void orth_gb300_last_status(orth_gb300_status* status) {
    if (status) *status = g_last_status;
}

void orth_gb300_last_host_timing(double out[4]) {
    if (out)
        for (int k = 0; k < 4; ++k) out[k] = g_last_host_timing[k];
}

int orth_gb300_set_host_precision(int precision) {
    if (precision != ORTH_GB300_FP64 && !is_split(precision)) return 4;
    std::lock_guard<std::mutex> lock(g_mu);
    g_host_precision = precision;
    return 0;
}

int orth_gb300_last_split_error(void) { return split_last_error(); }

int orth_gb300_shard_rows(long long m, int size, int rank, long long* row0, long long* msub) {
    if (m < 1 || size < 1 || rank < 0 || rank >= size || !row0 || !msub) return 2;
    i64 r0 = 0, ms = 0;
    shard_rows(m, size, rank, &r0, &ms);
    *row0 = r0;
    *msub = ms;
    return ceil_div(m, kShardRows) < size ? 2 : 0;
}

int orth_gb300_run_sharded(int variant, long long m, int n, int s, double* dXsub, long long ldX, double* dR,
                           int ldR, void* stream, const orth_gb300_comm* comm, orth_gb300_status* status) {
    std::lock_guard<std::mutex> lock(g_mu);
    return run_sharded(variant, m, n, s, dXsub, ldX, dR, ldR, (cudaStream_t)stream, comm, status);
}

int orth_gb300_set_intra_ortho(int mode) {
    if (mode != ORTH_GB300_INTRA_TSQR && mode != ORTH_GB300_INTRA_CHOLQR2) return 2;
    std::lock_guard<std::mutex> lock(g_mu);
    g_intra_mode = mode;
    return 0;
}

int orth_gb300_split_supported(int m, int n, int s) { return split_supported(m, n, s) ? 1 : 0; }

int orth_gb300_gram_dev(int m, int na, int b0, int nb, const double* dX, long long ldX, double* dC,
                        int ldc, int precision, void* stream) {
    std::lock_guard<std::mutex> lock(g_mu);
    const int n = na > b0 + nb ? na : b0 + nb;
    if (m < 1 || na < 1 || nb < 1 || b0 < 0 || ldX < m || ldc < na || !dX || !dC) return 2;
    if (precision != ORTH_GB300_FP64 && !is_split(precision)) return 4;
    const int s = (nb + 1) / 2 > 0 ? (nb + 1) / 2 : 1;
    if (is_split(precision) && (nb > 64 || !split_supported(m, n, s < 1 ? 1 : s))) return 4;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = init_ctx();
    if (rc) return 3;
    if (precision == ORTH_GB300_FP64) {
        if (scr().part.ensure((size_t)part_doubles(m, n, s, g_ctx.num_sms) * sizeof(double))) return 3;
        const int chunks = gram_chunks_fp64(m, na, nb, g_ctx.num_sms);
        rc = launch_gram_fp64(dX, ldX, m, 0, na, b0, nb, dC, ldc, scr().part.as<double>(), chunks, st);
    } else {
        if (scr().split.ensure((size_t)split_workspace_bytes(m, n, s, g_ctx.num_sms))) return 3;
        rc = split_begin(const_cast<double*>(dX), ldX, m, n, s, split_digits_of(precision), scr().split.as<char>(), scr().split.bytes,
                         g_ctx.num_sms, st);
        if (!rc)
            rc = launch_gram_split(dX, ldX, m, na, b0, nb, dC, ldc, scr().split.as<char>(), scr().split.bytes,
                                   g_ctx.num_sms, st);
        if (!rc) {
            int w = 0;
            rc = split_error_word(&w, st);
            if (!rc && w) rc = (int)cudaErrorLaunchTimeout;
        }
    }
    return rc ? 3 : 0;
}

int orth_gb300_split_batch_plan(int count, const int* m, const int* n, const int* s, long long free_bytes,
                                int max_slots, int* slot_of, int* order) {
    if (count < 1 || !m || !n || !s) return 0;
    std::vector<int> ord, slot;
    const int S = split_batch_plan(count, m, n, s, kNumSMsDefault, free_bytes, max_slots, ord, slot);
    for (int b = 0; b < count; ++b) {
        if (slot_of) slot_of[b] = slot[b];
        if (order) order[b] = ord[b];
    }
    return S;
}

int orth_gb300_split_slice_dev(long long m, int n, const double* dX, long long ldX, int planes,
                               unsigned short* dDigits, int* dExp, void* stream) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (m < 1 || n < 1 || n > 65535 || !dX || !dDigits || !dExp || ldX < m || (planes != 6 && planes != 7)) return 2;
    cudaStream_t st = (cudaStream_t)stream;
    if (init_ctx()) return 3;
    if (g_ctx.metric.ensure((size_t)n * sizeof(unsigned long long))) return 3;
    int rc = split_slice_columns(dX, ldX, m, n, planes, dDigits, dExp, g_ctx.metric.as<unsigned long long>(), st);
    if (!rc) rc = (int)cudaStreamSynchronize(st);
    return rc ? 3 : 0;
}

void orth_gb300_set_gram_chunk_rows(long long rows) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_gram_chunk_rows = rows > 0 ? rows : 0;
}

int orth_gb300_accuracy_dev(int m, int n, const double* dX, long long ldX, const double* dQ, long long ldQ,
                            const double* dR, int ldR, int gram_precision, double* dE, int lde, void* stream,
                            double out[3]) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (m < 1 || n < 1 || !dX || !dQ || !dR || !out || ldX < m || ldQ < m || ldR < n) return 2;
    if (dE && lde < n) return 2;
    if (gram_precision != ORTH_GB300_FP64 && gram_precision != ORTH_GB300_SPLIT_BF16) return 4;
    if (gram_precision == ORTH_GB300_SPLIT_BF16 && !split_supported(m, n, 16)) return 4;
    cudaStream_t st = (cudaStream_t)stream;
    if (init_ctx()) return 3;
    constexpr int GW = 32;   // Gram column group
    // Layout of the metric buffer: G (n x n) | E (n x n, unless the caller's) |
    // residual partials | out[3].
    const i64 nn = (i64)n * n;
    const i64 pd = metrics_part_doubles(m, n);
    if (g_ctx.metric.ensure((size_t)(2 * nn + pd + 8) * sizeof(double))) return 3;
    double* G = g_ctx.metric.as<double>();
    double* E = dE ? dE : G + nn;
    const int ldE = dE ? lde : n;
    double* part = G + 2 * nn;
    double* dout = part + pd;
    int rc = 0;
    if (gram_precision == ORTH_GB300_FP64) {
        i64 need = 0;
        for (int na = GW; na < n + GW; na += GW) {
            const int a = na < n ? na : n;
            const i64 v = (i64)gram_chunks_fp64(m, a, GW, g_ctx.num_sms) * a * GW;
            if (v > need) need = v;
        }
        if (scr().part.ensure((size_t)(need + 1024) * sizeof(double))) return 3;
    } else {
        if (scr().split.ensure((size_t)split_workspace_bytes(m, n, 16, g_ctx.num_sms))) return 3;
        rc = split_begin(const_cast<double*>(dQ), ldQ, m, n, 16, 7, scr().split.as<char>(), scr().split.bytes,
                         g_ctx.num_sms, st);
        if (rc) return 3;
    }
    // Upper block triangle of Q^T Q, one 32-column group at a time.
    for (int c0 = 0; c0 < n && !rc; c0 += GW) {
        const int nb = n - c0 < GW ? n - c0 : GW;
        const int na = c0 + nb;
        if (gram_precision == ORTH_GB300_FP64) {
            const int chunks = gram_chunks_fp64(m, na, nb, g_ctx.num_sms);
            rc = launch_gram_fp64(dQ, ldQ, m, 0, na, c0, nb, G + (i64)c0 * n, n, scr().part.as<double>(), chunks, st);
        } else {
            rc = launch_gram_split(dQ, ldQ, m, na, c0, nb, G + (i64)c0 * n, n, scr().split.as<char>(),
                                   scr().split.bytes, g_ctx.num_sms, st);
        }
    }
    if (!rc && gram_precision != ORTH_GB300_FP64) {
        int w = 0;
        rc = split_error_word(&w, st);
        if (!rc && w) rc = (int)cudaErrorLaunchTimeout;
    }
    if (!rc) rc = launch_loo_finish(G, n, n, E, ldE, dout, st);
    if (!rc) rc = launch_residual(dX, ldX, dQ, ldQ, m, n, dR, ldR, part, dout, st);
    if (!rc) rc = (int)cudaMemcpyAsync(out, dout, 3 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (!rc) rc = (int)cudaStreamSynchronize(st);
    return rc ? 3 : 0;
}

int orth_gb300_sync_count(int variant, int n, int s) {
    if (s < 1 || n < 2 * s) return -1;
    const int p = nblocks_after_first(n, s);
    switch (variant) {
        case ORTH_GB300_BCGSI2P1S: return 2 + (p - 1);   // first step 2, then 1 per step
        case ORTH_GB300_BCGSI21S: return 2 + (p - 1);
        case ORTH_GB300_BCGSPIPI2: return 2 * p;
        case ORTH_GB300_BCGSI2: return 2 * p;
        case ORTH_GB300_BCGSI2P2S: return 2 + (p - 1);
        default: return -1;
    }
}

long long orth_gb300_last_launch_count(void) { return g_last_launches; }

long long orth_gb300_last_reduction_count(void) { return g_last_reductions; }

void orth_gb300_profile(int on) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (auto& p : g_prof.pending) { g_prof.pool.push_back(p.a); g_prof.pool.push_back(p.b); }
    g_prof.pending.clear();
    for (int c = 0; c < kProfClasses; ++c) {
        g_prof.ms[c] = 0; g_prof.launches[c] = 0; g_prof.flops[c] = 0; g_prof.bytes[c] = 0; g_prof.traffic[c] = 0;
        g_prof.calls[c] = 0;
    }
    g_prof.on = on != 0;
}

int orth_gb300_profile_classes(void) { return kProfClasses; }

int orth_gb300_profile_read(double* ms, long long* launches, double* flops, double* bytes) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (auto& p : g_prof.pending) {
        float e = 0.f;
        cudaError_t ce = cudaEventSynchronize(p.b);
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(&e, p.a, p.b);
        if (ce != cudaSuccess) return (int)ce;
        g_prof.ms[p.cls] += e;
        g_prof.pool.push_back(p.a);
        g_prof.pool.push_back(p.b);
    }
    g_prof.pending.clear();
    for (int c = 0; c < kProfClasses; ++c) {
        if (ms) ms[c] = g_prof.ms[c];
        if (launches) launches[c] = g_prof.launches[c];
        if (flops) flops[c] = g_prof.flops[c];
        if (bytes) bytes[c] = g_prof.bytes[c];
    }
    return 0;
}

int orth_gb300_profile_traffic(double* bytes, long long* calls) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (int c = 0; c < kProfClasses; ++c) {
        if (bytes) bytes[c] = g_prof.traffic[c];
        if (calls) calls[c] = g_prof.calls[c];
    }
    return 0;
}

int orth_gb300_reserve(int m, int n, int s) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!valid_args(m, n, s, m, n)) return 2;
    int rc = reserve(m, n, s, split_supported(m, n, s) ? ORTH_GB300_SPLIT_BF16 : ORTH_GB300_FP64);
    return rc ? 3 : 0;
}

void orth_gb300_release(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (Scratch& sc : g_scratch) {
        sc.part.release();
        sc.small.release();
        sc.status.release();
        sc.tsqr.release();
        sc.split.release();
    }
    split_forget_workspaces();
    g_ctx.gram.release();
    g_ctx.metric.release();
    g_ctx.hostX.release();
    g_ctx.hostR.release();
    if (g_ctx.hostR_stage) cudaFreeHost(g_ctx.hostR_stage);
    g_ctx.hostR_stage = nullptr;
    g_ctx.hostR_stage_bytes = 0;
    host_stage_release();
}

const char* orth_gb300_version(void) { return "orth_gb300 0.1 (sm_103a)"; }

}  // extern "C"
