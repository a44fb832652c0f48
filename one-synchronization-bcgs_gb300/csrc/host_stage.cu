// Staging slots and the host copy pool for pageable orth.h buffers (host_stage.h).
#include "host_stage.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "../../include/orth_gb300.h"

namespace bcgs {

CopyPool::CopyPool(int workers) {
    for (int i = 0; i < workers; ++i) workers_.emplace_back([this] { worker(); });
}

CopyPool::~CopyPool() {
    {
        std::lock_guard<std::mutex> lock(mu_);
        stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
}

// Part p of job j: a contiguous range, 64-byte aligned except at the end.
void CopyPool::run_part(const Job& j, int p) const {
    const size_t b0 = (j.bytes * (size_t)p / (size_t)j.parts) & ~(size_t)63;
    const size_t b1 = p + 1 == j.parts ? j.bytes : (j.bytes * (size_t)(p + 1) / (size_t)j.parts) & ~(size_t)63;
    if (b1 > b0) std::memcpy(j.dst + b0, j.src + b0, b1 - b0);
}

// A worker claims one part at a time under the lock and reports it done under the
// lock, so once a job's parts are all done no worker touches it again.
void CopyPool::worker() {
    std::unique_lock<std::mutex> lock(mu_);
    for (;;) {
        cv_.wait(lock, [&] { return stop_ || !queue_.empty(); });
        if (queue_.empty()) return;   // stop_
        Job* j = queue_.front();
        const int p = j->next++;
        if (j->next >= j->parts) queue_.pop_front();
        lock.unlock();
        run_part(*j, p);
        lock.lock();
        if (++j->done == j->parts) cv_done_.notify_all();
    }
}

void CopyPool::copy(void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return;
    Job j;
    j.dst = static_cast<char*>(dst);
    j.src = static_cast<const char*>(src);
    j.bytes = bytes;
    // Pieces of at least 8 MB each, at most one per thread.
    const size_t max_parts = std::max<size_t>(1, bytes >> 23);
    j.parts = (int)std::min<size_t>((size_t)threads(), max_parts);
    std::unique_lock<std::mutex> lock(mu_);
    if (j.parts > 1) {
        queue_.push_back(&j);
        cv_.notify_all();
    }
    while (j.next < j.parts) {
        const int p = j.next++;
        if (j.next >= j.parts && j.parts > 1) {
            auto it = std::find(queue_.begin(), queue_.end(), &j);
            if (it != queue_.end()) queue_.erase(it);
        }
        lock.unlock();
        run_part(j, p);
        lock.lock();
        ++j.done;
    }
    cv_done_.wait(lock, [&] { return j.done == j.parts; });
}

namespace {
std::mutex g_stage_mu;
HostStage* g_stage = nullptr;
bool g_stage_failed = false;
constexpr size_t kSlotBytes = (size_t)256 << 20;
constexpr int kUpSlots = 4, kDownSlots = 4;
}  // namespace

HostStage* host_stage() {
    std::lock_guard<std::mutex> lock(g_stage_mu);
    if (g_stage || g_stage_failed) return g_stage;
    // ORTH_GB300_HOST_STAGING=0: leave pageable copies to the driver (no pinned
    // slots, no copy threads), for hosts that cannot spare the 2 GB.
    if (const char* v = std::getenv("ORTH_GB300_HOST_STAGING")) {
        if (v[0] == '0') {
            g_stage_failed = true;
            return nullptr;
        }
    }
    HostStage* h = new HostStage;
    h->slot_bytes = kSlotBytes;
    bool ok = true;
    for (int i = 0; i < kUpSlots + kDownSlots && ok; ++i) {
        void* p = nullptr;
        ok = orth_gb300_host_alloc(kSlotBytes, &p) == 0;
        if (ok) (i < kUpSlots ? h->up : h->down).push_back(p);
    }
    if (!ok) {
        for (void* p : h->up) orth_gb300_host_free(p);
        for (void* p : h->down) orth_gb300_host_free(p);
        delete h;
        g_stage_failed = true;
        return nullptr;
    }
    const unsigned hw = std::thread::hardware_concurrency();
    // The upload and the download copy at the same time; each uses the pool.
    const int workers = (int)std::max(1u, std::min(hw > 2 ? hw / 2 : 1u, 8u)) - 1;
    h->pool = new CopyPool(workers > 0 ? workers : 0);
    g_stage = h;
    return g_stage;
}

void host_stage_release() {
    std::lock_guard<std::mutex> lock(g_stage_mu);
    if (!g_stage) return;
    delete g_stage->pool;
    for (void* p : g_stage->up) orth_gb300_host_free(p);
    for (void* p : g_stage->down) orth_gb300_host_free(p);
    delete g_stage;
    g_stage = nullptr;
    g_stage_failed = false;
}

}  // namespace bcgs
