// Staging for pageable host buffers of the orth.h entry points.
//
// A copy between the device and pageable memory goes through the driver's own
// bounce buffers at the rate of one host thread's memcpy (13-16 GB/s measured on
// a GB300 node for malloc'd memory, 25-43 GB/s with several threads issuing).
// The orth.h calls instead copy pageable X through a few page-locked, huge-page
// slots of their own: host threads copy between the caller's buffer and a slot
// (split over a small pool of workers), and the copy engines move the slot
// to or from the device at the page-locked rate.
#pragma once

#include <condition_variable>
#include <cstddef>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

namespace bcgs {

// Host memcpy split over a pool of worker threads; the calling thread works too.
// Several callers may copy at once (each call is one job in a shared queue).
class CopyPool {
public:
    explicit CopyPool(int workers);
    ~CopyPool();
    void copy(void* dst, const void* src, size_t bytes);
    int threads() const { return (int)workers_.size() + 1; }

private:
    struct Job {
        char* dst;
        const char* src;
        size_t bytes;
        int parts, next = 0, done = 0;
    };
    void run_part(const Job& j, int p) const;
    void worker();
    std::vector<std::thread> workers_;
    std::mutex mu_;
    std::condition_variable cv_, cv_done_;
    std::deque<Job*> queue_;
    bool stop_ = false;
};

// Page-locked slots (from orth_gb300_host_alloc) and the copy pool, kept for the
// process: `up` slots for X going to the device, `down` for Q coming back.
struct HostStage {
    size_t slot_bytes = 0;
    std::vector<void*> up, down;
    CopyPool* pool = nullptr;
};

// The process's staging (created on first use); null if its memory cannot be had.
HostStage* host_stage();
// Frees the staging slots and stops the copy threads.
void host_stage_release();

}  // namespace bcgs
