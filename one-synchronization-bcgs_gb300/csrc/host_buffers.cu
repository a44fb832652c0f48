// Pinned host buffers backed by transparent huge pages.
//
// The orth.h entry points stream X to the GPU and Q back while the QR runs, so on
// a host-buffer call the host link is the other bound beside the kernels. On a
// GB300 node (Grace host, NVLink-C2C, 64 KB base pages) the rate of a long copy
// depends on how its host buffer was made. Measured for 32 GiB each way, three
// repetitions:
//   * cudaHostAlloc:                              81-100 GB/s H2D, 85-139 GB/s D2H;
//   * mmap + madvise(MADV_HUGEPAGE) + cudaHostRegister: 210 GB/s H2D, 193 GB/s D2H;
//   * mmap without huge pages + cudaHostRegister: 25-34 GB/s after the first copy.
// A huge page (512 MB on a 64 KB-page kernel) gives the copy engines one
// translation where 64 KB pages give 8192, so a 34 GB buffer no longer outruns
// the translation caches.
//
// orth_gb300_host_alloc makes such a buffer: an anonymous mapping aligned to the
// huge-page size, advised MADV_HUGEPAGE, faulted in by a few host threads (one
// write per huge page; the kernel zero-fills), then registered with the CUDA
// driver (page-locked, usable by async copies). A host whose memory is too
// fragmented to give huge pages backs such a mapping with base pages, the slow
// case above; when less than 3/4 of a buffer of 64 MB or more came as huge pages
// (AnonHugePages in /proc/self/smaps), the mapping is dropped and the buffer comes
// from cudaHostAlloc instead, zero-filled by the same threads.
// orth_gb300_host_free undoes either.
#include <sys/mman.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/orth_gb300.h"

namespace bcgs {
namespace {

struct Mapping {
    void* raw;          // the anonymous mapping (null: a cudaHostAlloc buffer)
    size_t raw_bytes;
    size_t len;         // usable bytes from the returned pointer
};
std::mutex g_host_mu;
std::map<void*, Mapping> g_host_maps;

// The kernel's PMD huge-page size, or 2 MiB when it does not say.
size_t huge_page_bytes() {
    size_t hp = (size_t)2 << 20;
    if (FILE* f = std::fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
        unsigned long long v = 0;
        if (std::fscanf(f, "%llu", &v) == 1 && v >= 4096 && (v & (v - 1)) == 0) hp = (size_t)v;
        std::fclose(f);
    }
    return hp;
}

// One write per `step` bytes of [p, p + bytes), split over a few threads.
void fault_in(char* p, size_t bytes, size_t step) {
    const size_t pages = (bytes + step - 1) / step;
    unsigned hw = std::thread::hardware_concurrency();
    const size_t nt = std::min<size_t>(std::max(1u, std::min(hw, 16u)), pages);
    auto work = [&](size_t t) {
        for (size_t i = t; i < pages; i += nt) p[i * step] = 0;
    };
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& x : th) x.join();
}

// Zeroes [p, p + bytes) with the same threads.
void zero_fill(char* p, size_t bytes) {
    unsigned hw = std::thread::hardware_concurrency();
    const size_t nt = std::max<size_t>(1, std::min<size_t>(std::min(hw, 16u), (bytes >> 26) + 1));
    auto work = [&](size_t t) {
        const size_t b0 = bytes * t / nt, b1 = bytes * (t + 1) / nt;
        std::memset(p + b0, 0, b1 - b0);
    };
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& x : th) x.join();
}

}  // namespace

// Bytes of [p, p + len) backed by transparent huge pages: the AnonHugePages of the
// mappings that overlap the range (/proc/self/smaps), or -1 if it cannot be read.
long long huge_backed_bytes(const void* p, size_t len) {
    FILE* f = std::fopen("/proc/self/smaps", "r");
    if (!f) return -1;
    const unsigned long long lo = (unsigned long long)(uintptr_t)p, hi = lo + len;
    char line[512];
    bool in = false;
    long long total = 0;
    while (std::fgets(line, sizeof line, f)) {
        unsigned long long a = 0, b = 0;
        if (std::sscanf(line, "%llx-%llx ", &a, &b) == 2) {   // a mapping's header line
            in = a < hi && b > lo;
            continue;
        }
        unsigned long long kb = 0;
        if (in && std::sscanf(line, "AnonHugePages: %llu kB", &kb) == 1) total += (long long)kb * 1024;
    }
    std::fclose(f);
    return total;
}

}  // namespace bcgs

using namespace bcgs;

extern "C" int orth_gb300_host_alloc(size_t bytes, void** ptr) {
    if (ptr == nullptr || bytes == 0) return 2;
    *ptr = nullptr;
    const size_t hp = huge_page_bytes();
    const size_t len = (bytes + hp - 1) / hp * hp;
    const size_t raw_bytes = len + hp;   // room to align the start to a huge page
    void* raw = mmap(nullptr, raw_bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (raw == MAP_FAILED) return 6;
    char* p = reinterpret_cast<char*>(((uintptr_t)raw + hp - 1) / hp * hp);
    (void)madvise(p, len, MADV_HUGEPAGE);   // best effort: without it the pages are base-size
    fault_in(p, len, hp);
    const long long huge = huge_backed_bytes(p, len);
    if (huge >= 0 && bytes >= ((size_t)64 << 20) && (double)huge < 0.75 * (double)len) {
        munmap(raw, raw_bytes);
        void* q = nullptr;
        if (cudaHostAlloc(&q, bytes, cudaHostAllocDefault) != cudaSuccess) {
            (void)cudaGetLastError();
            return 3;
        }
        zero_fill(static_cast<char*>(q), bytes);
        std::lock_guard<std::mutex> lock(g_host_mu);
        g_host_maps[q] = Mapping{nullptr, 0, bytes};
        *ptr = q;
        return 0;
    }
    if (cudaHostRegister(p, len, cudaHostRegisterDefault) != cudaSuccess) {
        (void)cudaGetLastError();
        munmap(raw, raw_bytes);
        return 3;
    }
    {
        std::lock_guard<std::mutex> lock(g_host_mu);
        g_host_maps[p] = Mapping{raw, raw_bytes, len};
    }
    *ptr = p;
    return 0;
}

extern "C" int orth_gb300_host_buffer_info(const void* ptr, int* kind, long long* huge_bytes) {
    if (ptr == nullptr || kind == nullptr || huge_bytes == nullptr) return 2;
    Mapping mp;
    {
        std::lock_guard<std::mutex> lock(g_host_mu);
        auto it = g_host_maps.find(const_cast<void*>(ptr));
        if (it == g_host_maps.end()) return 2;
        mp = it->second;
    }
    *kind = mp.raw ? 1 : 2;
    *huge_bytes = huge_backed_bytes(ptr, mp.len);
    return 0;
}

extern "C" int orth_gb300_host_free(void* ptr) {
    if (ptr == nullptr) return 0;
    Mapping mp;
    {
        std::lock_guard<std::mutex> lock(g_host_mu);
        auto it = g_host_maps.find(ptr);
        if (it == g_host_maps.end()) return 2;
        mp = it->second;
        g_host_maps.erase(it);
    }
    if (!mp.raw) return cudaFreeHost(ptr) == cudaSuccess ? 0 : 3;
    const cudaError_t ce = cudaHostUnregister(ptr);
    munmap(mp.raw, mp.raw_bytes);
    return ce == cudaSuccess ? 0 : 3;
}
