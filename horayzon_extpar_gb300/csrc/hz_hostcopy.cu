// hz_hostcopy.cu -- host <-> device copies for caller buffers of any kind.
//
// The host entry points receive the caller's arrays as they are; from Python
// (numpy) and Fortran these are ordinary pageable allocations, for which a
// cudaMemcpy runs through the driver's own small staging buffers at a
// fraction of the link bandwidth. Page-locked buffers go straight through
// cudaMemcpyAsync. Pageable ones are moved through two page-locked chunks:
// the device copies one chunk while host threads copy the other between the
// chunk and the caller's array.
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "hz_internal.h"

namespace hz {

namespace {

constexpr size_t kChunkBytes = 16u << 20;  // per staging chunk
constexpr int kMaxThreads = 8;

bool is_page_locked(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

}  // namespace

// Page-locked chunks, their events and a pool of host threads for memcpy.
struct Staging {
  void* chunk[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv_job, cv_done;
  char* dst = nullptr;
  const char* src = nullptr;
  size_t bytes = 0;
  unsigned long long generation = 0;
  int pending = 0;
  bool stop = false;
  // Upload ring: the chunk the next upload piece uses, and whether a chunk's
  // last device copy may still be reading it (its `done` event is pending).
  int next = 0;
  bool in_flight[2] = {false, false};

  ~Staging() {
    {
      std::lock_guard<std::mutex> l(mu);
      stop = true;
    }
    cv_job.notify_all();
    for (auto& t : workers) t.join();
    for (int k = 0; k < 2; k++) {
      if (chunk[k]) cudaFreeHost(chunk[k]);
      if (done[k]) cudaEventDestroy(done[k]);
    }
  }

  cudaError_t init() {
    for (int k = 0; k < 2; k++) {
      cudaError_t e = cudaMallocHost(&chunk[k], kChunkBytes);
      if (e != cudaSuccess) return e;
      e = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming);
      if (e != cudaSuccess) return e;
    }
    const unsigned hw = std::thread::hardware_concurrency();
    const int n = std::max(1, std::min<int>(kMaxThreads, hw > 1 ? (int)hw / 2 : 1));
    for (int w = 0; w < n; w++) workers.emplace_back([this, w, n] { work(w, n); });
    return cudaSuccess;
  }

  void work(int w, int n) {
    unsigned long long seen = 0;
    for (;;) {
      char* d;
      const char* s;
      size_t b;
      {
        std::unique_lock<std::mutex> l(mu);
        cv_job.wait(l, [&] { return stop || generation != seen; });
        if (stop) return;
        seen = generation;
        d = dst;
        s = src;
        b = bytes;
      }
      const size_t part = (b + n - 1) / n;
      const size_t lo = std::min(b, part * (size_t)w), hi = std::min(b, lo + part);
      if (hi > lo) std::memcpy(d + lo, s + lo, hi - lo);
      {
        std::lock_guard<std::mutex> l(mu);
        if (--pending == 0) cv_done.notify_one();
      }
    }
  }

  // memcpy spread over the worker threads; returns when all parts are done.
  void parallel_copy(void* d, const void* s, size_t b) {
    if (b < (1u << 20) || workers.size() < 2) {
      std::memcpy(d, s, b);
      return;
    }
    std::unique_lock<std::mutex> l(mu);
    dst = static_cast<char*>(d);
    src = static_cast<const char*>(s);
    bytes = b;
    pending = (int)workers.size();
    generation++;
    cv_job.notify_all();
    cv_done.wait(l, [&] { return pending == 0; });
  }
};

cudaError_t staging_create(Staging** out) {
  Staging* st = new Staging();
  const cudaError_t e = st->init();
  if (e != cudaSuccess) {
    delete st;
    *out = nullptr;
    return e;
  }
  *out = st;
  return cudaSuccess;
}

void staging_destroy(Staging* st) { delete st; }

cudaError_t copy_to_host(Staging* st, void* dst, const void* src_dev, size_t bytes,
                         cudaStream_t s) {
  if (bytes == 0) return cudaSuccess;
  if (!st || is_page_locked(dst))
    return cudaMemcpyAsync(dst, src_dev, bytes, cudaMemcpyDeviceToHost, s);
  const char* src = static_cast<const char*>(src_dev);
  char* out = static_cast<char*>(dst);
  // Uploads still reading a chunk finish first (they may be on another
  // stream); afterwards the chunks are free.
  for (int k = 0; k < 2; k++) {
    if (st->in_flight[k]) {
      const cudaError_t e = cudaEventSynchronize(st->done[k]);
      if (e != cudaSuccess) return e;
      st->in_flight[k] = false;
    }
  }
  const size_t n = (bytes + kChunkBytes - 1) / kChunkBytes;
  for (size_t i = 0; i <= n; i++) {
    if (i < n) {  // device -> chunk i % 2 (that chunk's previous contents are copied out)
      const size_t off = i * kChunkBytes, len = std::min(kChunkBytes, bytes - off);
      cudaError_t e = cudaMemcpyAsync(st->chunk[i % 2], src + off, len, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaEventRecord(st->done[i % 2], s);
      if (e != cudaSuccess) return e;
    }
    if (i > 0) {  // chunk i - 1 -> caller, overlapping the copy of chunk i
      const size_t j = i - 1, off = j * kChunkBytes, len = std::min(kChunkBytes, bytes - off);
      const cudaError_t e = cudaEventSynchronize(st->done[j % 2]);
      if (e != cudaSuccess) return e;
      st->parallel_copy(out + off, st->chunk[j % 2], len);
    }
  }
  return cudaSuccess;
}

cudaError_t copy_from_host(Staging* st, void* dst_dev, const void* src, size_t bytes,
                           cudaStream_t s) {
  if (bytes == 0) return cudaSuccess;
  if (!st || is_page_locked(src))
    return cudaMemcpyAsync(dst_dev, src, bytes, cudaMemcpyHostToDevice, s);
  const char* in = static_cast<const char*>(src);
  char* dst = static_cast<char*>(dst_dev);
  // Pieces go through the two chunks in turn, across calls: a chunk is
  // refilled only after its previous device copy has left it, so the host
  // copy of one piece overlaps the device copy of the one before. The
  // caller's buffer is no longer needed when this returns.
  for (size_t off = 0; off < bytes; off += kChunkBytes) {
    const size_t len = std::min(kChunkBytes, bytes - off);
    const int k = st->next;
    if (st->in_flight[k]) {
      const cudaError_t e = cudaEventSynchronize(st->done[k]);
      if (e != cudaSuccess) return e;
    }
    st->parallel_copy(st->chunk[k], in + off, len);
    cudaError_t e = cudaMemcpyAsync(dst + off, st->chunk[k], len, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(st->done[k], s);
    if (e != cudaSuccess) return e;
    st->in_flight[k] = true;
    st->next = k ^ 1;
  }
  return cudaSuccess;
}

}  // namespace hz
