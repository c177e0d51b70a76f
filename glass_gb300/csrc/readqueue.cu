// Raw FITS read queue (RawFitsReadQueue, native_bindings.cpp:2605-2915):
// a pool of host threads that read byte ranges of files (the big-endian
// uint16 data units of FITS lights) into caller-owned buffers - normally
// pinned host memory that the decode + calibration entry points then copy to
// the device - and report completions in order of finishing.  Host code
// only; reads use pread on one descriptor per job, so jobs on different files
// run in parallel across the workers.
#include <fcntl.h>
#include <unistd.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

struct gg_read_queue {
  struct Job {
    uint64_t frame_index = 0;
    std::string path;
    uint64_t offset = 0;
    size_t bytes = 0;
    unsigned char* out = nullptr;
  };
  struct Done {
    uint64_t frame_index = 0;
    std::string path;
    uint64_t bytes_read = 0;
    double open_s = 0.0, read_s = 0.0, total_s = 0.0;
    std::string error;
  };

  std::mutex mutex;
  std::condition_variable job_cv, done_cv;
  std::deque<Job> jobs;
  std::deque<Done> done;
  std::vector<std::thread> workers;
  size_t active = 0;
  bool closing = false;
  bool joined = false;
  uint64_t submitted = 0, completed = 0, requested_bytes = 0;

  explicit gg_read_queue(int count) {
    const int n = count <= 0 ? 1 : count;
    for (int i = 0; i < n; ++i) workers.emplace_back([this]() { loop(); });
  }

  static double since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  void loop() {
    for (;;) {
      Job job;
      {
        std::unique_lock<std::mutex> lock(mutex);
        job_cv.wait(lock, [this]() { return closing || !jobs.empty(); });
        if (jobs.empty()) return;  // closing and drained
        job = std::move(jobs.front());
        jobs.pop_front();
        ++active;
      }
      Done d;
      d.frame_index = job.frame_index;
      d.path = job.path;
      const auto t0 = std::chrono::steady_clock::now();
      const int fd = ::open(job.path.c_str(), O_RDONLY);
      d.open_s = since(t0);
      if (fd < 0) {
        d.error = std::string("open failed: ") + std::strerror(errno);
      } else {
        const auto t1 = std::chrono::steady_clock::now();
        size_t got = 0;
        while (got < job.bytes) {
          const ssize_t r = ::pread(fd, job.out + got, job.bytes - got, static_cast<off_t>(job.offset + got));
          if (r < 0) {
            if (errno == EINTR) continue;
            d.error = std::string("read failed: ") + std::strerror(errno);
            break;
          }
          if (r == 0) {
            d.error = "file ended " + std::to_string(job.bytes - got) + " bytes before the requested range";
            break;
          }
          got += static_cast<size_t>(r);
        }
        d.read_s = since(t1);
        d.bytes_read = got;
        ::close(fd);
      }
      d.total_s = since(t0);
      {
        std::lock_guard<std::mutex> lock(mutex);
        --active;
        ++completed;
        done.push_back(std::move(d));
      }
      done_cv.notify_all();
    }
  }

  void close_and_join() {
    {
      std::lock_guard<std::mutex> lock(mutex);
      if (closing && joined) return;
      closing = true;
    }
    job_cv.notify_all();
    done_cv.notify_all();
    for (auto& w : workers)
      if (w.joinable()) w.join();
    {
      std::lock_guard<std::mutex> lock(mutex);
      joined = true;
    }
    done_cv.notify_all();
  }

  ~gg_read_queue() { close_and_join(); }
};

using namespace gg;

extern "C" {

int gg_read_queue_create(int32_t workers, gg_read_queue** out) {
  GG_API_BEGIN
  require(out != nullptr, "null argument");
  require(workers >= 0 && workers <= 256, "worker_count must be in [0, 256] (0 means 1)");
  *out = new gg_read_queue(workers);
  GG_API_END
}

int gg_read_queue_submit(gg_read_queue* q, uint64_t frame_index, const char* path, uint64_t data_offset,
                         uint64_t byte_count, void* host_out, uint64_t* pending_after) {
  GG_API_BEGIN
  require(q != nullptr && path != nullptr && host_out != nullptr, "null argument");
  require(byte_count > 0, "native raw FITS queue byte count must be non-empty");
  gg_read_queue::Job job;
  job.frame_index = frame_index;
  job.path = path;
  job.offset = data_offset;
  job.bytes = static_cast<size_t>(byte_count);
  job.out = static_cast<unsigned char*>(host_out);
  size_t pending = 0;
  {
    std::lock_guard<std::mutex> lock(q->mutex);
    if (q->closing) fail(GG_ERR_RUNTIME, "native raw FITS queue is closed");
    q->requested_bytes += byte_count;
    q->jobs.push_back(std::move(job));
    ++q->submitted;
    pending = q->jobs.size() + q->active;
  }
  q->job_cv.notify_one();
  if (pending_after) *pending_after = pending;
  GG_API_END
}

int gg_read_queue_wait(gg_read_queue* q, double timeout_s, gg_read_completion_t* out, int32_t* has_completion) {
  GG_API_BEGIN
  require(q != nullptr && out != nullptr && has_completion != nullptr, "null argument");
  *has_completion = 0;
  gg_read_queue::Done d;
  {
    std::unique_lock<std::mutex> lock(q->mutex);
    const auto ready = [q]() { return !q->done.empty() || (q->closing && q->jobs.empty() && q->active == 0); };
    if (timeout_s < 0.0) {
      q->done_cv.wait(lock, ready);
    } else if (!q->done_cv.wait_for(lock, std::chrono::duration<double>(timeout_s), ready)) {
      return GG_OK;  // timed out: no completion
    }
    if (q->done.empty()) return GG_OK;
    d = std::move(q->done.front());
    q->done.pop_front();
  }
  std::memset(out, 0, sizeof(*out));
  out->frame_index = d.frame_index;
  out->bytes_read = d.bytes_read;
  out->file_open_s = d.open_s;
  out->file_read_s = d.read_s;
  out->total_s = d.total_s;
  *has_completion = 1;
  if (!d.error.empty())
    fail(GG_ERR_RUNTIME, "native raw FITS queue read failed for frame " + std::to_string(d.frame_index) + " (" +
                             d.path + "): " + d.error);
  GG_API_END
}

int gg_read_queue_stats(gg_read_queue* q, gg_read_queue_stats_t* out) {
  GG_API_BEGIN
  require(q != nullptr && out != nullptr, "null argument");
  std::lock_guard<std::mutex> lock(q->mutex);
  out->worker_count = static_cast<uint64_t>(q->workers.size());
  out->submitted_count = q->submitted;
  out->completed_count = q->completed;
  out->queued_count = static_cast<uint64_t>(q->jobs.size());
  out->active_count = static_cast<uint64_t>(q->active);
  out->ready_count = static_cast<uint64_t>(q->done.size());
  out->requested_bytes = q->requested_bytes;
  out->closed = q->closing ? 1 : 0;
  out->pad = 0;
  GG_API_END
}

int gg_read_queue_close(gg_read_queue* q) {
  GG_API_BEGIN
  require(q != nullptr, "null argument");
  q->close_and_join();
  GG_API_END
}

int gg_read_queue_destroy(gg_read_queue* q) {
  GG_API_BEGIN
  delete q;
  GG_API_END
}

}  // extern "C"
