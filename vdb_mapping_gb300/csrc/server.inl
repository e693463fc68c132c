// server.inl — continuous-batching request loop over a batch of maps
// (vdbg_server_*), included by vdb_gb300.cu.
//
// No counterpart in the reference, whose per-source worker threads
// (VDBMapping.hpp:1383-1430) each integrate one sensor's data into one map.
// Here every map stays resident in one device pool and one worker thread
// serves all sensor streams:
//   * submit() copies a scan into pinned staging and queues it on its map's
//     FIFO; it never waits for the GPU.
//   * The worker forms each step from the oldest queued scan of every map
//     that has one (so a map's scans are applied in submission order, one per
//     step), admits them against the device-memory budget, and inserts them
//     in one batched call. Scans that arrive while a step runs join the next
//     step: the batch is re-formed every step, not at fixed boundaries.
//   * poll() hands back completed requests with their submit, start and done
//     times (steady clock, ns) and status.
// A scan's result is the same whatever it is batched with: the batched call
// gives every map the result of inserting its scan alone.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>

namespace {

int64_t now_ns()
{
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
    .count();
}

// Device bytes one leaf slot costs: values, active mask, origin, flags, plus
// the batch channel's update masks and touched entry.
constexpr int64_t kLeafSlotBytes = 512 * 4 + 8 * 8 + 16 + 4 + 16 * 8 + 4;

struct ServerRequest
{
  uint64_t tag    = 0;
  int map         = 0;
  int64_t n       = 0;
  double origin[3] = {0, 0, 0};
  float* host     = nullptr;  // pinned, n * 16 bytes
  size_t cap      = 0;        // bytes of `host`
  int64_t submit_ns = 0;
};

// Pinned host buffers, reused by size (cudaMallocHost is slow and serialising).
class PinnedPool
{
public:
  ~PinnedPool()
  {
    for (auto& kv : free_) cudaFreeHost(kv.second);
  }
  float* acquire(size_t bytes, size_t* cap)
  {
    auto it = free_.lower_bound(bytes);
    if (it != free_.end() && it->first <= 2 * bytes)
    {
      float* p = it->second;
      *cap     = it->first;
      held_ -= it->first;
      free_.erase(it);
      return p;
    }
    size_t c = 4096;
    while (c < bytes) c <<= 1;
    void* p = nullptr;
    if (cudaMallocHost(&p, c) != cudaSuccess) return nullptr;
    *cap = c;
    return static_cast<float*>(p);
  }
  void release(float* p, size_t cap)
  {
    if (!p) return;
    if (held_ + cap > kMaxHeld)
    {
      cudaFreeHost(p);
      return;
    }
    free_.emplace(cap, p);
    held_ += cap;
  }

private:
  static constexpr size_t kMaxHeld = size_t(1) << 30;
  std::multimap<size_t, float*> free_;
  size_t held_ = 0;
};

} // namespace

struct vdbg_server
{
  vdbg_map* m = nullptr;
  vdbg_server_options opt{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<std::deque<ServerRequest>> pending;  // per map, FIFO
  std::deque<vdbg_server_result> done;
  size_t queued       = 0;
  bool stop           = false;
  PinnedPool pool;
  std::thread worker;
  // Admission: expected new leaves of a scan, per map (moving average).
  std::vector<double> new_leaves_est;
  vdbg_server_stats stats{};
};

namespace {

void server_complete(vdbg_server* sv, const ServerRequest& r, int status, int64_t start, int64_t end, int batch)
{
  vdbg_server_result res{};
  res.tag        = r.tag;
  res.map        = r.map;
  res.status     = status;
  res.points     = r.n;
  res.submit_ns  = r.submit_ns;
  res.start_ns   = start;
  res.done_ns    = end;
  res.batch_maps = batch;
  sv->done.push_back(res);
}

void server_loop(vdbg_server* sv)
{
  vdbg_map* m   = sv->m;
  const int nm  = static_cast<int>(m->conf.size());
  std::vector<ServerRequest> step;
  std::vector<const float*> parts(static_cast<size_t>(nm), nullptr);
  std::vector<int64_t> counts(static_cast<size_t>(nm), 0);
  std::vector<double> origins(static_cast<size_t>(nm) * 3, 0.0);
  cudaSetDevice(m->device);
  for (;;)
  {
    step.clear();
    {
      std::unique_lock<std::mutex> lock(sv->mu);
      sv->cv_work.wait(lock, [&] { return sv->stop || sv->queued > 0; });
      if (sv->queued == 0 && sv->stop) break;
      // Form the step: the head of every map's queue, within the budget.
      const int64_t budget = sv->opt.memory_budget_bytes;
      int64_t projected    = m->bytes;
      int64_t slots_free   = static_cast<int64_t>(m->capacity) - static_cast<int64_t>(m->n_leaves);
      const int max_maps   = sv->opt.max_batch_maps > 0 ? sv->opt.max_batch_maps : nm;
      for (int i = 0; i < nm && static_cast<int>(step.size()) < max_maps; ++i)
      {
        if (sv->pending[i].empty()) continue;
        const int64_t need = static_cast<int64_t>(sv->new_leaves_est[i] * 1.25) + 1;
        int64_t grow       = 0;
        // The pool grows in place by at least a quarter (grow_for).
        int64_t grow_slots = 0;
        if (need > slots_free) grow_slots = std::max<int64_t>(need - slots_free, static_cast<int64_t>(m->capacity) / 4);
        grow = grow_slots * kLeafSlotBytes;
        if (budget > 0 && projected + grow > budget && !step.empty()) continue;  // wait for a later step
        if (budget > 0 && projected + grow > budget)
        {
          // Nothing else is running that could make room: the map cannot grow.
          ServerRequest r = sv->pending[i].front();
          sv->pending[i].pop_front();
          --sv->queued;
          const int64_t t = now_ns();
          server_complete(sv, r, VDBG_ERR_OUT_OF_MEMORY, t, t, 0);
          sv->pool.release(r.host, r.cap);
          sv->stats.rejected += 1;
          continue;
        }
        projected += grow;
        slots_free = slots_free + grow_slots - need;
        step.push_back(sv->pending[i].front());
        sv->pending[i].pop_front();
        --sv->queued;
      }
      sv->cv_done.notify_all();
    }
    if (step.empty()) continue;
    std::fill(parts.begin(), parts.end(), nullptr);
    std::fill(counts.begin(), counts.end(), 0);
    for (const ServerRequest& r : step)
    {
      parts[r.map]           = r.host;
      counts[r.map]          = r.n;
      origins[3 * r.map + 0] = r.origin[0];
      origins[3 * r.map + 1] = r.origin[1];
      origins[3 * r.map + 2] = r.origin[2];
    }
    const uint32_t leaves_before = m->n_leaves;
    const int64_t t0             = now_ns();
    vdbg_scan_stats st{};
    const int status = batch_insert_impl(m, nullptr, parts.data(), counts.data(), 16, origins.data(), 0, m->stream,
                                         &st);
    const int64_t t1 = now_ns();
    {
      std::lock_guard<std::mutex> lock(sv->mu);
      int64_t total = 0;
      for (const ServerRequest& r : step) total += r.n;
      const double fresh = static_cast<double>(m->n_leaves - std::min(m->n_leaves, leaves_before));
      for (const ServerRequest& r : step)
      {
        // Split the step's new leaves over its scans by point count.
        const double share = total > 0 ? fresh * static_cast<double>(r.n) / static_cast<double>(total) : 0.0;
        sv->new_leaves_est[r.map] = 0.7 * sv->new_leaves_est[r.map] + 0.3 * share;
        server_complete(sv, r, status, t0, t1, static_cast<int>(step.size()));
        sv->pool.release(r.host, r.cap);
      }
      sv->stats.steps += 1;
      sv->stats.requests_done += step.size();
      sv->stats.rays += st.rays;
      sv->stats.updates += st.updates;
      sv->stats.busy_ns += t1 - t0;
      if (static_cast<int64_t>(step.size()) > sv->stats.max_step_maps) sv->stats.max_step_maps = step.size();
      sv->cv_done.notify_all();
    }
  }
}

} // namespace

extern "C" {

int vdbg_server_create(vdbg_map* batch, const vdbg_server_options* options, vdbg_server** out)
{
  if (!out) return VDBG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!batch || !batch->batch) return VDBG_ERR_INVALID_ARGUMENT;
  vdbg_server* sv = new vdbg_server();
  sv->m           = batch;
  if (options) sv->opt = *options;
  if (sv->opt.queue_capacity <= 0) sv->opt.queue_capacity = 4096;
  if (sv->opt.memory_budget_bytes > 0 &&
      (batch->max_bytes == 0 || batch->max_bytes > sv->opt.memory_budget_bytes))
    batch->max_bytes = sv->opt.memory_budget_bytes;
  sv->pending.resize(batch->conf.size());
  sv->new_leaves_est.assign(batch->conf.size(), 0.0);
  sv->worker = std::thread(server_loop, sv);
  *out       = sv;
  return VDBG_OK;
}

int vdbg_server_submit(vdbg_server* sv, int map, const float* xyz, int64_t n, int64_t stride, const double origin[3],
                       uint64_t tag)
{
  if (!sv || !origin || map < 0 || map >= static_cast<int>(sv->pending.size())) return VDBG_ERR_INVALID_ARGUMENT;
  if (bad_points(xyz, n, stride)) return VDBG_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    if (sv->stop) return VDBG_ERR_INVALID_ARGUMENT;
    if (static_cast<int64_t>(sv->queued) >= sv->opt.queue_capacity) return VDBG_ERR_BUSY;
  }
  ServerRequest r;
  r.tag       = tag;
  r.map       = map;
  r.n         = n;
  r.origin[0] = origin[0];
  r.origin[1] = origin[1];
  r.origin[2] = origin[2];
  r.submit_ns = now_ns();
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    r.host = sv->pool.acquire(static_cast<size_t>(std::max<int64_t>(n, 1)) * 16, &r.cap);
  }
  if (!r.host) return VDBG_ERR_OUT_OF_MEMORY;
  // Stage as pcl::PointXYZ rows (x, y, z, pad).
  const char* src = reinterpret_cast<const char*>(xyz);
  if (stride == 16)
  {
    std::memcpy(r.host, src, static_cast<size_t>(n) * 16);
  }
  else
  {
    for (int64_t i = 0; i < n; ++i)
    {
      const float* p  = reinterpret_cast<const float*>(src + i * stride);
      r.host[4 * i + 0] = p[0];
      r.host[4 * i + 1] = p[1];
      r.host[4 * i + 2] = p[2];
      r.host[4 * i + 3] = 0.f;
    }
  }
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->pending[map].push_back(r);
    ++sv->queued;
    sv->stats.requests_submitted += 1;
    if (static_cast<int64_t>(sv->queued) > sv->stats.max_queued) sv->stats.max_queued = sv->queued;
  }
  sv->cv_work.notify_one();
  return VDBG_OK;
}

int vdbg_server_poll(vdbg_server* sv, vdbg_server_result* out, int capacity, int wait_ms, int* n_out)
{
  if (!sv || !n_out || capacity < 0 || (capacity > 0 && !out)) return VDBG_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lock(sv->mu);
  if (sv->done.empty() && wait_ms > 0)
    sv->cv_done.wait_for(lock, std::chrono::milliseconds(wait_ms), [&] { return !sv->done.empty(); });
  int k = 0;
  while (k < capacity && !sv->done.empty())
  {
    out[k++] = sv->done.front();
    sv->done.pop_front();
  }
  *n_out = k;
  return VDBG_OK;
}

int vdbg_server_drain(vdbg_server* sv, int wait_ms)
{
  if (!sv) return VDBG_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lock(sv->mu);
  const auto until = std::chrono::steady_clock::now() + std::chrono::milliseconds(wait_ms);
  while (sv->queued > 0 || sv->stats.requests_done + sv->stats.rejected < sv->stats.requests_submitted)
  {
    if (sv->cv_done.wait_until(lock, until) == std::cv_status::timeout) return VDBG_ERR_TIMEOUT;
  }
  return VDBG_OK;
}

int vdbg_server_get_stats(vdbg_server* sv, vdbg_server_stats* out)
{
  if (!sv || !out) return VDBG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(sv->mu);
  *out        = sv->stats;
  out->queued = static_cast<int64_t>(sv->queued);
  out->device_bytes = sv->m->bytes;
  return VDBG_OK;
}

int vdbg_server_destroy(vdbg_server* sv)
{
  if (!sv) return VDBG_OK;
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  if (sv->worker.joinable()) sv->worker.join();
  for (auto& q : sv->pending)
    for (ServerRequest& r : q) sv->pool.release(r.host, r.cap);
  delete sv;
  return VDBG_OK;
}

} // extern "C"
