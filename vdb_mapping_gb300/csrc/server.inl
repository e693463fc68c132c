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
//   * Steps are pipelined over two sets of scan buffers: while the device
//     marks and sweeps step k, the worker forms step k + 1 from what has
//     arrived, and its upload and ray preparation (clip, quantise, sort) run
//     on a second stream beside step k's kernels. Step k + 1's marking waits
//     only for its own preparation and for step k's end (the update grid and
//     the pools are step k's until then), so its scans see the same map as
//     without the overlap.
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

// One step's scan buffers on the device: points, ray records, the ray order
// and the scan table, with the status block the preparation counts into.
struct PrepSet
{
  char* pts          = nullptr;
  size_t pts_cap     = 0;
  int4* rays         = nullptr;
  int* order         = nullptr;
  uint16_t* ray_scan = nullptr;
  size_t ray_cap     = 0;
  uint32_t* hist     = nullptr;
  uint32_t* cursor   = nullptr;
  ScanGeom* geom     = nullptr;
  uint32_t* first    = nullptr;
  ScanGeom* h_geom   = nullptr;  // pinned staging of geom and first
  uint32_t* h_first  = nullptr;
  DevStatus* st      = nullptr;
  cudaEvent_t ready  = nullptr;  // the preparation is complete
  ScanTable table{};
  int64_t total      = 0;
  int status         = VDBG_OK;  // a step that cannot be cast (an origin out of range)
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
  PrepSet prep[2];
  cudaStream_t prep_stream = nullptr;
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

// Forms a step from the head of every map's queue, within the memory budget
// (the caller holds sv->mu). Scans that cannot fit even alone are completed
// with OUT_OF_MEMORY.
void form_step(vdbg_server* sv, std::vector<ServerRequest>& step)
{
  vdbg_map* m          = sv->m;
  const int nm         = static_cast<int>(m->conf.size());
  const int64_t budget = sv->opt.memory_budget_bytes;
  int64_t projected    = m->bytes;
  int64_t slots_free   = static_cast<int64_t>(m->capacity) - static_cast<int64_t>(m->n_leaves);
  const int max_maps   = sv->opt.max_batch_maps > 0 ? sv->opt.max_batch_maps : nm;
  step.clear();
  for (int i = 0; i < nm && static_cast<int>(step.size()) < max_maps; ++i)
  {
    if (sv->pending[i].empty()) continue;
    const int64_t need = static_cast<int64_t>(sv->new_leaves_est[i] * 1.25) + 1;
    // The pool grows in place by at least a quarter (grow_for).
    int64_t grow_slots = 0;
    if (need > slots_free) grow_slots = std::max<int64_t>(need - slots_free, static_cast<int64_t>(m->capacity) / 4);
    const int64_t grow = grow_slots * kLeafSlotBytes;
    if (budget > 0 && projected + grow > budget && !step.empty()) continue;  // wait for a later step
    if (budget > 0 && projected + grow > budget)
    {
      // Nothing else is in the step that could be dropped: the map cannot grow.
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

void free_prep(vdbg_map* m, PrepSet& p)
{
  dev_free(m, p.pts, p.pts_cap);
  dev_free(m, p.rays, p.ray_cap);
  dev_free(m, p.order, p.ray_cap);
  dev_free(m, p.ray_scan, p.ray_cap);
  dev_free(m, p.hist, m->buckets);
  dev_free(m, p.cursor, m->buckets + kScanMaxTiles);
  dev_free(m, p.geom, m->conf.size());
  dev_free(m, p.first, m->conf.size() + 1);
  dev_free(m, p.st, 1);
  if (p.h_geom) cudaFreeHost(p.h_geom);
  if (p.h_first) cudaFreeHost(p.h_first);
  if (p.ready) cudaEventDestroy(p.ready);
  p = PrepSet{};
}

// Buffers of a step of `total` points (grown on demand).
int ensure_prep(vdbg_map* m, PrepSet& p, int64_t total)
{
  const size_t nm = m->conf.size();
  if (!p.st)
  {
    VDBG_TRY(dev_alloc(m, &p.st, 1));
    VDBG_TRY(dev_alloc(m, &p.hist, m->buckets));
    VDBG_TRY(dev_alloc(m, &p.cursor, m->buckets + kScanMaxTiles));
    VDBG_TRY(dev_alloc(m, &p.geom, nm));
    VDBG_TRY(dev_alloc(m, &p.first, nm + 1));
    VDBG_CUDA(cudaMemset(p.hist, 0, m->buckets * sizeof(uint32_t)));
    if (cudaMallocHost(reinterpret_cast<void**>(&p.h_geom), sizeof(ScanGeom) * nm) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void**>(&p.h_first), sizeof(uint32_t) * (nm + 1)) != cudaSuccess)
      return VDBG_ERR_OUT_OF_MEMORY;
    VDBG_CUDA(cudaEventCreateWithFlags(&p.ready, cudaEventDisableTiming));
  }
  const size_t need_pts = static_cast<size_t>(total) * 16;
  if (need_pts > p.pts_cap)
  {
    dev_free(m, p.pts, p.pts_cap);
    p.pts_cap = 0;
    const size_t cap = std::max(need_pts, p.pts_cap * 3 / 2);
    VDBG_TRY(dev_alloc(m, &p.pts, cap));
    p.pts_cap = cap;
  }
  if (static_cast<size_t>(total) > p.ray_cap)
  {
    dev_free(m, p.rays, p.ray_cap);
    dev_free(m, p.order, p.ray_cap);
    dev_free(m, p.ray_scan, p.ray_cap);
    p.ray_cap        = 0;
    const size_t cap = static_cast<size_t>(total) + static_cast<size_t>(total) / 2;
    VDBG_TRY(dev_alloc(m, &p.rays, cap));
    VDBG_TRY(dev_alloc(m, &p.order, cap));
    VDBG_TRY(dev_alloc(m, &p.ray_scan, cap));
    p.ray_cap = cap;
  }
  return VDBG_OK;
}

// Queues a step's upload and ray preparation (VDBMapping.hpp:499-519 for
// every point: clip, quantise, sort) on stream `ps` into buffer set `p`. The
// kernels only touch `p`, so they may run beside another step's marking.
int queue_prep(vdbg_map* m, PrepSet& p, const std::vector<ServerRequest>& step, cudaStream_t ps)
{
  const int nm = static_cast<int>(m->conf.size());
  p.status     = VDBG_OK;
  p.total      = 0;
  std::vector<int64_t> counts(static_cast<size_t>(nm), 0);
  std::vector<const ServerRequest*> by_map(static_cast<size_t>(nm), nullptr);
  for (const ServerRequest& r : step)
  {
    counts[r.map] = r.n;
    by_map[r.map] = &r;
    p.total += r.n;
  }
  VDBG_TRY(ensure_prep(m, p, std::max<int64_t>(p.total, 1)));
  p.h_first[0] = 0;
  for (int i = 0; i < nm; ++i)
  {
    p.h_first[i + 1] = p.h_first[i] + static_cast<uint32_t>(counts[i]);
    ScanGeom g{};
    bool coord_range   = false;
    const double range = m->conf[i].max_range;
    if (counts[i] > 0 && range > 0 && scan_geom_for(m, i, by_map[i]->origin, range, &g, &coord_range))
    {
    }
    else
    {
      // An origin outside the index range fails the whole step unmarked, as
      // the batched call does.
      if (coord_range) p.status = VDBG_ERR_COORD_RANGE;
      g     = ScanGeom{};
      g.map = -1;
    }
    p.h_geom[i] = g;
  }
  ScanTable t{};
  if (nm == 1)
  {
    t = single_table(p.h_geom[0]);
  }
  else
  {
    t.n        = nm;
    t.geom     = p.geom;
    t.first    = p.first;
    t.ray_scan = p.ray_scan;
  }
  set_edges(m, t);
  p.table = t;
  if (p.status != VDBG_OK || p.total == 0) return VDBG_OK;
  for (const ServerRequest& r : step)
    VDBG_CUDA(cudaMemcpyAsync(p.pts + static_cast<size_t>(p.h_first[r.map]) * 16, r.host,
                              static_cast<size_t>(r.n) * 16, cudaMemcpyHostToDevice, ps));
  if (nm > 1)
  {
    VDBG_CUDA(cudaMemcpyAsync(p.geom, p.h_geom, sizeof(ScanGeom) * nm, cudaMemcpyHostToDevice, ps));
    VDBG_CUDA(cudaMemcpyAsync(p.first, p.h_first, sizeof(uint32_t) * (nm + 1), cudaMemcpyHostToDevice, ps));
  }
  VDBG_CUDA(cudaMemsetAsync(p.st, 0, sizeof(DevStatus), ps));
  const unsigned blocks = static_cast<unsigned>((p.total + 255) / 256);
  k_prep<<<blocks, 256, 0, ps>>>(p.pts, nullptr, p.total, 16, t, p.rays, nm > 1 ? p.ray_scan : nullptr, p.hist,
                                 p.st);
  launch_scan(p.hist, p.cursor, static_cast<uint32_t>(kBucketsPerScan * t.n), p.st, ps);
  k_scatter<<<blocks, 256, 0, ps>>>(p.rays, p.total, t, p.cursor, p.order);
  VDBG_CUDA(cudaGetLastError());
  VDBG_CUDA(cudaEventRecord(p.ready, ps));
  return VDBG_OK;
}

// The marking and sweep of a prepared step (the batched insertion's, from
// the rays in `p`), on the map's stream.
int run_prepped(vdbg_map* m, PrepSet& p, vdbg_scan_stats* stats)
{
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (p.status != VDBG_OK) return p.status;
  cudaStream_t s = m->stream;
  Channel& c     = m->channels[0];
  VDBG_TRY(begin_call(m, s));
  const uint32_t leaves_before = m->n_leaves;
  if (p.total == 0) return VDBG_OK;
  uint32_t seg = std::max<uint32_t>(m->run_seg, kMinRunSeg);
  if (m->passes_last > 1)
  {
    const uint64_t want  = static_cast<uint64_t>(m->run_seg) * m->passes_last * 2;
    const uint64_t limit = m->run_budget / (17ull * m->dda_warps);
    seg                  = static_cast<uint32_t>(std::min<uint64_t>(want, limit));
  }
  VDBG_TRY(ensure_runs(m, seg));
  const RunBuffer rb =
    run_buffer(m, m->run_key, m->run_bits, m->run_slab, m->run_count, m->run_prefix, m->run_seg, m->dda_warps);
  VDBG_CUDA(cudaStreamWaitEvent(s, p.ready, 0));
  k_absorb_prep<<<1, 1, 0, s>>>(m->d_status, p.st);
  VDBG_CUDA(cudaGetLastError());
  c.pending  = true;
  bool swept = false;
  int d = run_dda_passes(m, c, p.rays, p.order, p.total, p.table, rb, m->lstate, m->wstate, true, s, true, &swept);
  int call_status = VDBG_OK;
  if (d == VDBG_OK && swept)
  {
    record_timings(m);
    fill_stats(m, leaves_before, stats);
    VDBG_TRY(end_call(m, s));
    return VDBG_OK;
  }
  if (d == VDBG_ERR_COORD_RANGE)
  {
    call_status = d;
  }
  else if (d != VDBG_OK)
  {
    if (d != VDBG_ERR_CUDA) discard_marking(m, c, s);
    return d;
  }
  VDBG_TRY(reset_changes(m, s));
  if (c.pending) VDBG_TRY(launch_sweep(m, c, s));
  VDBG_TRY(fetch_status(m, s));
  if (m->h_status->error != 0u) return map_error(m->h_status->error);
  record_timings(m);
  VDBG_TRY(finish_sweep(m, c, s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  fill_stats(m, leaves_before, stats);
  VDBG_TRY(end_call(m, s));
  return call_status;
}

void server_loop(vdbg_server* sv)
{
  vdbg_map* m = sv->m;
  cudaSetDevice(m->device);
  std::vector<ServerRequest> step[2];
  int prep_status[2] = {VDBG_OK, VDBG_OK};
  int cur            = 0;
  bool have_cur      = false;
  for (;;)
  {
    if (!have_cur)
    {
      {
        std::unique_lock<std::mutex> lock(sv->mu);
        sv->cv_work.wait(lock, [&] { return sv->stop || sv->queued > 0; });
        if (sv->queued == 0 && sv->stop) break;
        form_step(sv, step[cur]);
      }
      if (step[cur].empty()) continue;
      prep_status[cur] = queue_prep(m, sv->prep[cur], step[cur], sv->prep_stream);
    }
    // While the device runs this step, the next one is formed from what has
    // arrived and prepared on the second stream.
    const int nxt  = cur ^ 1;
    bool have_next = false;
    m->pre_wait    = [&]() {
      {
        std::lock_guard<std::mutex> lock(sv->mu);
        if (sv->queued == 0) return;
        form_step(sv, step[nxt]);
      }
      if (step[nxt].empty()) return;
      prep_status[nxt] = queue_prep(m, sv->prep[nxt], step[nxt], sv->prep_stream);
      have_next        = true;
    };
    const int64_t t0 = now_ns();
    vdbg_scan_stats st{};
    const uint32_t leaves_before = m->n_leaves;
    const int status = prep_status[cur] != VDBG_OK ? prep_status[cur] : run_prepped(m, sv->prep[cur], &st);
    const int64_t t1 = now_ns();
    m->pre_wait      = nullptr;
    {
      std::lock_guard<std::mutex> lock(sv->mu);
      int64_t total = 0;
      for (const ServerRequest& r : step[cur]) total += r.n;
      const double fresh = static_cast<double>(m->n_leaves - std::min(m->n_leaves, leaves_before));
      for (const ServerRequest& r : step[cur])
      {
        // Split the step's new leaves over its scans by point count.
        const double share = total > 0 ? fresh * static_cast<double>(r.n) / static_cast<double>(total) : 0.0;
        sv->new_leaves_est[r.map] = 0.7 * sv->new_leaves_est[r.map] + 0.3 * share;
        server_complete(sv, r, status, t0, t1, static_cast<int>(step[cur].size()));
        sv->pool.release(r.host, r.cap);
      }
      sv->stats.steps += 1;
      sv->stats.requests_done += step[cur].size();
      sv->stats.rays += st.rays;
      sv->stats.updates += st.updates;
      sv->stats.busy_ns += t1 - t0;
      if (have_next) sv->stats.overlapped_steps += 1;
      if (static_cast<int64_t>(step[cur].size()) > sv->stats.max_step_maps) sv->stats.max_step_maps = step[cur].size();
      sv->cv_done.notify_all();
    }
    step[cur].clear();
    cur      = nxt;
    have_cur = have_next;
  }
  cudaStreamSynchronize(sv->prep_stream);
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
  if (cudaSetDevice(batch->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&sv->prep_stream, cudaStreamNonBlocking) != cudaSuccess)
  {
    delete sv;
    return VDBG_ERR_CUDA;
  }
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
  cudaSetDevice(sv->m->device);
  for (PrepSet& p : sv->prep) free_prep(sv->m, p);
  if (sv->prep_stream) cudaStreamDestroy(sv->prep_stream);
  delete sv;
  return VDBG_OK;
}

} // extern "C"
