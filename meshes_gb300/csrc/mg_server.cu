// Native continuous-batching scheduler over resident meshes (the C side of meshes_gb300.serve).
//
// A scheduler thread owned by the server runs ticks.  Each tick:
//   * retires finished ticks (CUDA events, in order): copies each request's results from the tick's
//     pinned staging buffer to the caller's output buffers, frees the tick's arena span and staging
//     buffer, and publishes the request tags as completed;
//   * admits queued requests, oldest first, while their device buffers fit in the largest free span of
//     a fixed device arena (admission by free device memory) and the tick has slots left;
//   * packs them: one pinned staging buffer holds the per-request descriptors and work items (items
//     sorted longest first), the queue heads and the inputs; one host->device copy, one persistent
//     forward launch over all admitted requests (mg_batched_propagate), one persistent back-propagation
//     launch and a deterministic gradient reduction for the gradient requests, one device->host copy of
//     every result, one event;
//   * rotates over several streams, so a tick starts while earlier ones are still on the GPU; at most
//     one tick per stream is in flight, so under load the queue gathers requests into larger ticks.
// Each request's work items cover only its own vectors, so its result does not depend on the mix.
// Clients submit from any thread; mg_server_wait blocks (without the caller holding any lock) until
// tags complete.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/meshes_gb300.h"
#include "mg_launch.h"

namespace {

constexpr size_t kAlign = 256;
size_t al(size_t n) { return (n + kAlign - 1) / kAlign * kAlign; }

struct Req {
  unsigned long long tag;
  int mesh, b;
  const void* x;
  const void* gy;
  void* y;
  float* dp;
  void* gx;
  size_t bytes;       // device bytes (admission)
};

struct Tick {
  std::vector<Req> reqs;
  cudaEvent_t ev = nullptr;
  size_t dev_off = 0, dev_bytes = 0;
  unsigned char* host = nullptr;
  size_t host_cap = 0;
  std::vector<size_t> o_y, o_dp, o_gx;    // host offsets of each request's results (dp, gx: gradient requests)
};

struct Arena {
  size_t size = 0;
  std::vector<std::pair<size_t, size_t>> free_;   // (offset, length), sorted by offset
  void init(size_t n) { size = n; free_.assign(1, {0, n}); }
  bool alloc(size_t n, size_t* off) {
    n = al(n);
    for (size_t i = 0; i < free_.size(); ++i)
      if (free_[i].second >= n) {
        *off = free_[i].first;
        if (free_[i].second == n) free_.erase(free_.begin() + i);
        else free_[i] = {free_[i].first + n, free_[i].second - n};
        return true;
      }
    return false;
  }
  void release(size_t off, size_t n) {
    n = al(n);
    free_.push_back({off, n});
    std::sort(free_.begin(), free_.end());
    std::vector<std::pair<size_t, size_t>> m;
    for (auto& f : free_) {
      if (!m.empty() && m.back().first + m.back().second == f.first) m.back().second += f.second;
      else m.push_back(f);
    }
    free_.swap(m);
  }
  size_t largest() const {
    size_t l = 0;
    for (auto& f : free_) l = std::max(l, f.second);
    return l;
  }
};

}  // namespace

struct mg_server {
  std::vector<mg_server_mesh> meshes;
  int device = 0, grid = 0, max_per_tick = 512;
  size_t smem_fwd = 0, smem_bwd = 0;
  unsigned char* arena_dev = nullptr;
  Arena arena;
  int* status = nullptr;
  std::vector<cudaStream_t> streams;
  int next_stream = 0;
  std::vector<std::pair<unsigned char*, size_t>> pinned_free;
  std::vector<unsigned char*> pinned_all;   // every staging buffer, freed by mg_server_destroy

  std::mutex qmu;
  std::condition_variable qcv;
  std::deque<Req> queue;
  bool running = true;

  std::mutex dmu;
  std::condition_variable dcv;
  std::vector<unsigned long long> done;
  std::string error;                     // guarded by dmu
  std::atomic<bool> failed{false};

  std::deque<Tick> inflight;             // scheduler thread only
  std::atomic<long long> completed{0}, ticks{0}, queued{0};
  std::thread worker;

  size_t request_bytes(const mg_server_mesh& m, int b, bool grad) const {
    const size_t fe = al((size_t)b * m.N * (m.cls == MG_BCLS_R8 ? 4 : 8));
    if (!grad) return 2 * fe;
    const size_t n_items = (size_t)(b + m.cap - 1) / m.cap;
    const size_t np2 = (size_t)m.G * (m.cls == MG_BCLS_C16 ? 16 : 8) / 2;
    return 4 * fe + al((size_t)m.L * (m.N / 2) * m.n_p * 4) + al(n_items * m.L * np2 * 8);
  }

  unsigned char* pinned_get(size_t n, size_t* cap) {
    for (size_t i = 0; i < pinned_free.size(); ++i)
      if (pinned_free[i].second >= n) {
        auto p = pinned_free[i];
        pinned_free.erase(pinned_free.begin() + i);
        *cap = p.second;
        return p.first;
      }
    const size_t c = std::max(n, (size_t)1 << 20);
    void* p = nullptr;
    if (cudaHostAlloc(&p, c, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    *cap = c;
    pinned_all.push_back(static_cast<unsigned char*>(p));
    return static_cast<unsigned char*>(p);
  }

  // A failed tick (launch or CUDA error) stops the scheduler: queued requests are dropped and every
  // waiter learns of the failure from mg_server_wait; the client fails its pending requests.
  void fail_all(const std::string& why) {
    {
      std::lock_guard<std::mutex> lk(qmu);
      queued -= (long long)queue.size();
      queue.clear();
    }
    std::lock_guard<std::mutex> lk(dmu);
    if (error.empty()) error = why;
    failed = true;
    dcv.notify_all();
  }

  bool retire() {
    bool any = false;
    while (!inflight.empty()) {
      Tick& t = inflight.front();
      const cudaError_t q = cudaEventQuery(t.ev);
      if (q == cudaErrorNotReady) break;
      if (q != cudaSuccess) {
        fail_all(std::string("tick failed: ") + cudaGetErrorString(q));
        return false;
      }
      std::vector<unsigned long long> tags;
      size_t g = 0;
      for (size_t i = 0; i < t.reqs.size(); ++i) {
        const Req& r = t.reqs[i];
        const mg_server_mesh& m = meshes[r.mesh];
        const size_t fb = (size_t)r.b * m.N * (m.cls == MG_BCLS_R8 ? 4 : 8);
        std::memcpy(r.y, t.host + t.o_y[i], fb);
        if (r.gy) {
          std::memcpy(r.dp, t.host + t.o_dp[g], (size_t)m.L * (m.N / 2) * m.n_p * 4);
          std::memcpy(r.gx, t.host + t.o_gx[g], fb);
          ++g;
        }
        tags.push_back(r.tag);
      }
      arena.release(t.dev_off, t.dev_bytes);
      pinned_free.push_back({t.host, t.host_cap});
      cudaEventDestroy(t.ev);
      completed += (long long)t.reqs.size();
      inflight.pop_front();
      {
        std::lock_guard<std::mutex> lk(dmu);
        done.insert(done.end(), tags.begin(), tags.end());
      }
      dcv.notify_all();
      any = true;
    }
    return any;
  }

  bool launch_tick() {
    // at most one tick in flight per stream: under load requests gather in the queue meanwhile, so
    // ticks grow with the load instead of the GPU paying per-tick overheads for every arrival
    if (inflight.size() >= streams.size()) return false;
    std::vector<Req> reqs;
    {
      std::lock_guard<std::mutex> lk(qmu);
      if (queue.empty()) return false;
      const size_t largest = arena.largest();
      const size_t room = largest > 65536 ? largest - 65536 : 0;   // descriptors and items: 64 KB + 2 KB/request
      size_t need = 0;
      while (!queue.empty() && (int)reqs.size() < max_per_tick) {
        const Req& r = queue.front();
        if (need + r.bytes + 2048 * (reqs.size() + 1) > room) break;   // wait for ticks to retire
        need += r.bytes;
        reqs.push_back(r);
        queue.pop_front();
      }
      queued -= (long long)reqs.size();
    }
    if (reqs.empty()) return false;
    pack(std::move(reqs));
    return true;
  }

  void pack(std::vector<Req> reqs) {
    const size_t K = reqs.size();
    std::vector<size_t> gidx;
    for (size_t i = 0; i < K; ++i)
      if (reqs[i].gy) gidx.push_back(i);
    const size_t KG = gidx.size();
    std::vector<size_t> fe(K), nit(K), np2(K);
    size_t n_if = 0, n_ib = 0, n_x = 0, n_gy = 0, n_dp = 0, n_pt = 0;
    for (size_t i = 0; i < K; ++i) {
      const mg_server_mesh& m = meshes[reqs[i].mesh];
      fe[i] = al((size_t)reqs[i].b * m.N * (m.cls == MG_BCLS_R8 ? 4 : 8));
      nit[i] = (size_t)(reqs[i].b + m.cap - 1) / m.cap;
      np2[i] = (size_t)m.G * (m.cls == MG_BCLS_C16 ? 16 : 8) / 2;
      n_if += nit[i];
      n_x += fe[i];
      if (reqs[i].gy) {
        n_ib += nit[i];
        n_gy += fe[i];
        n_dp += al((size_t)m.L * (m.N / 2) * m.n_p * 4);
        n_pt += al(nit[i] * m.L * np2[i] * 8);
      }
    }
    const size_t off_df = 0;
    const size_t off_db = off_df + al(K * sizeof(mg_batch_mesh));
    const size_t off_if = off_db + al(std::max<size_t>(KG, 1) * sizeof(mg_batch_mesh));
    const size_t off_ib = off_if + al(std::max<size_t>(n_if, 1) * sizeof(mg_batch_item));
    const size_t off_head = off_ib + al(std::max<size_t>(n_ib, 1) * sizeof(mg_batch_item));
    const size_t off_x = off_head + kAlign;
    const size_t off_gy = off_x + n_x;
    const size_t in_bytes = off_gy + n_gy;
    const size_t off_y = in_bytes;
    const size_t off_gx = off_y + n_x;
    const size_t off_dp = off_gx + n_gy;
    const size_t out_end = off_dp + n_dp;
    const size_t off_pt = out_end;
    const size_t total = off_pt + n_pt;
    size_t dev_off = 0;
    if (!arena.alloc(total, &dev_off)) {   // fragmentation: put the requests back in front
      std::lock_guard<std::mutex> lk(qmu);
      for (size_t i = K; i-- > 0;) queue.push_front(reqs[i]);
      queued += (long long)K;
      return;
    }
    Tick t;
    t.host = pinned_get(total, &t.host_cap);
    if (!t.host) {
      arena.release(dev_off, total);
      fail_all("cudaHostAlloc failed");
      return;
    }
    unsigned char* h = t.host;
    unsigned char* base = arena_dev + dev_off;
    auto* df = reinterpret_cast<mg_batch_mesh*>(h + off_df);
    auto* db = reinterpret_cast<mg_batch_mesh*>(h + off_db);
    std::memset(h, 0, off_x);                          // descriptors, items, queue heads
    struct It {
      size_t cost;
      int mesh, v0, vend, part;
    };
    std::vector<It> itf, itb;
    itf.reserve(n_if);
    itb.reserve(n_ib);
    size_t ox = 0, og = 0, odp = 0, opt = 0;
    t.o_y.resize(K);
    for (size_t i = 0, j = 0; i < K; ++i) {
      const Req& r = reqs[i];
      const mg_server_mesh& m = meshes[r.mesh];
      const size_t fb = (size_t)r.b * m.N * (m.cls == MG_BCLS_R8 ? 4 : 8);
      std::memcpy(h + off_x + ox, r.x, fb);
      mg_batch_mesh& d = df[i];
      d.N = m.N; d.L = m.L; d.B = r.b; d.ldu = m.N;
      d.cls = m.cls; d.G = m.G; d.CL = m.fwd_CL; d.S = m.fwd_S;
      d.layer_bytes = m.fwd_layer_bytes; d.n_items = 0; d.ldp = 0; d.n_p = m.n_p;
      d.tiles = m.fwd_tiles; d.kinds = m.fwd_kinds;
      d.in0 = base + off_x + ox; d.out0 = base + off_y + ox;
      t.o_y[i] = off_y + ox;
      const size_t cost = (size_t)m.L * np2[i] * m.cap;
      for (size_t k = 0; k < nit[i]; ++k)
        itf.push_back({cost, (int)i, (int)(k * m.cap), (int)std::min<size_t>((k + 1) * m.cap, r.b), (int)k});
      if (r.gy) {
        std::memcpy(h + off_gy + og, r.gy, fb);
        mg_batch_mesh& e = db[j];
        e = d;
        e.CL = m.bwd_CL; e.S = m.bwd_S; e.layer_bytes = m.bwd_layer_bytes;
        e.tiles = m.bwd_tiles; e.kinds = m.bwd_kinds;
        e.n_items = (int)nit[i]; e.ldp = m.N / 2 * m.n_p;
        e.in0 = base + off_y + ox; e.in1 = base + off_gy + og; e.out0 = nullptr; e.out1 = base + off_gx + og;
        e.dp = reinterpret_cast<float*>(base + off_dp + odp); e.partial = base + off_pt + opt;
        t.o_gx.push_back(off_gx + og);
        t.o_dp.push_back(off_dp + odp);
        for (size_t k = 0; k < nit[i]; ++k)
          itb.push_back({cost, (int)j, (int)(k * m.cap), (int)std::min<size_t>((k + 1) * m.cap, r.b), (int)k});
        og += fe[i];
        odp += al((size_t)m.L * (m.N / 2) * m.n_p * 4);
        opt += al(nit[i] * m.L * np2[i] * 8);
        ++j;
      }
      ox += fe[i];
    }
    auto by_cost = [](const It& a, const It& b) { return a.cost > b.cost; };
    std::stable_sort(itf.begin(), itf.end(), by_cost);
    std::stable_sort(itb.begin(), itb.end(), by_cost);
    auto* if_ = reinterpret_cast<mg_batch_item*>(h + off_if);
    auto* ib_ = reinterpret_cast<mg_batch_item*>(h + off_ib);
    for (size_t n = 0; n < itf.size(); ++n) if_[n] = mg_batch_item{itf[n].mesh, itf[n].v0, itf[n].vend, itf[n].part};
    for (size_t n = 0; n < itb.size(); ++n) ib_[n] = mg_batch_item{itb[n].mesh, itb[n].v0, itb[n].vend, itb[n].part};

    cudaStream_t st = streams[next_stream];
    next_stream = (next_stream + 1) % (int)streams.size();
    cudaError_t e = cudaMemcpyAsync(base, h, in_bytes, cudaMemcpyHostToDevice, st);
    int head_rc = MG_OK;
    int* head = reinterpret_cast<int*>(base + off_head);
    if (e == cudaSuccess)
      head_rc = mg_batched_propagate(MG_OP_FWD, reinterpret_cast<const mg_batch_mesh*>(base + off_df), (int)K,
                                     reinterpret_cast<const mg_batch_item*>(base + off_if), (int)n_if, head, grid,
                                     smem_fwd, status, st);
    if (e == cudaSuccess && head_rc == MG_OK && KG) {
      head_rc = mg_batched_propagate(MG_OP_BWD, reinterpret_cast<const mg_batch_mesh*>(base + off_db), (int)KG,
                                     reinterpret_cast<const mg_batch_item*>(base + off_ib), (int)n_ib, head + 1, grid,
                                     smem_bwd, status, st);
      if (head_rc == MG_OK)
        head_rc = mg_batched_reduce(reinterpret_cast<const mg_batch_mesh*>(base + off_db), (int)KG, st);
    }
    if (e == cudaSuccess && head_rc == MG_OK)
      e = cudaMemcpyAsync(h + off_y, base + off_y, out_end - off_y, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && head_rc == MG_OK) e = cudaEventCreateWithFlags(&t.ev, cudaEventDisableTiming);
    if (e == cudaSuccess && head_rc == MG_OK) e = cudaEventRecord(t.ev, st);
    t.dev_off = dev_off;
    t.dev_bytes = total;
    t.reqs = std::move(reqs);
    inflight.push_back(std::move(t));
    ticks += 1;
    if (e != cudaSuccess || head_rc != MG_OK)
      fail_all(e != cudaSuccess ? std::string("tick launch: ") + cudaGetErrorString(e) : std::string("tick launch failed"));
  }

  void loop() {
    cudaSetDevice(device);
    for (;;) {
      bool progressed = retire();
      if (failed) break;
      progressed |= launch_tick();
      if (failed) break;
      {
        std::unique_lock<std::mutex> lk(qmu);
        if (!running && queue.empty() && inflight.empty()) break;
        if (!progressed) qcv.wait_for(lk, std::chrono::microseconds(inflight.empty() ? 2000 : 20));
      }
    }
    // leave nothing on the GPU that refers to the arena
    for (auto& t : inflight)
      if (t.ev) cudaEventSynchronize(t.ev);
    std::lock_guard<std::mutex> lk(dmu);
    dcv.notify_all();
  }
};

extern "C" {

mg_server* mg_server_create(const mg_server_mesh* meshes, int n_meshes, size_t arena_bytes, int n_streams,
                            int max_per_tick, int grid, size_t smem_fwd, size_t smem_bwd, int device) {
  if (!meshes || n_meshes < 1 || arena_bytes < (1u << 20) || n_streams < 1 || max_per_tick < 1 || grid < 1) {
    mg::set_last_error(MG_E_ARG, "mg_server_create: bad arguments");
    return nullptr;
  }
  for (int i = 0; i < n_meshes; ++i) {
    const mg_server_mesh& m = meshes[i];
    if (m.N < 2 || m.L < 0 || m.cap < 1 || m.G < 1 || m.G > 32 || m.cls < MG_BCLS_C8 || m.cls > MG_BCLS_R8 ||
        !m.fwd_tiles || !m.fwd_kinds || !m.bwd_tiles || !m.bwd_kinds) {
      mg::set_last_error(MG_E_ARG, "mg_server_create: bad mesh descriptor %d", i);
      return nullptr;
    }
  }
  auto* s = new mg_server();
  s->meshes.assign(meshes, meshes + n_meshes);
  s->device = device;
  s->grid = grid;
  s->max_per_tick = max_per_tick;
  s->smem_fwd = smem_fwd;
  s->smem_bwd = smem_bwd;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaMalloc(&s->arena_dev, arena_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(s->status, 0, sizeof(int));
  for (int i = 0; e == cudaSuccess && i < n_streams; ++i) {
    cudaStream_t st;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) s->streams.push_back(st);
  }
  if (e != cudaSuccess) {
    mg::set_last_error(MG_E_CUDA, "mg_server_create: %s", cudaGetErrorString(e));
    for (auto st : s->streams) cudaStreamDestroy(st);
    if (s->arena_dev) cudaFree(s->arena_dev);
    if (s->status) cudaFree(s->status);
    delete s;
    return nullptr;
  }
  s->arena.init(arena_bytes);
  s->worker = std::thread([s] { s->loop(); });
  return s;
}

int mg_server_request_bytes(const mg_server* s, int mesh, int b, int grad, size_t* out) {
  if (!s || mesh < 0 || mesh >= (int)s->meshes.size() || b < 1 || !out)
    return mg::set_last_error(MG_E_ARG, "mg_server_request_bytes: bad arguments");
  *out = s->request_bytes(s->meshes[mesh], b, grad != 0);
  return MG_OK;
}

int mg_server_submit(mg_server* s, int mesh, int b, const void* x, const void* gy, void* y, float* dp, void* gx,
                     unsigned long long tag) {
  if (!s) return mg::set_last_error(MG_E_ARG, "mg_server_submit: no server");
  if (mesh < 0 || mesh >= (int)s->meshes.size()) return mg::set_last_error(MG_E_ARG, "no mesh %d", mesh);
  if (b < 1 || !x || !y || (gy && (!dp || !gx))) return mg::set_last_error(MG_E_ARG, "mg_server_submit: bad buffers");
  Req r{tag, mesh, b, x, gy, y, dp, gx, s->request_bytes(s->meshes[mesh], b, gy != nullptr)};
  if (r.bytes + 65536 + 2048 > s->arena.size)
    return mg::set_last_error(MG_E_WORKSPACE, "request needs %zu bytes, above the %zu-byte arena", r.bytes,
                              s->arena.size);
  {
    std::lock_guard<std::mutex> lk(s->qmu);
    if (!s->running) return mg::set_last_error(MG_E_ARG, "server stopped");
    if (s->failed) return mg::set_last_error(MG_E_CUDA, "server failed");
    s->queue.push_back(r);
    s->queued += 1;
  }
  s->qcv.notify_one();
  return MG_OK;
}

int mg_server_wait(mg_server* s, unsigned long long* tags, int max, int timeout_us) {
  if (!s || !tags || max < 1) return mg::set_last_error(MG_E_ARG, "mg_server_wait: bad arguments");
  std::unique_lock<std::mutex> lk(s->dmu);
  if (s->done.empty() && !s->failed && timeout_us > 0)
    s->dcv.wait_for(lk, std::chrono::microseconds(timeout_us), [s] { return !s->done.empty() || s->failed; });
  if (s->done.empty() && s->failed) return mg::set_last_error(MG_E_CUDA, "server failed: %s", s->error.c_str());
  const int n = (int)std::min<size_t>(max, s->done.size());
  std::copy(s->done.begin(), s->done.begin() + n, tags);
  s->done.erase(s->done.begin(), s->done.begin() + n);
  return n;
}

int mg_server_stats(mg_server* s, long long* out) {
  if (!s || !out) return mg::set_last_error(MG_E_ARG, "mg_server_stats: bad arguments");
  out[0] = s->completed;
  out[1] = s->ticks;
  out[2] = s->queued;
  return MG_OK;
}

int mg_server_status(mg_server* s) {
  if (!s) return mg::set_last_error(MG_E_ARG, "mg_server_status: no server");
  int v = 0;
  cudaError_t e = cudaMemcpy(&v, s->status, sizeof(int), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? v : mg::set_last_error(MG_E_CUDA, "mg_server_status: %s", cudaGetErrorString(e));
}

void mg_server_destroy(mg_server* s, int drain) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->qmu);
    s->running = false;
    if (!drain) {
      s->queued -= (long long)s->queue.size();
      s->queue.clear();
    }
  }
  s->qcv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto* p : s->pinned_all) cudaFreeHost(p);
  for (auto st : s->streams) cudaStreamDestroy(st);
  cudaFree(s->arena_dev);
  cudaFree(s->status);
  delete s;
}

}  // extern "C"
