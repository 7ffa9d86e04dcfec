// server.cu — a request server for LBVH build / refit / cast on one GPU.
//
// Clients register meshes (kept in pinned host memory) and submit requests;
// a dispatcher thread admits each request when a slot (a CUDA stream with its
// own preallocated scratch and output buffers) is free and the request's mesh
// is resident in HBM, evicting least-recently-used idle meshes to stay under
// the device-memory budget.  Admitted requests run concurrently, one per
// slot, so requests arriving while others are on the GPU are admitted as
// slots and memory free up and their work overlaps on the device.  Work on
// one mesh is ordered across slots by the mesh's completion event.  A
// completion thread polls the slots' events while requests are in flight
// (and sleeps otherwise), so a finished request is seen within microseconds;
// a host-function callback in the stream would add the driver's callback
// thread to every request's latency.  Latency timestamps are on the steady
// clock.
//
// Results are a pure function of the request, so a request gives the same
// bits alone or in any mix: a mesh's tree topology is always built from its
// rest pose, and the request's `frame` selects the vertex state (frame 0 =
// rest, frame f > 0 = rest + a*sin(phase_v + f + axis) with phase_v a hash of
// (mesh seed, v)), reached by a refit of the resident tree when it differs
// from the mesh's current state.
//
//   DM_REQ_BUILD_CAST   full LBVH build from the rest pose, state -> frame, pixel cast
//   DM_REQ_REFIT_CAST   state -> frame on the resident tree (refit), pixel cast
//   DM_REQ_CAST_RAYS    state -> frame if needed, cast of explicit rays
//
// dm_plain_run_trace runs the same requests the straightforward way for
// comparison: one at a time, each uploading its mesh, building, refitting,
// casting, downloading and synchronizing, with nothing kept resident.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/delmsh_gb300.h"
#include "dm_device.cuh"
#include "dm_internal.h"

struct dm_server;

namespace dm {
namespace {

uint64_t now_ns() {
  return static_cast<uint64_t>(
      std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
          .count());
}

inline size_t a256(size_t x) { return (x + 255) / 256 * 256; }

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// v = rest + amp * sin(phase_v + frame + axis)
__global__ void k_deform(uint32_t num_vtx, const float* __restrict__ rest, float* __restrict__ out, uint32_t seed,
                         uint32_t frame, float amp) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_vtx) return;
  const float phase = static_cast<float>(hash32(seed ^ (i * 0x9E3779B9u))) * (6.2831853f / 4294967296.0f);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float s = sinf(__fadd_rn(phase, static_cast<float>(frame + d)));
    out[3ull * i + d] = __fadd_rn(rest[3ull * i + d], __fmul_rn(amp, s));
  }
}

struct HostMesh {
  uint32_t T = 0, V = 0, seed = 0;
  uint32_t* tri = nullptr;  // pinned copies
  float* vtx = nullptr;
};

// Device arrays of one mesh, carved from one stream-ordered allocation.
struct DevMesh {
  void* block = nullptr;
  size_t bytes = 0;
  uint32_t* tri = nullptr;
  float* rest = nullptr;
  float* vtx = nullptr;
  uint32_t* bvh = nullptr;
  float* aabb = nullptr;
  uint32_t* other = nullptr;
  uint32_t* flags = nullptr;
  bool uploaded = false, built = false;
  int64_t frame = -1;  // vertex state currently in vtx (with amp)
  float amp = 0.0f;
  int inflight = 0;
  uint64_t last_use = 0;
  cudaEvent_t last = nullptr;  // completion of the latest work on this mesh
  bool has_last = false;
};

size_t mesh_bytes(uint32_t T, uint32_t V) {
  return a256(12ull * T) + 2 * a256(12ull * V) + a256(12ull * (2 * T - 1)) + a256(24ull * (2 * T - 1)) +
         a256(4ull * T) + a256(4 * refit_flags_words(T));
}

void carve(DevMesh& m, uint32_t T, uint32_t V) {
  char* p = static_cast<char*>(m.block);
  m.tri = reinterpret_cast<uint32_t*>(p);
  p += a256(12ull * T);
  m.rest = reinterpret_cast<float*>(p);
  p += a256(12ull * V);
  m.vtx = reinterpret_cast<float*>(p);
  p += a256(12ull * V);
  m.bvh = reinterpret_cast<uint32_t*>(p);
  p += a256(12ull * (2 * T - 1));
  m.aabb = reinterpret_cast<float*>(p);
  p += a256(24ull * (2 * T - 1));
  m.other = reinterpret_cast<uint32_t*>(p);
  p += a256(4ull * T);
  m.flags = reinterpret_cast<uint32_t*>(p);
}

struct Slot {
  cudaStream_t stream = nullptr;
  void* build_scratch = nullptr;
  size_t build_bytes = 0;
  void* cast_scratch = nullptr;
  size_t cast_bytes = 0;
  float* d_transform = nullptr;
  float* d_rays = nullptr;  // max_out origins then max_out directions
  uint32_t* d_hit = nullptr;
  float* d_t = nullptr;
  cudaEvent_t done = nullptr;  // recorded after the slot's current request
  bool busy = false;
};

struct Job {
  uint64_t ticket = 0;
  dm_request req{};
  dm_result res{};
  int slot = -1;
  bool done = false;
  dm_server* srv = nullptr;
};

}  // namespace
}  // namespace dm

struct dm_server {
  int device = 0;
  // resident meshes' blocks come from this pool, which keeps freed memory
  // (release threshold: never) so that admitting a mesh after an eviction, or
  // for the first time after a synchronisation, maps no memory; nullptr: the
  // device's default pool
  cudaMemPool_t pool = nullptr;
  size_t budget = 0, used = 0, slot_bytes = 0;
  uint32_t max_tri = 0, max_out = 0;
  std::vector<dm::Slot> slots;
  std::unordered_map<uint32_t, dm::HostMesh> host;
  std::unordered_map<uint32_t, dm::DevMesh> dev;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<dm::Job*> queue;
  std::unordered_map<uint64_t, dm::Job*> jobs;
  uint64_t next_ticket = 1, use_clock = 0;
  std::thread dispatcher;
  std::thread completer;
  std::vector<dm::Job*> inflight;  // admitted requests whose work is on the GPU
  bool stop = false;
  bool stop_completer = false;  // set once the dispatcher has exited
  dm_server_stats stats{};  // guarded by mu, except the two counters below
  std::atomic<uint64_t> builds{0}, refits{0};
};

namespace dm {
namespace {

int fill_error(dm_result* r, int code) {
  r->status = code;
  return code;
}

// Enqueues the state change (build / deform / refit) that brings mesh m to
// `frame` on stream st.  Caller owns m (dispatcher thread or plain runner).
int prepare_mesh(cudaStream_t st, const HostMesh& hm, DevMesh& m, uint32_t kind, uint32_t frame, float amp,
                 const Slot& sl, dm_server* counters) {
  cudaError_t e = cudaSuccess;
  if (!m.uploaded) {
    if ((e = cudaMemcpyAsync(m.tri, hm.tri, 12ull * hm.T, cudaMemcpyHostToDevice, st)) != cudaSuccess) return DM_ERR_CUDA;
    if ((e = cudaMemcpyAsync(m.rest, hm.vtx, 12ull * hm.V, cudaMemcpyHostToDevice, st)) != cudaSuccess) return DM_ERR_CUDA;
    if ((e = cudaMemsetAsync(m.flags, 0, 4ull * hm.T, st)) != cudaSuccess) return DM_ERR_CUDA;
    m.uploaded = true;
  }
  if (kind == DM_REQ_BUILD_CAST || !m.built) {
    if (cudaMemcpyAsync(m.vtx, m.rest, 12ull * hm.V, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return DM_ERR_CUDA;
    const int rc = build_keep_ranges(st, hm.T, m.tri, hm.V, m.vtx, m.bvh, m.aabb, m.other, sl.build_scratch,
                                     sl.build_bytes);
    if (rc != DM_OK) return rc;
    m.built = true;
    m.frame = 0;
    m.amp = 0.0f;
    if (counters) counters->builds++;
  }
  if (m.frame != static_cast<int64_t>(frame) || (frame != 0 && m.amp != amp)) {
    if (frame == 0) {
      if (cudaMemcpyAsync(m.vtx, m.rest, 12ull * hm.V, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return DM_ERR_CUDA;
    } else {
      k_deform<<<(hm.V + 255) / 256, 256, 0, st>>>(hm.V, m.rest, m.vtx, hm.seed, frame, amp);
    }
    launch_refit_windowed(st, hm.T, Segments{1, nullptr, nullptr}, hm.V, m.bvh, m.other, m.tri, m.vtx, nullptr,
                          m.aabb, m.flags, nullptr, device_status_word());
    m.frame = frame;
    m.amp = amp;
    if (counters) counters->refits++;
  }
  return cudaGetLastError() == cudaSuccess ? DM_OK : DM_ERR_CUDA;
}

// Enqueues the cast of a request and the download of its results.
int cast_request(cudaStream_t st, const HostMesh& hm, const DevMesh& m, const dm_request& r, const Slot& sl) {
  MeshView mv{hm.T, hm.V, m.tri, m.vtx, m.bvh, m.aabb};
  CastScratch cs;
  const uint32_t n = (r.kind == DM_REQ_CAST_RAYS) ? r.num_ray : r.img_w * r.img_h;
  cast_scratch_carve(sl.cast_scratch, n, hm.T, &cs);
  if (cudaMemsetAsync(cs.counters, 0, 16, st) != cudaSuccess) return DM_ERR_CUDA;
  CastOut o{sl.d_hit, sl.d_t, nullptr};
  if (r.kind == DM_REQ_CAST_RAYS) {
    float* org = sl.d_rays;
    float* dir = sl.d_rays + 3ull * n;
    if (cudaMemcpyAsync(org, r.ray_org, 12ull * n, cudaMemcpyHostToDevice, st) != cudaSuccess) return DM_ERR_CUDA;
    if (cudaMemcpyAsync(dir, r.ray_dir, 12ull * n, cudaMemcpyHostToDevice, st) != cudaSuccess) return DM_ERR_CUDA;
    launch_cast_rays(st, n, org, dir, mv, o, cs, device_status_word());
  } else {
    if (cudaMemcpyAsync(sl.d_transform, r.transform_ndc2world, 64, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return DM_ERR_CUDA;
    launch_cast_pixels(st, r.img_w, r.img_h, sl.d_transform, mv, o, cs, device_status_word());
  }
  if (r.out_tri && cudaMemcpyAsync(r.out_tri, sl.d_hit, 4ull * n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return DM_ERR_CUDA;
  if (r.out_t && cudaMemcpyAsync(r.out_t, sl.d_t, 4ull * n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return DM_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? DM_OK : DM_ERR_CUDA;
}

// Marks job j finished (status e) at time t; called with the lock held.
void finish(dm_server* S, Job* j, int e, uint64_t t) {
  if (e != DM_OK) j->res.status = e;
  j->res.t_done_ns = t;
  j->done = true;
  S->slots[j->slot].busy = false;
  auto it = S->dev.find(j->req.mesh_id);
  if (it != S->dev.end()) it->second.inflight--;
  S->stats.completed++;
}

// Polls the completion events of the requests in flight.
void complete_loop(dm_server* S) {
  cudaSetDevice(S->device);
  std::vector<Job*> pending;
  std::vector<std::pair<Job*, int>> finished;
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv.wait(lk, [&] { return S->stop_completer || !S->inflight.empty(); });
    if (S->inflight.empty()) break;  // stopping, and nothing left in flight
    pending = S->inflight;
    lk.unlock();
    finished.clear();
    for (Job* j : pending) {
      const cudaError_t e = cudaEventQuery(S->slots[j->slot].done);
      if (e != cudaErrorNotReady) finished.emplace_back(j, e == cudaSuccess ? DM_OK : DM_ERR_CUDA);
    }
    const uint64_t t = now_ns();
    if (finished.empty()) std::this_thread::yield();
    lk.lock();
    if (finished.empty()) continue;
    for (auto& f : finished) {
      S->inflight.erase(std::find(S->inflight.begin(), S->inflight.end(), f.first));
      finish(S, f.first, f.second, t);
    }
    S->cv.notify_all();
  }
}

int free_slot(dm_server* S) {
  for (size_t i = 0; i < S->slots.size(); ++i)
    if (!S->slots[i].busy) return static_cast<int>(i);
  return -1;
}

bool all_idle(dm_server* S) {
  for (const auto& sl : S->slots)
    if (sl.busy) return false;
  return S->queue.empty();
}

// Makes mesh `id` resident (allocating and evicting under the budget).
// Called with the lock held; may wait on the condition variable.  Returns
// nullptr with *err set when the mesh can never fit.
DevMesh* ensure_resident(dm_server* S, uint32_t id, int slot, std::unique_lock<std::mutex>& lk, int* err) {
  auto hit = S->dev.find(id);
  if (hit != S->dev.end() && hit->second.block) {
    S->stats.resident_hits++;
    return &hit->second;
  }
  const HostMesh& hm = S->host.at(id);
  const size_t bytes = mesh_bytes(hm.T, hm.V);
  if (bytes + S->slot_bytes > S->budget) {
    *err = DM_ERR_INVALID_ARGUMENT;
    return nullptr;
  }
  cudaStream_t st = S->slots[slot].stream;
  while (S->used + bytes > S->budget) {
    DevMesh* victim = nullptr;
    uint32_t victim_id = 0;
    for (auto& kv : S->dev)
      if (kv.first != id && kv.second.block && kv.second.inflight == 0 &&
          (!victim || kv.second.last_use < victim->last_use)) {
        victim = &kv.second;
        victim_id = kv.first;
      }
    if (!victim) {  // everything resident is in use: wait for completions
      S->cv.wait(lk);
      continue;
    }
    if (victim->has_last) cudaStreamWaitEvent(st, victim->last, 0);
    cudaFreeAsync(victim->block, st);
    S->used -= victim->bytes;
    victim->block = nullptr;
    victim->uploaded = victim->built = false;
    victim->frame = -1;
    S->stats.evictions++;
    (void)victim_id;
  }
  DevMesh& m = S->dev[id];
  if (!m.last) cudaEventCreateWithFlags(&m.last, cudaEventDisableTiming);
  const cudaError_t ae = S->pool ? cudaMallocFromPoolAsync(&m.block, bytes, S->pool, st)
                                 : cudaMallocAsync(&m.block, bytes, st);
  if (ae != cudaSuccess) {
    m.block = nullptr;
    *err = DM_ERR_CUDA;
    return nullptr;
  }
  m.bytes = bytes;
  carve(m, hm.T, hm.V);
  m.uploaded = m.built = false;
  m.frame = -1;
  S->used += bytes;
  return &m;
}

void dispatch_loop(dm_server* S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv.wait(lk, [&] { return S->stop || !S->queue.empty(); });
    if (S->queue.empty()) break;  // stop requested and nothing left
    const int s = free_slot(S);
    if (s < 0) {
      S->cv.wait(lk);
      continue;
    }
    Job* j = S->queue.front();
    int err = DM_OK;
    DevMesh* m = ensure_resident(S, j->req.mesh_id, s, lk, &err);
    S->queue.pop_front();
    if (!m) {
      fill_error(&j->res, err);
      j->res.t_admit_ns = j->res.t_done_ns = now_ns();
      j->done = true;
      S->stats.completed++;
      S->cv.notify_all();
      continue;
    }
    j->res.resident_hit = m->built ? 1u : 0u;
    j->res.t_admit_ns = now_ns();
    j->slot = s;
    Slot& sl = S->slots[s];
    sl.busy = true;
    m->inflight++;
    m->last_use = ++S->use_clock;
    const HostMesh& hm = S->host.at(j->req.mesh_id);
    lk.unlock();
    // Only this thread changes mesh state and enqueues work, so the mesh
    // fields below are safe without the lock (the completion thread only touches inflight).
    const cudaStream_t st = sl.stream;
    int rc = DM_OK;
    if (m->has_last && cudaStreamWaitEvent(st, m->last, 0) != cudaSuccess) rc = DM_ERR_CUDA;
    if (rc == DM_OK) rc = prepare_mesh(st, hm, *m, j->req.kind, j->req.frame, j->req.deform_amplitude, sl, S);
    if (rc == DM_OK) rc = cast_request(st, hm, *m, j->req, sl);
    if (rc == DM_OK && cudaEventRecord(m->last, st) != cudaSuccess) rc = DM_ERR_CUDA;
    if (rc == DM_OK && cudaEventRecord(sl.done, st) != cudaSuccess) rc = DM_ERR_CUDA;
    if (rc == DM_OK) {
      m->has_last = true;
      j->res.status = DM_OK;
    } else {
      cudaStreamSynchronize(st);
    }
    lk.lock();
    if (rc == DM_OK) {
      S->inflight.push_back(j);
    } else {
      fill_error(&j->res, rc);
      finish(S, j, rc, now_ns());
    }
    S->cv.notify_all();
  }
}

int check_request(const dm_server* S, const dm_request* r) {
  if (!r) return set_error(DM_ERR_INVALID_ARGUMENT, "NULL request");
  if (S->host.find(r->mesh_id) == S->host.end())
    return set_error(DM_ERR_INVALID_ARGUMENT, "mesh %u is not registered", r->mesh_id);
  if (r->kind > DM_REQ_CAST_RAYS) return set_error(DM_ERR_INVALID_ARGUMENT, "unknown request kind %u", r->kind);
  const uint64_t n = r->kind == DM_REQ_CAST_RAYS ? r->num_ray : static_cast<uint64_t>(r->img_w) * r->img_h;
  if (n == 0 || n > S->max_out)
    return set_error(DM_ERR_INVALID_ARGUMENT, "request of %llu rays outside 1..%u", (unsigned long long)n, S->max_out);
  // a pixel cast pads its image to whole warp tiles, counted in 32 bits
  if (r->kind != DM_REQ_CAST_RAYS && (uint64_t{r->img_w} + 31) * (uint64_t{r->img_h} + 31) > 0xFFFFFFFFull)
    return set_error(DM_ERR_INVALID_ARGUMENT, "image of %u x %u pixels pads to too many tile slots", r->img_w,
                     r->img_h);
  if (r->kind == DM_REQ_CAST_RAYS && (!r->ray_org || !r->ray_dir))
    return set_error(DM_ERR_INVALID_ARGUMENT, "ray arrays must not be NULL");
  if (r->kind != DM_REQ_CAST_RAYS && !r->transform_ndc2world)
    return set_error(DM_ERR_INVALID_ARGUMENT, "transform_ndc2world must not be NULL");
  return DM_OK;
}

void sleep_until_ns(uint64_t t) {
  for (;;) {
    const uint64_t n = now_ns();
    if (n >= t) return;
    if (t - n > 200000) std::this_thread::sleep_for(std::chrono::nanoseconds(t - n - 100000));
    else std::this_thread::yield();
  }
}

}  // namespace
}  // namespace dm

extern "C" {

int dm_server_create(int device, size_t budget_bytes, int num_slots, uint32_t max_tri, uint32_t max_out,
                     dm_server** out) {
  using namespace dm;
  if (!out || num_slots < 1 || num_slots > 64 || max_tri < 1 || max_out < 1)
    return set_error(DM_ERR_INVALID_ARGUMENT, "invalid server parameters");
  if (cudaSetDevice(device) != cudaSuccess) return set_error(DM_ERR_CUDA, "cudaSetDevice(%d) failed", device);
  dm_server* S = new dm_server();
  S->device = device;
  S->budget = budget_bytes;
  S->max_tri = max_tri;
  S->max_out = max_out;
  S->slots.resize(num_slots);
  for (auto& sl : S->slots) {
    sl.build_bytes = build_scratch_bytes(max_tri);
    sl.cast_bytes = cast_scratch_bytes(max_out, max_tri);
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&sl.build_scratch, sl.build_bytes) != cudaSuccess ||
        cudaMalloc(&sl.cast_scratch, sl.cast_bytes) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void**>(&sl.d_transform), 64) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void**>(&sl.d_rays), 24ull * max_out) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void**>(&sl.d_hit), 4ull * max_out) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void**>(&sl.d_t), 4ull * max_out) != cudaSuccess) {
      dm_server_destroy(S);
      return set_error(DM_ERR_CUDA, "allocating server slots failed");
    }
    S->slot_bytes += sl.build_bytes + sl.cast_bytes + 64 + 32ull * max_out;
  }
  S->used = S->slot_bytes;
  S->stats.bytes_budget = budget_bytes;
  {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&S->pool, &props) == cudaSuccess) {
      uint64_t keep = ~uint64_t{0};
      cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    } else {
      cudaGetLastError();  // pools unsupported: the default pool
      S->pool = nullptr;
    }
  }
  if (S->slot_bytes > budget_bytes) {
    dm_server_destroy(S);
    return set_error(DM_ERR_INVALID_ARGUMENT, "budget smaller than the slots' own memory");
  }
  S->dispatcher = std::thread(dispatch_loop, S);
  S->completer = std::thread(complete_loop, S);
  *out = S;
  return DM_OK;
}

int dm_server_register_mesh(dm_server* S, uint32_t mesh_id, const uint32_t* tri2vtx, uint32_t num_tri,
                            const float* vtx2xyz, uint32_t num_vtx, uint32_t deform_seed) {
  using namespace dm;
  if (!S || !tri2vtx || !vtx2xyz || num_tri < 1 || num_vtx < 1 || num_tri > S->max_tri)
    return set_error(DM_ERR_INVALID_ARGUMENT, "invalid mesh (triangles must be in 1..max_tri)");
  for (uint64_t i = 0; i < 3ull * num_tri; ++i)
    if (tri2vtx[i] >= num_vtx) return set_error(DM_ERR_INVALID_ARGUMENT, "vertex index out of range in mesh %u", mesh_id);
  HostMesh hm;
  hm.T = num_tri;
  hm.V = num_vtx;
  hm.seed = deform_seed;
  if (cudaMallocHost(reinterpret_cast<void**>(&hm.tri), 12ull * num_tri) != cudaSuccess ||
      cudaMallocHost(reinterpret_cast<void**>(&hm.vtx), 12ull * num_vtx) != cudaSuccess)
    return set_error(DM_ERR_CUDA, "pinned host allocation failed");
  std::memcpy(hm.tri, tri2vtx, 12ull * num_tri);
  std::memcpy(hm.vtx, vtx2xyz, 12ull * num_vtx);
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->host.find(mesh_id);
  if (it != S->host.end()) {
    auto d = S->dev.find(mesh_id);
    if (d != S->dev.end() && (d->second.block || d->second.inflight)) {
      cudaFreeHost(hm.tri);
      cudaFreeHost(hm.vtx);
      return set_error(DM_ERR_INVALID_ARGUMENT, "mesh %u is resident; it cannot be replaced", mesh_id);
    }
    cudaFreeHost(it->second.tri);
    cudaFreeHost(it->second.vtx);
  }
  S->host[mesh_id] = hm;
  return DM_OK;
}

int dm_server_submit(dm_server* S, const dm_request* req, uint64_t* ticket) {
  using namespace dm;
  if (!S || !ticket) return set_error(DM_ERR_INVALID_ARGUMENT, "NULL argument");
  Job* j = new Job();
  j->res.t_submit_ns = now_ns();
  std::lock_guard<std::mutex> lk(S->mu);
  if (int e = check_request(S, req)) {
    delete j;
    return e;
  }
  j->req = *req;
  j->srv = S;
  j->ticket = S->next_ticket++;
  S->jobs[j->ticket] = j;
  S->queue.push_back(j);
  S->stats.submitted++;
  *ticket = j->ticket;
  S->cv.notify_all();
  return DM_OK;
}

int dm_server_wait(dm_server* S, uint64_t ticket, dm_result* out) {
  using namespace dm;
  if (!S || !out) return set_error(DM_ERR_INVALID_ARGUMENT, "NULL argument");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(ticket);
  if (it == S->jobs.end()) return set_error(DM_ERR_INVALID_ARGUMENT, "unknown ticket %llu", (unsigned long long)ticket);
  Job* j = it->second;
  S->cv.wait(lk, [&] { return j->done; });
  *out = j->res;
  S->jobs.erase(it);
  delete j;
  return out->status;
}

int dm_server_run_trace(dm_server* S, uint32_t n, const dm_request* reqs, const double* arrival_s,
                        dm_result* results) {
  using namespace dm;
  if (!S || (n && (!reqs || !arrival_s || !results))) return set_error(DM_ERR_INVALID_ARGUMENT, "NULL argument");
  std::vector<uint64_t> tickets(n, 0);
  std::vector<uint64_t> sched(n, 0);
  const uint64_t t0 = now_ns() + 1000000;
  int rc = DM_OK;
  for (uint32_t i = 0; i < n; ++i) {
    sched[i] = t0 + static_cast<uint64_t>(arrival_s[i] * 1e9);
    sleep_until_ns(sched[i]);
    if (int e = dm_server_submit(S, reqs + i, &tickets[i])) {
      results[i] = dm_result{};
      results[i].status = e;
      rc = e;
    }
  }
  for (uint32_t i = 0; i < n; ++i) {
    if (!tickets[i]) continue;
    dm_server_wait(S, tickets[i], results + i);
    results[i].t_submit_ns = sched[i];  // latency counts from the scheduled arrival
  }
  return rc;
}

int dm_server_stats_get(dm_server* S, dm_server_stats* out) {
  using namespace dm;
  if (!S || !out) return set_error(DM_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->stats;
  out->builds = S->builds.load();
  out->refits = S->refits.load();
  out->bytes_resident = S->used - S->slot_bytes;
  out->bytes_slots = S->slot_bytes;
  uint32_t n = 0;
  for (auto& kv : S->dev)
    if (kv.second.block) ++n;
  out->meshes_resident = n;
  return DM_OK;
}

int dm_server_destroy(dm_server* S) {
  using namespace dm;
  if (!S) return DM_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  if (S->dispatcher.joinable()) S->dispatcher.join();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop_completer = true;
    S->cv.notify_all();
  }
  if (S->completer.joinable()) S->completer.join();
  cudaSetDevice(S->device);
  for (auto& sl : S->slots)
    if (sl.stream) cudaStreamSynchronize(sl.stream);
  for (auto& kv : S->dev) {
    if (kv.second.block) cudaFree(kv.second.block);
    if (kv.second.last) cudaEventDestroy(kv.second.last);
  }
  if (S->pool) cudaMemPoolDestroy(S->pool);
  for (auto& sl : S->slots) {
    cudaFree(sl.build_scratch);
    cudaFree(sl.cast_scratch);
    cudaFree(sl.d_transform);
    cudaFree(sl.d_rays);
    cudaFree(sl.d_hit);
    cudaFree(sl.d_t);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  for (auto& kv : S->host) {
    cudaFreeHost(kv.second.tri);
    cudaFreeHost(kv.second.vtx);
  }
  for (auto& kv : S->jobs) delete kv.second;
  delete S;
  return DM_OK;
}

int dm_plain_run_trace(dm_server* S, uint32_t n, const dm_request* reqs, const double* arrival_s,
                       dm_result* results) {
  using namespace dm;
  if (!S || (n && (!reqs || !arrival_s || !results))) return set_error(DM_ERR_INVALID_ARGUMENT, "NULL argument");
  cudaSetDevice(S->device);
  Slot& sl = S->slots[0];
  {
    // the plain path runs alone: wait until the server is idle
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv.wait(lk, [&] { return all_idle(S); });
    sl.busy = true;
  }
  const uint64_t t0 = now_ns() + 1000000;
  int rc = DM_OK;
  for (uint32_t i = 0; i < n; ++i) {
    dm_result& res = results[i];
    res = dm_result{};
    res.t_submit_ns = t0 + static_cast<uint64_t>(arrival_s[i] * 1e9);
    sleep_until_ns(res.t_submit_ns);
    res.t_admit_ns = now_ns();
    const dm_request& r = reqs[i];
    int e = check_request(S, &r);
    if (e == DM_OK) {
      const HostMesh& hm = S->host.at(r.mesh_id);
      DevMesh m;
      const size_t bytes = mesh_bytes(hm.T, hm.V);
      if (cudaMallocAsync(&m.block, bytes, sl.stream) != cudaSuccess) {
        e = DM_ERR_CUDA;
      } else {
        carve(m, hm.T, hm.V);
        e = prepare_mesh(sl.stream, hm, m, DM_REQ_BUILD_CAST, r.frame, r.deform_amplitude, sl, nullptr);
        if (e == DM_OK) e = cast_request(sl.stream, hm, m, r, sl);
        cudaFreeAsync(m.block, sl.stream);
      }
      if (cudaStreamSynchronize(sl.stream) != cudaSuccess && e == DM_OK) e = DM_ERR_CUDA;
    }
    res.status = e;
    res.t_done_ns = now_ns();
    if (e != DM_OK) rc = e;
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    sl.busy = false;
    S->cv.notify_all();
  }
  return rc;
}

}  // extern "C"
