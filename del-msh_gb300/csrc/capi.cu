// capi.cu — the library's C ABI (include/delmsh_gb300.h): argument checks,
// scratch layout, and the launch sequences of the LBVH build and ray cast.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <utility>

#include "../../include/delmsh_gb300.h"
#include "dm_device.cuh"
#include "dm_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(DM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define DM_CUDA(call)                                       \
  do {                                                      \
    const cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);     \
  } while (0)

#define DM_REQUIRE(cond, ...) \
  do {                        \
    if (!(cond)) return fail(DM_ERR_INVALID_ARGUMENT, __VA_ARGS__); \
  } while (0)

constexpr uint32_t kMaxElems = (1u << 30) - 1;  // sort look-back packs counts in 30 bits

// Device status word: kernels OR error bits into it (see dm::DeviceStatusBits).
// Its address is looked up once per device and kept for the life of the
// process, so the library must not be used across a cudaDeviceReset.
__device__ uint32_t g_status_word;

uint32_t* status_ptr() {
  static std::mutex mu;
  static uint32_t* cache[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!cache[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_status_word) != cudaSuccess) return nullptr;
    cache[dev] = static_cast<uint32_t*>(p);
  }
  return cache[dev];
}

inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Work items of a pixel cast: every image is padded to whole warp tiles of
// tile_w x (32 / tile_w) pixels, at most (w + 31) x (h + 31) slots whatever
// the tile shape; the kernels count them in 32 bits.
inline uint64_t padded_pixel_work(uint32_t img_w, uint32_t img_h, uint32_t num_image) {
  return (static_cast<uint64_t>(img_w) + 31) * (static_cast<uint64_t>(img_h) + 31) * num_image;
}

// Temporary device memory: the caller's, or stream-ordered allocation.
struct Scratch {
  void* ptr = nullptr;
  cudaStream_t stream = nullptr;
  bool owned = false;
  ~Scratch() {
    if (owned && ptr) cudaFreeAsync(ptr, stream);
  }
  int acquire(void* user, size_t user_bytes, size_t need, cudaStream_t s, bool* fresh) {
    stream = s;
    if (user) {
      if (user_bytes < need)
        return fail(DM_ERR_SCRATCH_TOO_SMALL, "scratch of %zu bytes is smaller than the %zu bytes needed", user_bytes,
                    need);
      if (reinterpret_cast<uintptr_t>(user) % 256 != 0) return fail(DM_ERR_INVALID_ARGUMENT, "scratch must be 256-byte aligned");
      ptr = user;
      if (fresh) *fresh = false;
      return DM_OK;
    }
    const cudaError_t e = cudaMallocAsync(&ptr, need, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(scratch)");
    owned = true;
    if (fresh) *fresh = true;
    return DM_OK;
  }
};

inline cudaStream_t as_stream(uint64_t p) { return reinterpret_cast<cudaStream_t>(static_cast<uintptr_t>(p)); }

// ------------------------------------------------------------ sort layout
// [header: hist 8*256 u32 | tile counters 16 u32][lookback][keys tmp][vals tmp]
struct SortLayout {
  size_t hist = 0, counters = 0, lookback = 0, keys = 0, vals = 0, zero_bytes = 0, total = 0;
};

SortLayout sort_layout(uint32_t n, int num_pass, size_t key_bytes, int radix = dm::kRadix) {
  SortLayout L;
  L.hist = 0;
  L.counters = std::max<size_t>(8 * 256, static_cast<size_t>(num_pass) * radix) * 4;
  L.lookback = align256(L.counters + 16 * 4);
  L.zero_bytes = L.lookback + align256(dm::sort_lookback_words(n, num_pass, radix) * 4);
  L.keys = L.zero_bytes;
  L.vals = L.keys + align256(static_cast<size_t>(n) * key_bytes);
  L.total = L.vals + align256(static_cast<size_t>(n) * 4);
  return L;
}

// -------------------------------------------------------- build layout
struct BuildLayout {
  size_t transform, aabb, ticket, height, front_bar, sort_hdr, partials, codes, akeys, avals, bvals, flags, tribox,
      front_counts, front_totals, total, zero_bytes, sort_bytes;
  SortLayout sort8, sort10;  // four 8-bit passes / three 10-bit passes
};

BuildLayout build_layout(uint32_t T) {
  BuildLayout L{};
  L.transform = 0;
  L.aabb = 64;
  L.ticket = 96;
  L.height = 100;
  L.front_bar = 104;
  L.sort_hdr = 256;
  L.sort8 = sort_layout(T, 4, 4);
  L.sort10 = sort_layout(T, 3, 4, dm::kRadix10);
  // header + lookback of either width (the tmp arrays are carved separately)
  L.sort_bytes = std::max(L.sort8.zero_bytes, L.sort10.zero_bytes);
  L.zero_bytes = L.sort_hdr + L.sort_bytes;
  L.partials = align256(L.zero_bytes);
  L.codes = L.partials + align256(dm::kAabbBlocks * 6 * 4);
  L.akeys = L.codes + align256(static_cast<size_t>(T) * 4);
  L.avals = L.akeys + align256(static_cast<size_t>(T) * 4);
  L.bvals = L.avals + align256(static_cast<size_t>(T) * 4);
  L.flags = L.bvals + align256(static_cast<size_t>(T) * 4);
  L.tribox = L.flags + align256(dm::refit_flags_words(T) * 4);
  L.front_counts = L.tribox + align256(static_cast<size_t>(T) * 24);
  L.front_totals = L.front_counts + align256(size_t{4} * dm::kRadix * dm::kAabbBlocks);
  L.total = L.front_totals + align256(size_t{4} * dm::kRadix);
  return L;
}

template <typename T>
T* at(void* base, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

int check_mesh(uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz) {
  DM_REQUIRE(num_tri >= 1, "num_tri must be >= 1 (got %u)", num_tri);
  DM_REQUIRE(num_tri <= kMaxElems, "num_tri %u exceeds the supported maximum %u", num_tri, kMaxElems);
  DM_REQUIRE(num_vtx >= 1, "num_vtx must be >= 1");
  DM_REQUIRE(tri2vtx && vtx2xyz, "tri2vtx / vtx2xyz must not be NULL");
  return DM_OK;
}

// Three 10-bit onesweep passes over 30-bit keys: (k0, iota) -> A -> B -> out.
void sort3(cudaStream_t s, uint32_t n, const uint32_t* k0, uint32_t* ak, uint32_t* av, uint32_t* bk, uint32_t* bv,
           uint32_t* ok, uint32_t* ov, uint32_t* hist, uint32_t* counters, uint32_t* lookback, uint32_t* status) {
  const size_t lbw = dm::sort_lookback_words(n, 1, dm::kRadix10);
  dm::launch_onesweep10_u32(s, n, 0, k0, nullptr, ak, av, hist, lookback, counters, status);
  dm::launch_onesweep10_u32(s, n, 10, ak, av, bk, bv, hist + dm::kRadix10, lookback + lbw, counters + 1, status);
  dm::launch_onesweep10_u32(s, n, 20, bk, bv, ok, ov, hist + 2 * dm::kRadix10, lookback + 2 * lbw, counters + 2,
                            status);
}

// The four onesweep passes over 30- or 32-bit keys: (k0, iota) -> A -> B -> A -> out.
void sort4(cudaStream_t s, uint32_t n, const uint32_t* k0, uint32_t* ak, uint32_t* av, uint32_t* bk, uint32_t* bv,
           uint32_t* ok, uint32_t* ov, uint32_t* hist, uint32_t* counters, uint32_t* lookback, uint32_t* status) {
  const size_t lbw = dm::sort_lookback_words(n, 1);
  dm::launch_onesweep_u32(s, n, 0, k0, nullptr, ak, av, hist, lookback, counters, status, true);
  dm::launch_onesweep_u32(s, n, 8, ak, av, bk, bv, hist + 256, lookback + lbw, counters + 1, status, true);
  dm::launch_onesweep_u32(s, n, 16, bk, bv, ak, av, hist + 512, lookback + 2 * lbw, counters + 2, status, true);
  dm::launch_onesweep_u32(s, n, 24, ak, av, ok, ov, hist + 768, lookback + 3 * lbw, counters + 3, status, true);
}

// ev (optional, 5 events): recorded before the first stage and after each of
// Morton, sort, topology and refit.
int build_impl(uint64_t stream_ptr, uint32_t T, const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz,
               uint32_t* bvhnodes, float* aabb, float* transform_out, uint32_t* tri2morton_out, uint32_t* idx2tri_out,
               uint32_t* idx2morton_out, uint32_t* height_out, void* scratch, size_t scratch_bytes,
               cudaEvent_t* ev = nullptr, uint32_t* other_end_out = nullptr) {
  if (int e = check_mesh(T, tri2vtx, num_vtx, vtx2xyz)) return e;
  DM_REQUIRE(bvhnodes && aabb, "bvhnodes / bvhnode2aabb must not be NULL");
  cudaStream_t s = as_stream(stream_ptr);
  const BuildLayout L = build_layout(T);
  Scratch sc;
  if (int e = sc.acquire(scratch, scratch_bytes, L.total, s, nullptr)) return e;
  void* base = sc.ptr;
  uint32_t* status = status_ptr();
  // the size class's choices (autotuned; every choice builds the same tree)
  const dm::BuildTuning bt = dm::build_tuning_for(T);
  const bool try_front = bt.build_path == 0 && T >= 2 && T <= dm::front_max_tri();
  const bool radix10 = bt.sort_radix == 10 || (bt.sort_radix == 0 && T <= dm::kRadix10MaxKeys);
  const SortLayout& SL = radix10 ? L.sort10 : L.sort8;
  // the front needs only the header zeroed; the separate kernels also their
  // histograms, tile counters and look-back words
  DM_CUDA(cudaMemsetAsync(base, 0, try_front ? L.sort_hdr : L.sort_hdr + SL.zero_bytes, s));
  DM_CUDA(cudaMemsetAsync(at<char>(base, L.flags), 0, static_cast<size_t>(T) * 4, s));
  float* transform = at<float>(base, L.transform);
  uint32_t* hist = at<uint32_t>(base, L.sort_hdr + SL.hist);
  uint32_t* counters = at<uint32_t>(base, L.sort_hdr + SL.counters);
  uint32_t* lookback = at<uint32_t>(base, L.sort_hdr + SL.lookback);
  uint32_t* codes = at<uint32_t>(base, L.codes);
  uint32_t* ak = at<uint32_t>(base, L.akeys);
  uint32_t* av = at<uint32_t>(base, L.avals);
  uint32_t* bv = at<uint32_t>(base, L.bvals);
  uint32_t* flags = at<uint32_t>(base, L.flags);
  uint32_t* height = at<uint32_t>(base, L.height);

  if (ev) DM_CUDA(cudaEventRecord(ev[0], s));
  // the centroids are kept (x, y, z in the sort's A keys / A values / B
  // values, idle until the sort) so that the Morton pass does not gather the
  // vertices again
  float* cent = at<float>(base, L.akeys);
  const size_t cstride = (L.avals - L.akeys) / 4;
  // Meshes with few shared vertices (triangle soups: V >= 2T) store each
  // triangle's box too, so that the refit reads one box per leaf instead of
  // gathering three scattered vertices in sorted order (4M-triangle soup:
  // refit 0.89 -> 0.63 ms).  Where vertices are shared the gathers are
  // cache-friendly and the extra store costs more than it saves (2M torus:
  // +8 us in the centroid pass, -3 us in the refit).
  float* tribox = num_vtx >= 2ull * T ? at<float>(base, L.tribox) : nullptr;
  // Meshes whose tiles fit on the GPU at once: centroids, fit, codes and the
  // four passes in one cooperative launch, computed -> (ak, av) -> (codes,
  // bv) -> (ak, av) -> (ok, ov), by default (codes, bv); other_end then takes
  // ak.  The profile's Morton stage is then empty and its sort stage covers
  // the whole front.
  bool front = false;
  if (try_front) {
    uint32_t* ok = idx2morton_out ? idx2morton_out : codes;
    uint32_t* ov = idx2tri_out ? idx2tri_out : bv;
    if (ev) DM_CUDA(cudaEventRecord(ev[1], s));
    front = dm::launch_build_front(s, T, tri2vtx, num_vtx, vtx2xyz, tribox, at<float>(base, L.partials),
                                   dm::kAabbBlocks, transform, at<float>(base, L.aabb), tri2morton_out, ak, av, codes,
                                   bv, ok, ov, at<uint32_t>(base, L.front_counts),
                                   at<uint32_t>(base, L.front_totals), at<uint32_t>(base, L.front_bar), status);
  }
  uint32_t* ok;
  uint32_t* ov;
  uint32_t* other_end;
  if (front) {
    ok = idx2morton_out ? idx2morton_out : codes;
    ov = idx2tri_out ? idx2tri_out : bv;
    other_end = other_end_out ? other_end_out : ak;
  } else {
    if (try_front)  // the cooperative launch was refused: zero what the separate kernels need
      DM_CUDA(cudaMemsetAsync(at<char>(base, L.sort_hdr), 0, SL.zero_bytes, s));
    dm::launch_centroid_aabb(s, T, tri2vtx, num_vtx, vtx2xyz, at<float>(base, L.partials),
                             at<uint32_t>(base, L.ticket), at<float>(base, L.aabb), transform, status, cent, cstride,
                             tribox);
    dm::launch_morton_tri(s, T, tri2vtx, num_vtx, vtx2xyz, transform, codes, hist, status, cent, cstride, radix10);
    if (tri2morton_out) DM_CUDA(cudaMemcpyAsync(tri2morton_out, codes, size_t{4} * T, cudaMemcpyDeviceToDevice, s));
    // 3 passes: codes -> (ak, av) -> (codes, bv) -> (ok, ov), by default the A
    //   buffers (dead after pass 2); other_end then takes bv.
    // 4 passes: codes -> (ak, av) -> (codes, bv) -> (ak, av) -> (ok, ov), by
    //   default (codes, bv) (dead after pass 2); other_end then takes ak.
    ok = idx2morton_out ? idx2morton_out : (radix10 ? ak : codes);
    ov = idx2tri_out ? idx2tri_out : (radix10 ? av : bv);
    if (ev) DM_CUDA(cudaEventRecord(ev[1], s));
    if (radix10) sort3(s, T, codes, ak, av, codes, bv, ok, ov, hist, counters, lookback, status);
    else sort4(s, T, codes, ak, av, codes, bv, ok, ov, hist, counters, lookback, status);
    other_end = other_end_out ? other_end_out : (radix10 ? bv : ak);
  }
  if (ev) DM_CUDA(cudaEventRecord(ev[2], s));
  dm::launch_topology(s, T, ok, ov, bvhnodes, other_end, bt.topo_threads);
  if (ev) DM_CUDA(cudaEventRecord(ev[3], s));
  // the height is only computed on request: it needs the tree-order climb
  dm::launch_refit_windowed(s, T, dm::Segments{1, nullptr, nullptr}, num_vtx, bvhnodes, other_end, tri2vtx, vtx2xyz,
                            nullptr, aabb, flags, height_out ? height : nullptr, status, tribox, false, ov);
  if (ev) DM_CUDA(cudaEventRecord(ev[4], s));
  if (transform_out) DM_CUDA(cudaMemcpyAsync(transform_out, transform, 64, cudaMemcpyDeviceToDevice, s));
  if (height_out) DM_CUDA(cudaMemcpyAsync(height_out, height, 4, cudaMemcpyDeviceToDevice, s));
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}


// ------------------------------------------------------------ batch layout
struct BatchLayout {
  int num_pass;
  size_t hist, counters, lookback, zero_bytes, transforms, keys_a, vals_a, keys_b, vals_b, other, flags, total;
};

BatchLayout batch_layout(uint32_t num_mesh, uint32_t total_tri) {
  BatchLayout L{};
  L.num_pass = dm::batch_num_pass(num_mesh);
  L.hist = 0;
  L.counters = 8 * 256 * 4;
  L.lookback = align256(L.counters + 16 * 4);
  L.zero_bytes = L.lookback + align256(dm::sort_lookback_words(total_tri, L.num_pass) * 4);
  L.transforms = L.zero_bytes;
  L.keys_a = L.transforms + align256(size_t{64} * num_mesh);
  L.vals_a = L.keys_a + align256(size_t{8} * total_tri);
  L.keys_b = L.vals_a + align256(size_t{4} * total_tri);
  L.vals_b = L.keys_b + align256(size_t{8} * total_tri);
  L.other = L.vals_b + align256(size_t{4} * total_tri);
  L.flags = L.other + align256(size_t{4} * total_tri);
  L.total = L.flags + align256(dm::refit_flags_words(total_tri) * 4);
  return L;
}

int check_batch(uint32_t num_mesh, const uint32_t* mesh2tri, const uint32_t* mesh2vtx, uint32_t total_tri,
                uint32_t total_vtx, const uint32_t* tri2vtx, const float* vtx2xyz) {
  DM_REQUIRE(num_mesh >= 1, "num_mesh must be >= 1");
  DM_REQUIRE(total_tri >= num_mesh, "every mesh needs at least one triangle (total_tri %u < num_mesh %u)", total_tri,
             num_mesh);
  DM_REQUIRE(total_tri <= kMaxElems, "total_tri %u exceeds the supported maximum %u", total_tri, kMaxElems);
  DM_REQUIRE(num_mesh <= (1u << 22), "num_mesh %u exceeds the supported maximum 4194304", num_mesh);
  DM_REQUIRE(total_vtx >= 1 && mesh2tri && mesh2vtx && tri2vtx && vtx2xyz, "NULL argument or empty vertex array");
  return DM_OK;
}

}  // namespace

namespace {
// Scratch of the drop-in refit: the derived other range ends, then the
// refit's arrival flags, hand-over queue and segment tree.
size_t refit_any_flags_offset(uint32_t T) { return align256(size_t{4} * T); }
size_t refit_any_scratch_bytes(uint32_t T) {
  return refit_any_flags_offset(T) + align256(size_t{4} * dm::refit_flags_words(T));
}

int refit_any(cudaStream_t s, uint32_t T, const uint32_t* bvhnodes, const uint32_t* tri2vtx, uint32_t V,
              const float* vtx0, const float* vtx1, float* aabb, void* scratch) {
  uint32_t* other_end = static_cast<uint32_t*>(scratch);
  uint32_t* flags = at<uint32_t>(scratch, refit_any_flags_offset(T));
  dm::launch_refit_any_tree(s, T, bvhnodes, tri2vtx, V, vtx0, vtx1, aabb, other_end, flags, status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}
}  // namespace

namespace dm {

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

uint32_t* device_status_word() { return status_ptr(); }

int build_keep_ranges(cudaStream_t s, uint32_t T, const uint32_t* tri2vtx, uint32_t V, const float* vtx2xyz,
                      uint32_t* bvhnodes, float* aabb, uint32_t* other_end_out, void* scratch, size_t scratch_bytes) {
  return build_impl(reinterpret_cast<uint64_t>(s), T, tri2vtx, V, vtx2xyz, bvhnodes, aabb, nullptr, nullptr, nullptr,
                    nullptr, nullptr, scratch, scratch_bytes, nullptr, other_end_out);
}

size_t build_scratch_bytes(uint32_t T) { return build_layout(T).total; }

namespace {
std::mutex g_tuning_mutex;
Tuning g_tuning;
std::atomic<uint32_t> g_wait_limit{kDefaultWaitLimit};
}  // namespace

namespace {
BuildTuning g_build_classes[kMaxBuildClasses];
uint32_t g_num_build_classes = 0;
}  // namespace

BuildTuning build_tuning_for(uint32_t num_tri) {
  std::lock_guard<std::mutex> lk(g_tuning_mutex);
  for (uint32_t i = 0; i < g_num_build_classes; ++i)
    if (num_tri <= g_build_classes[i].max_tri) return g_build_classes[i];
  return BuildTuning{};
}

bool set_build_classes(const BuildTuning* classes, uint32_t n) {
  if (n > static_cast<uint32_t>(kMaxBuildClasses) || (n > 0 && !classes)) return false;
  for (uint32_t i = 0; i < n; ++i) {
    const BuildTuning& c = classes[i];
    if (c.build_path > 1 || !(c.sort_radix == 0 || c.sort_radix == 8 || c.sort_radix == 10)) return false;
    if (!(c.topo_threads == 0 || c.topo_threads == 128 || c.topo_threads == 256 || c.topo_threads == 512))
      return false;
    if (i > 0 && c.max_tri <= classes[i - 1].max_tri) return false;  // ascending bounds
  }
  std::lock_guard<std::mutex> lk(g_tuning_mutex);
  for (uint32_t i = 0; i < n; ++i) g_build_classes[i] = classes[i];
  g_num_build_classes = n;
  return true;
}

uint32_t get_build_classes(BuildTuning* out, uint32_t cap) {
  std::lock_guard<std::mutex> lk(g_tuning_mutex);
  for (uint32_t i = 0; i < g_num_build_classes && i < cap; ++i) out[i] = g_build_classes[i];
  return g_num_build_classes;
}

uint32_t get_wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }
void set_wait_limit(uint32_t polls) { g_wait_limit.store(polls, std::memory_order_relaxed); }

Tuning get_tuning() {
  std::lock_guard<std::mutex> lk(g_tuning_mutex);
  return g_tuning;
}

bool set_tuning(const Tuning& t) {
  bool cast_ok = false;
  for (const auto& v : kCastVariants) cast_ok = cast_ok || (v[0] == t.cast_threads && v[1] == t.cast_stack);
  const bool tile_ok = t.tile_w == 2 || t.tile_w == 4 || t.tile_w == 8 || t.tile_w == 16 || t.tile_w == 32;
  const bool sort_ok = t.sort_window == 4 || t.sort_window == 8;
  const auto phase_ok = [](uint32_t v) { return v >= 1 && v <= 32; };
  if (!cast_ok || !tile_ok || !sort_ok) return false;
  if (!phase_ok(t.cast_refill_min) || !phase_ok(t.cast_leaf_min) || !phase_ok(t.cast_ascend_min)) return false;
  if (t.cast_long_steps < 1 || t.cast_long_steps > (1u << 30)) return false;
  if (t.batch_path > 1 || !(t.batch_cluster <= 2 || t.batch_cluster == 4)) return false;
  std::lock_guard<std::mutex> lk(g_tuning_mutex);
  g_tuning = t;
  return true;
}

}  // namespace dm

extern "C" {

const char* dm_version(void) { return "delmsh_gb300 0.1.0 (sm_103a)"; }

const char* dm_last_error(void) { return g_last_error.c_str(); }

int dm_device_status(uint32_t* bits, int clear) {
  uint32_t* p = status_ptr();
  if (!p) return fail(DM_ERR_CUDA, "device status word unavailable");
  DM_CUDA(cudaDeviceSynchronize());
  uint32_t v = 0;
  DM_CUDA(cudaMemcpy(&v, p, 4, cudaMemcpyDeviceToHost));
  if (clear) DM_CUDA(cudaMemset(p, 0, 4));
  if (bits) *bits = v;
  return DM_OK;
}

int dm_tuning_get(dm_tuning* out) {
  DM_REQUIRE(out, "NULL argument");
  const dm::Tuning t = dm::get_tuning();
  *out = dm_tuning{t.cast_threads,    t.cast_stack,    t.tile_w,          t.sort_window,
                   t.cast_refill_min, t.cast_leaf_min, t.cast_ascend_min, t.cast_long_steps,
                   t.batch_path,      t.batch_cluster};
  return DM_OK;
}

int dm_tuning_set(const dm_tuning* in) {
  DM_REQUIRE(in, "NULL argument");
  dm::Tuning t;
  t.cast_threads = in->cast_threads;
  t.cast_stack = in->cast_stack;
  t.tile_w = in->tile_w;
  t.sort_window = in->sort_window;
  const auto phase = [](uint32_t v) { return v == 0 ? dm::kDefaultPhaseMin : v; };
  t.cast_refill_min = phase(in->cast_refill_min);
  t.cast_leaf_min = phase(in->cast_leaf_min);
  t.cast_ascend_min = phase(in->cast_ascend_min);
  t.cast_long_steps = in->cast_long_steps == 0 ? dm::kDefaultLongSteps : in->cast_long_steps;
  t.batch_path = in->batch_path;
  t.batch_cluster = in->batch_cluster;
  DM_REQUIRE(dm::set_tuning(t),
             "unsupported tuning (cast %u threads x %u frames, tile_w %u, sort window %u, phase minima %u/%u/%u, "
             "long-ray steps %u, batch path %u, batch cluster %u)",
             in->cast_threads, in->cast_stack, in->tile_w, in->sort_window, t.cast_refill_min, t.cast_leaf_min,
             t.cast_ascend_min, t.cast_long_steps, t.batch_path, t.batch_cluster);
  return DM_OK;
}

int dm_build_classes_set(const dm_build_class* classes, uint32_t num_class) {
  DM_REQUIRE(num_class <= static_cast<uint32_t>(dm::kMaxBuildClasses), "at most %d build classes",
             dm::kMaxBuildClasses);
  DM_REQUIRE(num_class == 0 || classes, "NULL argument");
  dm::BuildTuning b[dm::kMaxBuildClasses];
  for (uint32_t i = 0; i < num_class; ++i)
    b[i] = dm::BuildTuning{classes[i].max_tri, classes[i].build_path, classes[i].sort_radix, classes[i].topo_threads};
  DM_REQUIRE(dm::set_build_classes(b, num_class),
             "unsupported build classes (bounds must ascend; build_path 0/1, sort_radix 0/8/10, topo_threads "
             "0/128/256/512)");
  return DM_OK;
}

int dm_build_classes_get(dm_build_class* out, uint32_t capacity, uint32_t* num_class) {
  DM_REQUIRE(num_class && (capacity == 0 || out), "NULL argument");
  dm::BuildTuning b[dm::kMaxBuildClasses];
  const uint32_t n = dm::get_build_classes(b, dm::kMaxBuildClasses);
  for (uint32_t i = 0; i < n && i < capacity; ++i)
    out[i] = dm_build_class{b[i].max_tri, b[i].build_path, b[i].sort_radix, b[i].topo_threads};
  *num_class = n;
  return DM_OK;
}

int dm_wait_limit_get(uint32_t* polls) {
  DM_REQUIRE(polls, "NULL argument");
  *polls = dm::get_wait_limit();
  return DM_OK;
}

int dm_wait_limit_set(uint32_t polls) {
  dm::set_wait_limit(polls == 0 ? dm::kDefaultWaitLimit : polls);
  return DM_OK;
}

size_t dm_selftest_bounded_wait_scratch_bytes(void) { return 4 * (3 * dm::kSortTile + 256 + 2 * 256 + 64); }

int dm_selftest_bounded_wait(uint64_t stream_ptr, uint32_t polls, void* scratch, size_t scratch_bytes) {
  DM_REQUIRE(polls >= 1 && polls <= (1u << 24), "polls must be in 1..2^24 (got %u)", polls);
  DM_REQUIRE(scratch, "scratch must not be NULL");
  const size_t need = dm_selftest_bounded_wait_scratch_bytes();
  DM_REQUIRE(scratch_bytes >= need, "scratch of %zu bytes is below the %zu needed", scratch_bytes, need);
  cudaStream_t s = as_stream(stream_ptr);
  uint32_t* w = static_cast<uint32_t*>(scratch);
  uint32_t* keys_in = w;                           // kSortTile keys (0)
  uint32_t* keys_out = keys_in + dm::kSortTile;    // never written (the tile holds no keys)
  uint32_t* vals_out = keys_out + dm::kSortTile;
  uint32_t* hist = vals_out + dm::kSortTile;       // 256 digit counts: all keys have digit 0
  uint32_t* lookback = hist + 256;                 // tiles 0 and 1, zero: tile 0 never publishes
  uint32_t* counter = lookback + 2 * 256;          // preset to 1: the only block draws tile 1
  DM_CUDA(cudaMemsetAsync(scratch, 0, need, s));
  const uint32_t n = dm::kSortTile, one = 1;
  DM_CUDA(cudaMemcpyAsync(hist, &n, 4, cudaMemcpyHostToDevice, s));
  DM_CUDA(cudaMemcpyAsync(counter, &one, 4, cudaMemcpyHostToDevice, s));
  dm::launch_onesweep_wait_probe(s, n, keys_in, keys_out, vals_out, hist, lookback, counter, status_ptr(), polls);
  DM_CUDA(cudaGetLastError());
  DM_CUDA(cudaStreamSynchronize(s));  // the host values above are stack copies
  return DM_OK;
}

int dm_mortons_vtx2morton_from_vtx2co(uint64_t stream_ptr, uint32_t num_vtx, uint32_t num_dim, const float* vtx2co,
                                      const float* transform_co2unit, uint32_t* vtx2morton) {
  DM_REQUIRE(num_dim == 2 || num_dim == 3, "num_dim must be 2 or 3 (got %u)", num_dim);
  DM_REQUIRE(transform_co2unit && vtx2morton && (vtx2co || num_vtx == 0), "NULL argument");
  if (num_vtx == 0) return DM_OK;
  dm::launch_vtx2morton(as_stream(stream_ptr), num_vtx, num_dim, vtx2co, transform_co2unit, vtx2morton);
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

size_t dm_array1d_argsort_scratch_bytes(uint32_t n) { return sort_layout(n, 4, 4).total; }

int dm_array1d_argsort(uint64_t stream_ptr, uint32_t n, uint32_t* idx2val, uint32_t* jdx2idx, void* scratch,
                       size_t scratch_bytes) {
  DM_REQUIRE(n <= kMaxElems, "n %u exceeds the supported maximum %u", n, kMaxElems);
  if (n == 0) return DM_OK;
  DM_REQUIRE(idx2val && jdx2idx, "NULL argument");
  cudaStream_t s = as_stream(stream_ptr);
  const SortLayout L = sort_layout(n, 4, 4);
  Scratch sc;
  if (int e = sc.acquire(scratch, scratch_bytes, L.total, s, nullptr)) return e;
  void* base = sc.ptr;
  DM_CUDA(cudaMemsetAsync(base, 0, L.zero_bytes, s));
  uint32_t* hist = at<uint32_t>(base, L.hist);
  uint32_t* tk = at<uint32_t>(base, L.keys);
  uint32_t* tv = at<uint32_t>(base, L.vals);
  dm::launch_digit_hist_u32(s, n, idx2val, 4, hist);
  sort4(s, n, idx2val, tk, tv, idx2val, jdx2idx, idx2val, jdx2idx, hist, at<uint32_t>(base, L.counters),
        at<uint32_t>(base, L.lookback), status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_mortons_make_bvhnodes_from_sorted_mortons(uint64_t stream_ptr, uint32_t n, const uint32_t* idx2obj,
                                                 const uint32_t* idx2morton, uint32_t* bvhnodes) {
  DM_REQUIRE(n >= 1, "n must be >= 1");
  DM_REQUIRE(n <= kMaxElems, "n %u exceeds the supported maximum %u", n, kMaxElems);
  DM_REQUIRE(idx2obj && idx2morton && bvhnodes, "NULL argument");
  dm::launch_topology(as_stream(stream_ptr), n, idx2morton, idx2obj, bvhnodes);
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_bvhnode2aabb_update_aabb(uint64_t stream_ptr, uint32_t num_bvhnode, float* bvhnode2aabb, uint32_t i_bvhnode,
                                const uint32_t* bvhnodes, uint32_t num_elem, const uint32_t* elem2vtx,
                                uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1,
                                uint32_t* flags_scratch) {
  if (int e = check_mesh(num_elem, elem2vtx, num_vtx, vtx2xyz0)) return e;
  DM_REQUIRE(num_bvhnode == 2 * num_elem - 1, "num_bvhnode (%u) must be 2*num_elem-1 (%u)", num_bvhnode,
             2 * num_elem - 1);
  DM_REQUIRE(i_bvhnode == 0, "only i_bvhnode == 0 (the whole tree) is supported");
  DM_REQUIRE(bvhnode2aabb && bvhnodes, "NULL argument");
  cudaStream_t s = as_stream(stream_ptr);
  if (flags_scratch) {  // the caller's arrival flags alone: the parent-pointer climb
    dm::launch_refit(s, num_elem, bvhnodes, elem2vtx, num_vtx, vtx2xyz0, vtx2xyz1, bvhnode2aabb, flags_scratch,
                     nullptr, status_ptr());
    DM_CUDA(cudaGetLastError());
    return DM_OK;
  }
  Scratch sc;
  bool fresh = false;
  const size_t need = refit_any_scratch_bytes(num_elem);
  if (int e = sc.acquire(nullptr, 0, need, s, &fresh)) return e;
  DM_CUDA(cudaMemsetAsync(static_cast<unsigned char*>(sc.ptr) + refit_any_flags_offset(num_elem), 0,
                          size_t{4} * num_elem, s));
  return refit_any(s, num_elem, bvhnodes, elem2vtx, num_vtx, vtx2xyz0, vtx2xyz1, bvhnode2aabb, sc.ptr);
}

size_t dm_bvhnode2aabb_update_aabb_scratch_bytes(uint32_t num_elem) { return refit_any_scratch_bytes(num_elem); }

int dm_bvhnode2aabb_update_aabb_ex(uint64_t stream_ptr, uint32_t num_bvhnode, float* bvhnode2aabb,
                                   const uint32_t* bvhnodes, uint32_t num_elem, const uint32_t* elem2vtx,
                                   uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1, void* scratch,
                                   size_t scratch_bytes) {
  if (int e = check_mesh(num_elem, elem2vtx, num_vtx, vtx2xyz0)) return e;
  DM_REQUIRE(num_bvhnode == 2 * num_elem - 1, "num_bvhnode (%u) must be 2*num_elem-1 (%u)", num_bvhnode,
             2 * num_elem - 1);
  DM_REQUIRE(bvhnode2aabb && bvhnodes && scratch, "NULL argument");
  const size_t need = refit_any_scratch_bytes(num_elem);
  DM_REQUIRE(scratch_bytes >= need, "scratch of %zu bytes is below the %zu needed", scratch_bytes, need);
  return refit_any(as_stream(stream_ptr), num_elem, bvhnodes, elem2vtx, num_vtx, vtx2xyz0, vtx2xyz1, bvhnode2aabb,
                   scratch);
}

size_t dm_trimesh3_build_scratch_bytes(uint32_t num_tri) { return build_layout(num_tri).total; }

int dm_trimesh3_make_bvhnodes_bvhnode2aabb(uint64_t stream_ptr, uint32_t num_tri, const uint32_t* tri2vtx,
                                           uint32_t num_vtx, const float* vtx2xyz, uint32_t* bvhnodes,
                                           float* bvhnode2aabb, void* scratch, size_t scratch_bytes) {
  return build_impl(stream_ptr, num_tri, tri2vtx, num_vtx, vtx2xyz, bvhnodes, bvhnode2aabb, nullptr, nullptr, nullptr,
                    nullptr, nullptr, scratch, scratch_bytes);
}

int dm_trimesh3_build_ex(uint64_t stream_ptr, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                         const float* vtx2xyz, uint32_t* bvhnodes, float* bvhnode2aabb, float* transform_out,
                         uint32_t* tri2morton_out, uint32_t* idx2tri_out, uint32_t* idx2morton_out,
                         uint32_t* height_out, void* scratch, size_t scratch_bytes) {
  return build_impl(stream_ptr, num_tri, tri2vtx, num_vtx, vtx2xyz, bvhnodes, bvhnode2aabb, transform_out,
                    tri2morton_out, idx2tri_out, idx2morton_out, height_out, scratch, scratch_bytes);
}

int dm_trimesh3_build_profiled(uint64_t stream_ptr, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                               const float* vtx2xyz, uint32_t* bvhnodes, float* bvhnode2aabb, void* scratch,
                               size_t scratch_bytes, float* stage_ms) {
  DM_REQUIRE(stage_ms, "stage_ms must not be NULL");
  cudaEvent_t ev[5] = {};
  for (auto& e : ev) DM_CUDA(cudaEventCreate(&e));
  int rc = build_impl(stream_ptr, num_tri, tri2vtx, num_vtx, vtx2xyz, bvhnodes, bvhnode2aabb, nullptr, nullptr,
                      nullptr, nullptr, nullptr, scratch, scratch_bytes, ev);
  if (rc == DM_OK) {
    const cudaError_t e = cudaEventSynchronize(ev[4]);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventSynchronize");
    for (int i = 0; rc == DM_OK && i < 4; ++i) cudaEventElapsedTime(stage_ms + i, ev[i], ev[i + 1]);
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

size_t dm_cast_scratch_bytes(uint32_t num_ray, uint32_t num_tri) { return dm::cast_scratch_bytes(num_ray, num_tri); }

int dm_pix2tri_by_raycast(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, uint32_t* pix2tri, float* pix2t,
                          uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz,
                          const uint32_t* bvhnodes, const float* bvhnode2aabb, const float* transform_ndc2world,
                          void* scratch, size_t scratch_bytes) {
  if (int e = check_mesh(num_tri, tri2vtx, num_vtx, vtx2xyz)) return e;
  DM_REQUIRE(bvhnodes && bvhnode2aabb && transform_ndc2world && pix2tri, "NULL argument");
  const uint64_t num_pix = static_cast<uint64_t>(img_w) * img_h;
  DM_REQUIRE(num_pix <= kMaxElems, "image of %llu pixels exceeds the supported maximum", (unsigned long long)num_pix);
  DM_REQUIRE(padded_pixel_work(img_w, img_h, 1) <= kMaxElems,
             "image of %u x %u pixels pads to too many tile slots", img_w, img_h);
  if (num_pix == 0) return DM_OK;
  cudaStream_t s = as_stream(stream_ptr);
  const uint32_t n = static_cast<uint32_t>(num_pix);
  Scratch sc;
  if (int e = sc.acquire(scratch, scratch_bytes, dm::cast_scratch_bytes(n, num_tri), s, nullptr)) return e;
  dm::CastScratch cs;
  dm::cast_scratch_carve(sc.ptr, n, num_tri, &cs);
  DM_CUDA(cudaMemsetAsync(cs.counters, 0, 16, s));
  dm::MeshView m{num_tri, num_vtx, tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb};
  dm::CastOut o{pix2tri, pix2t, nullptr};
  dm::launch_cast_pixels(s, img_w, img_h, transform_ndc2world, m, o, cs, status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_search_bvh3_first_intersection_ray(uint64_t stream_ptr, uint32_t num_ray, const float* ray_org,
                                          const float* ray_dir, uint32_t* hit_tri, float* hit_t, float* hit_bc,
                                          uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                                          const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb,
                                          void* scratch, size_t scratch_bytes) {
  if (int e = check_mesh(num_tri, tri2vtx, num_vtx, vtx2xyz)) return e;
  DM_REQUIRE(num_ray <= kMaxElems, "num_ray %u exceeds the supported maximum", num_ray);
  if (num_ray == 0) return DM_OK;
  DM_REQUIRE(ray_org && ray_dir && hit_tri && bvhnodes && bvhnode2aabb, "NULL argument");
  cudaStream_t s = as_stream(stream_ptr);
  Scratch sc;
  if (int e = sc.acquire(scratch, scratch_bytes, dm::cast_scratch_bytes(num_ray, num_tri), s, nullptr)) return e;
  dm::CastScratch cs;
  dm::cast_scratch_carve(sc.ptr, num_ray, num_tri, &cs);
  DM_CUDA(cudaMemsetAsync(cs.counters, 0, 16, s));
  dm::MeshView m{num_tri, num_vtx, tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb};
  dm::CastOut o{hit_tri, hit_t, hit_bc};
  dm::launch_cast_rays(s, num_ray, ray_org, ray_dir, m, o, cs, status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_pix2depth_update(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, float* pix2depth,
                        const uint32_t* pix2tri, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                        const float* vtx2xyz, const float* transform_ndc2world, void* scratch, size_t scratch_bytes) {
  if (int e = check_mesh(num_tri, tri2vtx, num_vtx, vtx2xyz)) return e;
  DM_REQUIRE(static_cast<uint64_t>(img_w) * img_h <= kMaxElems, "image of %u x %u pixels is too large", img_w, img_h);
  DM_REQUIRE(pix2depth && pix2tri && transform_ndc2world, "NULL argument");
  cudaStream_t s = as_stream(stream_ptr);
  Scratch sc;
  if (int e = sc.acquire(scratch, scratch_bytes, dm_render_scratch_bytes(), s, nullptr)) return e;
  float* world2ndc = static_cast<float*>(sc.ptr);
  dm::launch_inverse4(s, transform_ndc2world, world2ndc, status_ptr());
  dm::MeshView m{num_tri, num_vtx, tri2vtx, vtx2xyz, nullptr, nullptr};
  dm::launch_pix2depth(s, img_w, img_h, pix2depth, pix2tri, m, transform_ndc2world, world2ndc, status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_pix2depth_bwd_wrt_vtx2xyz(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, float* dldw_vtx2xyz,
                                 const uint32_t* pix2tri, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                                 const float* vtx2xyz, const float* dldw_pix2depth, const float* transform_ndc2world,
                                 void* scratch, size_t scratch_bytes) {
  if (int e = check_mesh(num_tri, tri2vtx, num_vtx, vtx2xyz)) return e;
  DM_REQUIRE(static_cast<uint64_t>(img_w) * img_h <= kMaxElems, "image of %u x %u pixels is too large", img_w, img_h);
  DM_REQUIRE(dldw_vtx2xyz && pix2tri && dldw_pix2depth && transform_ndc2world, "NULL argument");
  cudaStream_t s = as_stream(stream_ptr);
  Scratch sc;
  if (int e = sc.acquire(scratch, scratch_bytes, dm_render_scratch_bytes(), s, nullptr)) return e;
  float* world2ndc = static_cast<float*>(sc.ptr);
  dm::launch_inverse4(s, transform_ndc2world, world2ndc, status_ptr());
  dm::MeshView m{num_tri, num_vtx, tri2vtx, vtx2xyz, nullptr, nullptr};
  dm::launch_pix2depth_bwd(s, img_w, img_h, dldw_vtx2xyz, pix2tri, m, dldw_pix2depth, transform_ndc2world, world2ndc,
                           status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

size_t dm_render_scratch_bytes(void) { return 256; }

int dm_pix2tri_interpolate(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri,
                           uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz,
                           uint32_t num_vdim, const float* vtx2val, const float* transform_ndc2world, float* pix2val) {
  if (int e = check_mesh(num_tri, tri2vtx, num_vtx, vtx2xyz)) return e;
  DM_REQUIRE(static_cast<uint64_t>(img_w) * img_h * (num_vdim ? num_vdim : 1) <= (uint64_t{1} << 32) - 1,
             "image of %u x %u x %u values is too large", img_w, img_h, num_vdim);
  DM_REQUIRE(num_vdim >= 1, "num_vdim must be >= 1");
  DM_REQUIRE(pix2tri && vtx2val && transform_ndc2world && pix2val, "NULL argument");
  dm::MeshView m{num_tri, num_vtx, tri2vtx, vtx2xyz, nullptr, nullptr};
  dm::launch_interpolate(as_stream(stream_ptr), img_w, img_h, pix2tri, m, num_vdim, vtx2val, transform_ndc2world,
                         pix2val, status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_pix2tri_interpolate_bwd(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri,
                               uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz,
                               uint32_t num_vdim, const float* vtx2val, const float* transform_ndc2world,
                               const float* dldw_pix2val, float* dldw_vtx2xyz, float* dldw_vtx2val) {
  if (int e = check_mesh(num_tri, tri2vtx, num_vtx, vtx2xyz)) return e;
  DM_REQUIRE(static_cast<uint64_t>(img_w) * img_h * (num_vdim ? num_vdim : 1) <= (uint64_t{1} << 32) - 1,
             "image of %u x %u x %u values is too large", img_w, img_h, num_vdim);
  DM_REQUIRE(num_vdim >= 1, "num_vdim must be >= 1");
  DM_REQUIRE(pix2tri && vtx2val && transform_ndc2world && dldw_pix2val && dldw_vtx2xyz && dldw_vtx2val,
             "NULL argument");
  dm::MeshView m{num_tri, num_vtx, tri2vtx, vtx2xyz, nullptr, nullptr};
  dm::launch_interpolate_bwd(as_stream(stream_ptr), img_w, img_h, pix2tri, m, num_vdim, vtx2val, transform_ndc2world,
                             dldw_pix2val, dldw_vtx2xyz, dldw_vtx2val, status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

size_t dm_quad_oct_tree_scratch_bytes(uint32_t num_idx) { return dm::octree_scratch_bytes(num_idx); }

int dm_quad_oct_tree_bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode(
    uint64_t stream_ptr, uint32_t num_idx, const uint32_t* idx2morton, uint32_t num_dim, uint32_t max_depth,
    uint32_t* bnodes, uint32_t* bnode2depth, uint32_t* bnode2onode, uint32_t* idx2bnode, void* scratch,
    size_t scratch_bytes) {
  DM_REQUIRE(num_idx >= 2, "num_idx must be >= 2 (got %u)", num_idx);
  DM_REQUIRE(num_idx <= kMaxElems, "num_idx %u exceeds the supported maximum", num_idx);
  DM_REQUIRE(num_dim == 2 || num_dim == 3, "num_dim must be 2 or 3 (got %u)", num_dim);
  DM_REQUIRE(max_depth >= 1 && num_dim * max_depth <= 32, "num_dim * max_depth must be in 1..32");
  DM_REQUIRE(idx2morton && bnodes && bnode2depth && bnode2onode && idx2bnode, "NULL argument");
  cudaStream_t s = as_stream(stream_ptr);
  Scratch sc;
  if (int e = sc.acquire(scratch, scratch_bytes, dm::octree_scratch_bytes(num_idx), s, nullptr)) return e;
  dm::launch_octree_brt(s, num_idx, idx2morton, num_dim, max_depth, bnodes, bnode2depth, bnode2onode, idx2bnode,
                        static_cast<uint32_t*>(sc.ptr), status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_quad_oct_tree_make_tree_from_binary_radix_tree(
    uint64_t stream_ptr, uint32_t num_idx, const uint32_t* bnodes, const uint32_t* bnode2onode,
    const uint32_t* bnode2depth, const uint32_t* idx2bnode, const uint32_t* idx2morton, uint32_t num_dim,
    uint32_t max_depth, uint32_t num_onode, uint32_t* onodes, uint32_t* onode2depth, float* onode2center,
    uint32_t* idx2onode, float* idx2center) {
  DM_REQUIRE(num_idx >= 2 && num_idx <= kMaxElems, "num_idx must be in 2..%u (got %u)", kMaxElems, num_idx);
  DM_REQUIRE(num_dim == 2 || num_dim == 3, "num_dim must be 2 or 3 (got %u)", num_dim);
  DM_REQUIRE(max_depth >= 1 && num_dim * max_depth <= 32, "num_dim * max_depth must be in 1..32");
  DM_REQUIRE(num_onode >= 1 && num_onode <= num_idx - 1, "num_onode must be in 1..num_idx-1 (got %u)", num_onode);
  DM_REQUIRE(bnodes && bnode2onode && bnode2depth && idx2bnode && idx2morton && onodes && onode2depth &&
                 onode2center && idx2onode && idx2center,
             "NULL argument");
  dm::launch_octree_make(as_stream(stream_ptr), num_idx, bnodes, bnode2onode, bnode2depth, idx2bnode, idx2morton,
                         num_onode, max_depth, num_dim, onodes, onode2depth, onode2center, idx2onode, idx2center,
                         status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_quad_oct_tree_aggregate(uint64_t stream_ptr, uint32_t num_idx, uint32_t num_vdim, const float* idx2val,
                               const uint32_t* idx2onode, uint32_t num_link, const uint32_t* onodes,
                               uint32_t num_onode, float* onode2aggval) {
  DM_REQUIRE(num_link == 5 || num_link == 9, "num_link must be 5 (quadtree) or 9 (octree), got %u", num_link);
  DM_REQUIRE(idx2val && idx2onode && onodes && onode2aggval, "NULL argument");
  cudaStream_t s = as_stream(stream_ptr);
  DM_CUDA(cudaMemsetAsync(onode2aggval, 0, sizeof(float) * num_onode * num_vdim, s));
  dm::launch_octree_aggregate(s, num_idx, num_vdim, idx2val, idx2onode, num_link, onodes, num_onode, onode2aggval,
                              status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

int dm_trimesh3_self_intersection(uint64_t stream_ptr, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                                  const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb,
                                  uint32_t capacity, uint32_t* pairs, float* segments, uint32_t* count) {
  if (int e = check_mesh(num_tri, tri2vtx, num_vtx, vtx2xyz)) return e;
  DM_REQUIRE(bvhnodes && bvhnode2aabb && count && (capacity == 0 || (pairs && segments)), "NULL argument");
  cudaStream_t s = as_stream(stream_ptr);
  Scratch sc;
  const size_t need = dm::self_intersection_scratch_bytes(num_tri);
  if (int e = sc.acquire(nullptr, 0, need, s, nullptr)) return e;
  DM_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), s));
  dm::MeshView m{num_tri, num_vtx, tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb};
  if (dm::launch_self_intersection(s, m, capacity, pairs, segments, count, sc.ptr, need, status_ptr()) != 0)
    return fail(DM_ERR_CUDA, "self-intersection round failed: %s", cudaGetErrorString(cudaGetLastError()));
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

size_t dm_batch_build_scratch_bytes(uint32_t num_mesh, uint32_t total_tri) {
  return batch_layout(num_mesh, total_tri).total;
}

int dm_batch_trimesh3_build(uint64_t stream_ptr, uint32_t num_mesh, const uint32_t* mesh2tri,
                            const uint32_t* mesh2vtx, uint32_t total_tri, uint32_t total_vtx,
                            uint32_t max_tri_per_mesh, const uint32_t* tri2vtx, const float* vtx2xyz,
                            uint32_t* bvhnodes, float* bvhnode2aabb, uint32_t* heights, void* scratch,
                            size_t scratch_bytes) {
  if (int e = check_batch(num_mesh, mesh2tri, mesh2vtx, total_tri, total_vtx, tri2vtx, vtx2xyz)) return e;
  DM_REQUIRE(bvhnodes && bvhnode2aabb, "NULL argument");
  DM_REQUIRE(max_tri_per_mesh >= 1 && max_tri_per_mesh <= total_tri, "max_tri_per_mesh must be in 1..total_tri");
  cudaStream_t s = as_stream(stream_ptr);
  const BatchLayout L = batch_layout(num_mesh, total_tri);
  Scratch sc;
  if (int e = sc.acquire(scratch, scratch_bytes, L.total, s, nullptr)) return e;
  void* base = sc.ptr;
  uint32_t* status = status_ptr();
  const dm::Segments seg{num_mesh, mesh2tri, mesh2vtx};
  DM_CUDA(cudaMemsetAsync(at<char>(base, L.flags), 0, size_t{4} * total_tri, s));
  if (max_tri_per_mesh <= dm::kSegMaxTri && dm::get_tuning().batch_path == 0) {
    // every mesh sorted and linked on chip (the lists reuse the key buffer)
    uint32_t* seg_counters = at<uint32_t>(base, L.counters) + 8;
    DM_CUDA(cudaMemsetAsync(seg_counters, 0, 4 * sizeof(uint32_t), s));
    if (dm::launch_batch_seg_build(s, seg, max_tri_per_mesh, tri2vtx, vtx2xyz, bvhnodes, at<uint32_t>(base, L.other),
                                   at<uint32_t>(base, L.keys_a), seg_counters, status) != 0)
      return fail(DM_ERR_CUDA, "fused batch build launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    dm::launch_refit_windowed(s, total_tri, seg, 0, bvhnodes, at<uint32_t>(base, L.other), tri2vtx, vtx2xyz, nullptr,
                              bvhnode2aabb, at<uint32_t>(base, L.flags), heights, status);
    DM_CUDA(cudaGetLastError());
    return DM_OK;
  }
  DM_CUDA(cudaMemsetAsync(base, 0, L.zero_bytes, s));
  float* transforms = at<float>(base, L.transforms);
  uint32_t* hist = at<uint32_t>(base, L.hist);
  uint32_t* counters = at<uint32_t>(base, L.counters);
  uint32_t* lookback = at<uint32_t>(base, L.lookback);
  uint64_t* ka = at<uint64_t>(base, L.keys_a);
  uint64_t* kb = at<uint64_t>(base, L.keys_b);
  uint32_t* va = at<uint32_t>(base, L.vals_a);
  uint32_t* vb = at<uint32_t>(base, L.vals_b);
  dm::launch_batch_fit(s, seg, tri2vtx, vtx2xyz, transforms, status);
  dm::launch_batch_morton(s, total_tri, seg, tri2vtx, vtx2xyz, transforms, ka, hist, L.num_pass, status);
  const size_t lbw = dm::sort_lookback_words(total_tri, 1);
  uint64_t *ks = ka, *kd = kb;
  uint32_t *vs = nullptr, *vd = vb;
  for (int p = 0; p < L.num_pass; ++p) {
    dm::launch_onesweep_u64(s, total_tri, 8u * p, ks, vs, kd, vd, hist + 256 * p, lookback + lbw * p, counters + p,
                            status);
    std::swap(ks, kd);
    vs = vd;
    vd = (vd == vb) ? va : vb;
  }
  dm::launch_batch_topology(s, total_tri, seg, ks, vs, bvhnodes, at<uint32_t>(base, L.other));
  dm::launch_refit_windowed(s, total_tri, seg, 0, bvhnodes, at<uint32_t>(base, L.other), tri2vtx, vtx2xyz, nullptr,
                            bvhnode2aabb, at<uint32_t>(base, L.flags), heights, status);
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

size_t dm_batch_cast_scratch_bytes(uint32_t num_ray, uint32_t max_tri_per_mesh) {
  return dm::cast_scratch_bytes(num_ray, max_tri_per_mesh);
}

int dm_batch_pix2tri_by_raycast(uint64_t stream_ptr, uint32_t num_mesh, const uint32_t* mesh2tri,
                                const uint32_t* mesh2vtx, uint32_t total_tri, uint32_t total_vtx,
                                uint32_t max_tri_per_mesh, const uint32_t* tri2vtx, const float* vtx2xyz,
                                const uint32_t* bvhnodes, const float* bvhnode2aabb, uint32_t img_w, uint32_t img_h,
                                const float* transforms_ndc2world, uint32_t* pix2tri, float* pix2t, void* scratch,
                                size_t scratch_bytes) {
  if (int e = check_batch(num_mesh, mesh2tri, mesh2vtx, total_tri, total_vtx, tri2vtx, vtx2xyz)) return e;
  DM_REQUIRE(bvhnodes && bvhnode2aabb && transforms_ndc2world && pix2tri, "NULL argument");
  DM_REQUIRE(max_tri_per_mesh >= 1 && max_tri_per_mesh <= total_tri, "max_tri_per_mesh must be in 1..total_tri");
  const uint64_t num_ray = static_cast<uint64_t>(img_w) * img_h * num_mesh;
  DM_REQUIRE(num_ray <= kMaxElems, "%llu rays exceed the supported maximum", (unsigned long long)num_ray);
  DM_REQUIRE(padded_pixel_work(img_w, img_h, num_mesh) <= kMaxElems,
             "%u images of %u x %u pixels pad to too many tile slots", num_mesh, img_w, img_h);
  if (num_ray == 0) return DM_OK;
  cudaStream_t s = as_stream(stream_ptr);
  Scratch sc;
  const uint32_t n = static_cast<uint32_t>(num_ray);
  if (int e = sc.acquire(scratch, scratch_bytes, dm::cast_scratch_bytes(n, max_tri_per_mesh), s, nullptr)) return e;
  dm::CastScratch cs;
  dm::cast_scratch_carve(sc.ptr, n, max_tri_per_mesh, &cs);
  DM_CUDA(cudaMemsetAsync(cs.counters, 0, 16, s));
  dm::CastOut o{pix2tri, pix2t, nullptr};
  dm::launch_batch_cast_pixels(s, dm::Segments{num_mesh, mesh2tri, mesh2vtx}, max_tri_per_mesh, tri2vtx, vtx2xyz,
                               bvhnodes, bvhnode2aabb, img_w, img_h, transforms_ndc2world, o, cs, status_ptr());
  DM_CUDA(cudaGetLastError());
  return DM_OK;
}

}  // extern "C"
