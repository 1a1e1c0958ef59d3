// server.cpp -- a request loop with continuous batching (s2tc_server_*).
//
// Clients submit compression requests (host pixels in, host blocks out) from
// any thread.  One scheduler thread admits waiting requests in arrival order
// while their device memory fits the budget (one pool, sub-allocated), and
// launches every group of admitted requests as a round: the uploads on a copy
// stream, then per knob combination one batched dither launch and one
// batched encoder launch per block format on a compute stream, then the
// downloads.  Rounds use separate streams and slots, so a round admitted
// while earlier ones are still on the GPU overlaps them; a request's memory
// returns to the pool when its download completes.  The kernels and bytes are
// exactly those of tx_compress_dxtn for each request.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dither.h"
#include "encode.h"
#include "rand_glibc.h"
#include "s2tc_gb300.h"
#include "s2tc_types.h"

namespace s2tc {
namespace {

// Rounds in flight at most.  A round holds its slot from launch until the
// scheduler sees its download done (upload, kernels, download and the retire
// poll: a few hundred microseconds even for small requests), so under a steady
// stream of small requests the slot count bounds the rounds per second.
constexpr int kSlots = 16;
constexpr int kMaxRoundRequests = 256;    // requests per round at most
constexpr size_t kAlign = 256;

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int fmt_dxt(unsigned int fmt) {
  switch (fmt) {
    case S2TC_GL_COMPRESSED_RGB_S3TC_DXT1_EXT:
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT1_EXT: return DXT1;
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT3_EXT: return DXT3;
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT5_EXT: return DXT5;
    default: return -1;
  }
}

s2tc_options norm(const s2tc_options& in) {
  s2tc_options o = in;
  if (o.dither != DI_NONE && o.dither != DI_FLOYDSTEINBERG) o.dither = DI_SIMPLE;
  if (o.metric < 0 || o.metric > 7) o.metric = CD_WAVG;
  if (o.refine != RF_NEVER && o.refine != RF_LOOP) o.refine = RF_ALWAYS;
  return o;
}

// First-fit allocator over [0, size) (offsets, kAlign granularity).
class Pool {
 public:
  explicit Pool(size_t size) : size_(size) { free_[0] = size; }
  bool alloc(size_t n, size_t* off) {
    n = align_up(std::max<size_t>(n, 1), kAlign);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        *off = it->first;
        const size_t rest = it->second - n;
        const size_t start = it->first + n;
        free_.erase(it);
        if (rest) free_[start] = rest;
        used_ += n;
        high_ = std::max(high_, used_);
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t n) {
    n = align_up(std::max<size_t>(n, 1), kAlign);
    used_ -= n;
    auto it = free_.emplace(off, n).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t high_water() const { return high_; }

 private:
  size_t size_, used_ = 0, high_ = 0;
  std::map<size_t, size_t> free_;
};

struct Req {
  long long id = 0;
  const uint8_t* hsrc = nullptr;
  int w = 0, h = 0, sc = 4, dxt = 0;
  s2tc_options opt{};
  uint8_t* hdst = nullptr;
  long long dpitch = 0;
  bool device_io = false;      // hsrc / hdst are device pointers: no copies, no pool space
  long long npx = 0, bw = 0, bh = 0;
  size_t in_bytes = 0, tex_bytes = 0, out_bytes = 0, rand_bytes = 0, total = 0;
  std::vector<unsigned> rand;  // replayed rand() words (random-candidate mode, host loop)
  RandWindow win{};            // or the stream position they start at (device generator)
  bool dev_rand = false;
  size_t off = 0;              // pool allocation
  double t_submit = 0, t_done = 0;
  int status = 1;              // 1 pending, 0 done, < 0 error
  int round = -1;
};

struct Slot {
  bool busy = false;
  cudaStream_t compute = nullptr;
  cudaEvent_t uploaded = nullptr, computed = nullptr, done = nullptr;
  unsigned char* htab = nullptr;  // pinned table staging
  unsigned char* dtab = nullptr;  // device tables
  size_t tab_bytes = 0;
  unsigned char* scratch = nullptr;  // dither scratch of the round
  size_t scratch_bytes = 0;
  int* d_err = nullptr;              // the round's bounded-wait flag
  int* h_err = nullptr;              // pinned copy, valid once `done` fired
  std::vector<std::shared_ptr<Req>> reqs;
};

}  // namespace
}  // namespace s2tc

struct s2tc_server {
  std::mutex m;
  std::condition_variable cv_submit, cv_done;
  std::deque<std::shared_ptr<s2tc::Req>> waiting;
  std::unordered_map<long long, std::shared_ptr<s2tc::Req>> by_id;
  std::unique_ptr<s2tc::Pool> pool;
  unsigned char* base = nullptr;
  size_t budget = 0;
  s2tc::Slot slots[s2tc::kSlots];
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  int* d_err = nullptr;  // kSlots flags, one per slot
  int* h_err = nullptr;
  std::thread worker;
  bool stop = false;
  long long next_id = 1;
  int device = 0;
  // statistics
  long long rounds = 0, done = 0;
  int max_inflight = 0, max_round = 0;
};

namespace s2tc {
namespace {

// Launch one round in `sl` (tables staged in sl.htab).  Returns a status.
int launch_round(s2tc_server* sv, Slot& sl) {
  std::vector<std::shared_ptr<Req>>& rs = sl.reqs;
  cudaStream_t s = sl.compute;
  unsigned char* base = sv->base;
  // The round's tables are laid out first, and their size checked, before any
  // copy that reads a client's host buffer is enqueued.

  // group requests by knobs (the kernels take uniform knobs per launch)
  std::map<std::tuple<int, int, int, int>, std::vector<Req*>> groups;
  for (auto& r : rs) groups[{r->opt.dither, r->opt.metric, r->opt.nrandom, r->opt.refine}].push_back(r.get());
  // tables: per group DitherItem[n], tile offsets[n]; per group and format
  // EncodeArgs[k], block offsets[k]
  size_t toff = 0, soff = 0;
  const long long tile_tex = dither_tile_texels();
  std::vector<std::pair<size_t, size_t>> copies;  // (offset, bytes) of table pieces
  auto put = [&](const void* p, size_t n) {
    const size_t o = toff;
    std::memcpy(sl.htab + o, p, n);
    toff = align_up(toff + n, 16);
    return o;
  };
  struct Launch {
    int dither, metric, nrandom, refine;
    DitherWork dw;
    std::vector<DitherArgs> fs;
    std::vector<size_t> fs_scratch;
    EncodeWork ew[3];
    bool has[3];
  };
  std::vector<Launch> launches;
  for (auto& g : groups) {
    const std::vector<Req*>& v = g.second;
    Launch L{};
    std::tie(L.dither, L.metric, L.nrandom, L.refine) = g.first;
    const int n = int(v.size());
    std::vector<DitherItem> di(n);
    std::vector<long long> to(n);
    long long tiles = 0;
    std::vector<EncodeArgs> ea[3];
    std::vector<long long> eo[3];
    long long et[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
      Req* r = v[i];
      unsigned char* p = base + r->off;
      const uint8_t* din = r->device_io ? r->hsrc : p;
      uint32_t* tex = reinterpret_cast<uint32_t*>(p + align_up(r->in_bytes, kAlign));
      uint8_t* pout = p + align_up(r->in_bytes, kAlign) + align_up(r->tex_bytes, kAlign);
      uint8_t* dout = r->device_io ? r->hdst : pout;
      const unsigned* drand = reinterpret_cast<const unsigned*>(pout + align_up(r->out_bytes, kAlign));
      di[i] = DitherItem{din, r->w, r->h, r->sc, r->dxt == DXT1 ? 1 : r->dxt == DXT3 ? 4 : 8, tex};
      to[i] = tiles;
      tiles += (r->npx + tile_tex - 1) / tile_tex;
      EncodeArgs a{};
      a.t565 = tex;
      a.width = r->w;
      a.height = r->h;
      a.bw = int(r->bw);
      a.bh = int(r->bh);
      a.by0 = 0;
      a.nby = int(r->bh);
      a.dst = dout;
      const int bsz = r->dxt == DXT1 ? 8 : 16;
      a.pitch = r->device_io ? r->dpitch : r->bw * bsz;
      a.aligned = ((reinterpret_cast<uintptr_t>(dout) % bsz) == 0 && (a.pitch % bsz) == 0) ? 1 : 0;
      a.nrandom = r->opt.nrandom;
      a.rnd = r->rand_bytes ? drand : nullptr;
      a.prev_a1_first = -1;
      a.leftover_out = nullptr;
      eo[r->dxt].push_back(et[r->dxt]);
      et[r->dxt] += r->bw * r->bh;
      ea[r->dxt].push_back(a);
      if (L.dither == DI_FLOYDSTEINBERG) {
        DitherArgs da{};
        da.src = din;
        da.width = r->w;
        da.height = r->h;
        da.srccomps = r->sc;
        da.alphabits = di[i].alphabits;
        da.dst = tex;
        da.error = sl.d_err;
        L.fs.push_back(da);
        L.fs_scratch.push_back(soff);
        soff = align_up(soff + dither_fs_scratch_bytes(r->w, r->h), kAlign);
      }
    }
    if (L.dither != DI_FLOYDSTEINBERG) {
      const size_t o_di = put(di.data(), sizeof(DitherItem) * n);
      const size_t o_to = put(to.data(), sizeof(long long) * n);
      L.dw.items = reinterpret_cast<const DitherItem*>(sl.dtab + o_di);
      L.dw.tile_offsets = reinterpret_cast<const long long*>(sl.dtab + o_to);
      L.dw.nitems = n;
      L.dw.total_tiles = tiles;
      L.dw.error = sl.d_err;
      // scratch of this group's scan
      L.fs_scratch.push_back(soff);
      soff = align_up(soff + dither_batch_scratch_bytes(tiles), kAlign);
    }
    for (int d = 0; d < 3; ++d) {
      L.has[d] = !ea[d].empty();
      if (!L.has[d]) continue;
      const size_t o_ea = put(ea[d].data(), sizeof(EncodeArgs) * ea[d].size());
      const size_t o_eo = put(eo[d].data(), sizeof(long long) * eo[d].size());
      L.ew[d] = EncodeWork{};
      L.ew[d].items = reinterpret_cast<const EncodeArgs*>(sl.dtab + o_ea);
      L.ew[d].offsets = reinterpret_cast<const long long*>(sl.dtab + o_eo);
      L.ew[d].nitems = int(ea[d].size());
      L.ew[d].total = et[d];
      L.ew[d].nrandom = L.nrandom;
    }
    launches.push_back(std::move(L));
  }
  // rand() stream positions of the requests whose words the device generates
  std::vector<std::pair<size_t, Req*>> gens;
  for (auto& r : rs)
    if (r->dev_rand) gens.emplace_back(put(&r->win, sizeof(RandWindow)), r.get());
  if (toff > sl.tab_bytes || soff > sl.scratch_bytes) return S2TC_ERR_TOO_LARGE;
  if (cudaMemsetAsync(sl.d_err, 0, sizeof(int), s) != cudaSuccess) return S2TC_ERR_CUDA;
  // uploads
  for (auto& r : rs) {
    if (!r->device_io &&
        cudaMemcpyAsync(base + r->off, r->hsrc, r->in_bytes, cudaMemcpyHostToDevice, sv->copy_in) != cudaSuccess)
      return S2TC_ERR_CUDA;
    if (r->rand_bytes && !r->dev_rand &&
        cudaMemcpyAsync(base + r->off + align_up(r->in_bytes, kAlign) + align_up(r->tex_bytes, kAlign) +
                            align_up(r->out_bytes, kAlign),
                        r->rand.data(), r->rand_bytes, cudaMemcpyHostToDevice, sv->copy_in) != cudaSuccess)
      return S2TC_ERR_CUDA;
  }
  if (cudaEventRecord(sl.uploaded, sv->copy_in) != cudaSuccess) return S2TC_ERR_CUDA;
  if (cudaStreamWaitEvent(s, sl.uploaded, 0) != cudaSuccess) return S2TC_ERR_CUDA;
  if (toff && cudaMemcpyAsync(sl.dtab, sl.htab, toff, cudaMemcpyHostToDevice, s) != cudaSuccess) return S2TC_ERR_CUDA;
  for (auto& g : gens) {
    Req* r = g.second;
    uint32_t* drand = reinterpret_cast<uint32_t*>(base + r->off + align_up(r->in_bytes, kAlign) +
                                                  align_up(r->tex_bytes, kAlign) + align_up(r->out_bytes, kAlign));
    if (rand_fill(reinterpret_cast<const RandWindow*>(sl.dtab + g.first), drand, (long long)(r->rand_bytes / 4), s) !=
        cudaSuccess)
      return S2TC_ERR_CUDA;
  }
  for (Launch& L : launches) {
    if (L.dither == DI_FLOYDSTEINBERG) {
      for (size_t i = 0; i < L.fs.size(); ++i)
        if (launch_dither(L.fs[i], DI_FLOYDSTEINBERG, sl.scratch + L.fs_scratch[i], s) != cudaSuccess)
          return S2TC_ERR_CUDA;
    } else if (launch_dither_batch(L.dw, L.dither, sl.scratch + L.fs_scratch[0], s) != cudaSuccess) {
      return S2TC_ERR_CUDA;
    }
    const bool normal = L.nrandom >= 0 || L.metric == CD_NORMALMAP;
    for (int d = 0; d < 3; ++d)
      if (L.has[d] && launch_encode(L.ew[d], d, L.metric, normal, L.refine, s) != cudaSuccess) return S2TC_ERR_CUDA;
  }
  if (cudaEventRecord(sl.computed, s) != cudaSuccess) return S2TC_ERR_CUDA;
  if (cudaStreamWaitEvent(sv->copy_out, sl.computed, 0) != cudaSuccess) return S2TC_ERR_CUDA;
  if (cudaMemcpyAsync(sl.h_err, sl.d_err, sizeof(int), cudaMemcpyDeviceToHost, sv->copy_out) != cudaSuccess)
    return S2TC_ERR_CUDA;
  for (auto& r : rs) {
    if (r->device_io) continue;  // the encoder wrote the caller's device buffer
    const size_t row = size_t(r->bw) * (r->dxt == DXT1 ? 8 : 16);
    const uint8_t* dout = base + r->off + align_up(r->in_bytes, kAlign) + align_up(r->tex_bytes, kAlign);
    if (cudaMemcpy2DAsync(r->hdst, size_t(r->dpitch), dout, row, row, size_t(r->bh), cudaMemcpyDeviceToHost,
                          sv->copy_out) != cudaSuccess)
      return S2TC_ERR_CUDA;
  }
  if (cudaEventRecord(sl.done, sv->copy_out) != cudaSuccess) return S2TC_ERR_CUDA;
  return S2TC_OK;
}

void scheduler(s2tc_server* sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->m);
  for (;;) {
    // retire finished rounds
    int inflight = 0;
    for (Slot& sl : sv->slots) {
      if (!sl.busy) continue;
      const cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) {
        ++inflight;
        continue;
      }
      const double t = now_ms();
      const int flag = q == cudaSuccess ? *sl.h_err : 0;
      for (auto& r : sl.reqs) {
        r->t_done = t;
        r->status = q == cudaSuccess ? (flag ? -S2TC_ERR_TIMEOUT : 0) : -S2TC_ERR_CUDA;
        sv->pool->release(r->off, r->total);
        ++sv->done;
      }
      sl.reqs.clear();
      sl.busy = false;
      sv->cv_done.notify_all();
    }
    // admit and launch a round
    Slot* free_slot = nullptr;
    for (Slot& sl : sv->slots)
      if (!sl.busy) {
        free_slot = &sl;
        break;
      }
    if (free_slot && !sv->waiting.empty()) {
      std::vector<std::shared_ptr<Req>> take;
      while (!sv->waiting.empty() && int(take.size()) < kMaxRoundRequests) {
        auto& r = sv->waiting.front();
        size_t off;
        if (!sv->pool->alloc(r->total, &off)) break;  // arrival order: wait for memory
        r->off = off;
        r->round = int(sv->rounds);
        take.push_back(r);
        sv->waiting.pop_front();
      }
      if (!take.empty()) {
        free_slot->reqs = std::move(take);
        free_slot->busy = true;
        sv->max_round = std::max(sv->max_round, int(free_slot->reqs.size()));
        ++sv->rounds;
        // the round's requests and slot belong to the scheduler now: submitters
        // need not wait while its stream operations are issued
        lk.unlock();
        const int st = launch_round(sv, *free_slot);
        if (st != S2TC_OK) {
          // copies of this round may already be in flight (they read the
          // clients' host buffers and write the pool or the clients' outputs):
          // let them finish before the memory is released and the requests
          // are reported done
          cudaStreamSynchronize(sv->copy_in);
          cudaStreamSynchronize(free_slot->compute);
          cudaStreamSynchronize(sv->copy_out);
        }
        lk.lock();
        if (st != S2TC_OK) {
          for (auto& r : free_slot->reqs) {
            r->status = -st;
            r->t_done = now_ms();
            sv->pool->release(r->off, r->total);
            ++sv->done;
          }
          free_slot->reqs.clear();
          free_slot->busy = false;
          sv->cv_done.notify_all();
        } else {
          ++inflight;
        }
        sv->max_inflight = std::max(sv->max_inflight, inflight);
        continue;
      }
    }
    if (sv->stop && sv->waiting.empty() && inflight == 0) break;
    if (inflight > 0) {
      // poll the GPU; new arrivals wake us too
      sv->cv_submit.wait_for(lk, std::chrono::microseconds(20));
    } else {
      sv->cv_submit.wait(lk, [&] { return sv->stop || !sv->waiting.empty(); });
    }
  }
}

}  // namespace
}  // namespace s2tc

extern "C" {

int s2tc_server_create(s2tc_server** out, long long budget_bytes) {
  if (!out || budget_bytes <= 0) return S2TC_ERR_ARGUMENT;
  *out = nullptr;
  auto* sv = new s2tc_server();
  sv->budget = size_t(budget_bytes);
  cudaGetDevice(&sv->device);
  bool ok = cudaMalloc(reinterpret_cast<void**>(&sv->base), sv->budget) == cudaSuccess &&
            cudaMalloc(reinterpret_cast<void**>(&sv->d_err), 256) == cudaSuccess &&
            cudaMemset(sv->d_err, 0, 256) == cudaSuccess &&
            cudaMallocHost(reinterpret_cast<void**>(&sv->h_err), 256) == cudaSuccess &&
            cudaStreamCreateWithFlags(&sv->copy_in, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&sv->copy_out, cudaStreamNonBlocking) == cudaSuccess;
  // per-slot tables and scan scratch (outside the request budget)
  const size_t tab = size_t(s2tc::kMaxRoundRequests) *
                     (4 * (sizeof(s2tc::EncodeArgs) + sizeof(s2tc::DitherItem) + 64) + sizeof(s2tc::RandWindow) + 16);
  const size_t scratch = size_t(64) << 20;
  for (int k = 0; k < s2tc::kSlots && ok; ++k) {
    s2tc::Slot& sl = sv->slots[k];
    sl.d_err = sv->d_err + k;
    sl.h_err = sv->h_err + k;
    *sl.h_err = 0;
    sl.tab_bytes = tab;
    sl.scratch_bytes = scratch;
    ok = cudaStreamCreateWithFlags(&sl.compute, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&sl.uploaded, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&sl.computed, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) == cudaSuccess &&
         cudaMallocHost(reinterpret_cast<void**>(&sl.htab), tab) == cudaSuccess &&
         cudaMalloc(reinterpret_cast<void**>(&sl.dtab), tab) == cudaSuccess &&
         cudaMalloc(reinterpret_cast<void**>(&sl.scratch), scratch) == cudaSuccess;
  }
  if (!ok) {
    std::fprintf(stderr, "s2tc_gb300: s2tc_server_create: %s\n", cudaGetErrorString(cudaGetLastError()));
    s2tc_server_destroy(sv);
    return S2TC_ERR_NOMEM;
  }
  sv->pool.reset(new s2tc::Pool(sv->budget));
  sv->worker = std::thread(s2tc::scheduler, sv);
  *out = sv;
  return S2TC_OK;
}

static int server_submit(s2tc_server* sv, const void* src, int srccomps, int width, int height, unsigned int format,
                         const s2tc_options* opt, void* dst, long long dst_pitch, long long* id, bool device_io) {
  using namespace s2tc;
  if (!sv || !src || !dst || !opt || !id || width <= 0 || height <= 0) return S2TC_ERR_ARGUMENT;
  const int dxt = fmt_dxt(format);
  if (dxt < 0) return S2TC_ERR_FORMAT;
  auto r = std::make_shared<Req>();
  r->hsrc = static_cast<const uint8_t*>(src);
  r->w = width;
  r->h = height;
  r->sc = srccomps == 3 ? 3 : 4;
  r->dxt = dxt;
  r->opt = norm(*opt);
  r->hdst = static_cast<uint8_t*>(dst);
  r->npx = (long long)width * height;
  r->bw = (width + 3) / 4;
  r->bh = (height + 3) / 4;
  const long long row = r->bw * (dxt == s2tc::DXT1 ? 8 : 16);
  r->dpitch = dst_pitch > 0 ? dst_pitch : row;
  if (r->dpitch < row) return S2TC_ERR_ARGUMENT;
  r->device_io = device_io;
  r->in_bytes = device_io ? 0 : size_t(r->npx) * r->sc;
  r->tex_bytes = size_t(r->npx) * 4;
  r->out_bytes = device_io ? 0 : size_t(row) * r->bh;
  const bool normal = r->opt.nrandom >= 0 || r->opt.metric == CD_NORMALMAP;
  if (normal && r->opt.nrandom > 0) {
    // libc rand() drawn now, in submission order, as tx_compress_dxtn would
    const size_t words = size_t(r->bw * r->bh) * r->opt.nrandom * (dxt == s2tc::DXT5 ? 4 : 3);
    if ((long long)words >= kRandDeviceMin && rand_usable() && rand_prepare() == cudaSuccess &&
        rand_take((long long)words, &r->win)) {
      r->dev_rand = true;  // generated on the device when its round launches
    } else {
      r->rand.resize(words);
      for (size_t i = 0; i < words; ++i) r->rand[i] = unsigned(std::rand());
    }
    r->rand_bytes = words * 4;
  }
  r->total = align_up(r->in_bytes, kAlign) + align_up(r->tex_bytes, kAlign) + align_up(r->out_bytes, kAlign) +
             align_up(r->rand_bytes, kAlign);
  if (r->total > sv->budget) return S2TC_ERR_TOO_LARGE;
  std::lock_guard<std::mutex> lk(sv->m);
  r->id = sv->next_id++;
  r->t_submit = now_ms();
  sv->by_id[r->id] = r;
  sv->waiting.push_back(r);
  *id = r->id;
  sv->cv_submit.notify_one();
  return S2TC_OK;
}

int s2tc_server_submit(s2tc_server* sv, const void* src, int srccomps, int width, int height, unsigned int format,
                       const s2tc_options* opt, void* dst, long long dst_pitch, long long* id) {
  return server_submit(sv, src, srccomps, width, height, format, opt, dst, dst_pitch, id, false);
}

int s2tc_server_submit_device(s2tc_server* sv, const void* d_src, int srccomps, int width, int height,
                              unsigned int format, const s2tc_options* opt, void* d_dst, long long dst_pitch,
                              long long* id) {
  return server_submit(sv, d_src, srccomps, width, height, format, opt, d_dst, dst_pitch, id, true);
}

int s2tc_server_wait(s2tc_server* sv, long long id, double* latency_ms) {
  if (!sv) return S2TC_ERR_ARGUMENT;
  std::unique_lock<std::mutex> lk(sv->m);
  auto it = sv->by_id.find(id);
  if (it == sv->by_id.end()) return S2TC_ERR_ARGUMENT;
  std::shared_ptr<s2tc::Req> r = it->second;
  sv->cv_done.wait(lk, [&] { return r->status != 1; });
  if (latency_ms) *latency_ms = r->t_done - r->t_submit;
  sv->by_id.erase(it);
  return r->status < 0 ? -r->status : S2TC_OK;
}

int s2tc_server_stats(s2tc_server* sv, long long* rounds, long long* done, int* max_inflight_rounds,
                      int* max_round_requests, long long* pool_high_water) {
  if (!sv) return S2TC_ERR_ARGUMENT;
  std::lock_guard<std::mutex> lk(sv->m);
  if (rounds) *rounds = sv->rounds;
  if (done) *done = sv->done;
  if (max_inflight_rounds) *max_inflight_rounds = sv->max_inflight;
  if (max_round_requests) *max_round_requests = sv->max_round;
  if (pool_high_water) *pool_high_water = sv->pool ? (long long)sv->pool->high_water() : 0;
  return S2TC_OK;
}

void s2tc_server_destroy(s2tc_server* sv) {
  if (!sv) return;
  if (sv->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lk(sv->m);
      sv->stop = true;
    }
    sv->cv_submit.notify_all();
    sv->worker.join();
  }
  for (auto& sl : sv->slots) {
    if (sl.compute) cudaStreamDestroy(sl.compute);
    if (sl.uploaded) cudaEventDestroy(sl.uploaded);
    if (sl.computed) cudaEventDestroy(sl.computed);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.htab) cudaFreeHost(sl.htab);
    if (sl.dtab) cudaFree(sl.dtab);
    if (sl.scratch) cudaFree(sl.scratch);
  }
  if (sv->copy_in) cudaStreamDestroy(sv->copy_in);
  if (sv->copy_out) cudaStreamDestroy(sv->copy_out);
  if (sv->base) cudaFree(sv->base);
  if (sv->d_err) cudaFree(sv->d_err);
  if (sv->h_err) cudaFreeHost(sv->h_err);
  delete sv;
}

}  // extern "C"
