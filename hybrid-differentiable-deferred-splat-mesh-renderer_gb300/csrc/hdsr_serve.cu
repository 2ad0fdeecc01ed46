// hdsr_serve.cu — the serving loop (hdsr_server_*): resident scenes,
// per-(scene, viewport, colour format) compositor slots inside an HBM budget,
// one stream per slot, CUDA graphs for the kernels before the rasteriser.
//
// No reference counterpart; the per-scene, per-frame analogue is
// splatRenderer.ts loadScene (:866-961) and renderFrame (:1024-1140).
//
// Threads: callers submit and wait; one dispatcher thread owns every CUDA
// call of the server; completions arrive through cudaLaunchHostFunc
// callbacks, which only timestamp and queue the slot (no CUDA calls). The
// mutex is never held across a CUDA call: slot creation and destruction can
// synchronise the device, which waits for those callbacks.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/hdsr.h"
#include "hdsr_internal.cuh"

using namespace hdsr;

// -DHDSR_SERVER_TRACE: one stderr line per scheduler event
#ifdef HDSR_SERVER_TRACE
#define TRACE(...) (std::fprintf(stderr, "[hdsr-server] " __VA_ARGS__), std::fputc('\n', stderr), std::fflush(stderr))
#else
#define TRACE(...) ((void)0)
#endif

namespace {

using Clock = std::chrono::steady_clock;

struct Scene {
  hdsr_scene_views views{};
  uint64_t bytes = 0;
};

struct Slot {
  uint32_t scene_id = 0, width = 0, height = 0, color_format = 0;
  hdsr_compositor* h = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  float* pinned_u = nullptr;       // uniform staging (64 floats)
  uint32_t* pinned_ctl = nullptr;  // control block readback (kCtlWords)
  uint64_t bytes = 0;
  uint64_t capacity = 0;
  uint64_t last_used = 0;
  uint64_t frames = 0;
  uint64_t ticket = 0;
  bool busy = false;
};

struct Ticket {
  hdsr_request req{};
  hdsr_request_result res{};
  cudaEvent_t ready = nullptr;  // legacy-stream work issued before submit
  bool done = false;
};

struct Key {
  uint32_t scene_id, width, height, color_format;
  bool operator<(const Key& o) const {
    return std::tie(scene_id, width, height, color_format) < std::tie(o.scene_id, o.width, o.height, o.color_format);
  }
};

}  // namespace

struct hdsr_server {
  hdsr_server_config cfg{};
  int device = 0;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, Ticket> tickets;
  std::map<uint32_t, Scene> scenes;
  std::vector<Slot*> slots;
  std::deque<Slot*> completions;
  std::map<Key, uint64_t> learned_pairs;  // largest P seen per key: sizes new slots
  std::map<Key, uint64_t> learned_bytes;  // device bytes of the last slot made for a key
  uint64_t next_ticket = 1;
  uint64_t use_clock = 0;
  uint64_t events = 0;     // bumped (under mu) by every completion and submission
  uint32_t in_flight = 0;
  uint64_t scene_bytes = 0, slot_bytes = 0;
  uint32_t graphs = 0, evictions = 0;
  uint64_t completed = 0, reruns = 0;
  bool stop = false;
  std::thread dispatcher;
  char err[256] = {0};
};

namespace {

double ms_since(const hdsr_server* s) {
  return std::chrono::duration<double, std::milli>(Clock::now() - s->t0).count();
}

hdsr_status server_fail(hdsr_server* s, hdsr_status st, const char* msg) {
  if (s) std::snprintf(s->err, sizeof(s->err), "%s", msg);
  return st;
}

uint64_t scene_device_bytes(const hdsr_scene_views& v) {
  const uint64_t K = ((uint64_t)v.sh_degree + 1) * (v.sh_degree + 1) - 1;
  return (uint64_t)v.splat_count * (12 + 12 + 16 + 4 + 4 + 4 + 4 * (6 + 3 * K)) + v.normals_len * 4;
}

struct DoneCtx {
  hdsr_server* server;
  Slot* slot;
};

void CUDART_CB on_frame_done(void* p) {
  DoneCtx* c = static_cast<DoneCtx*>(p);
  hdsr_server* s = c->server;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->tickets.find(c->slot->ticket);
    if (it != s->tickets.end()) it->second.res.done_ms = ms_since(s);
    s->completions.push_back(c->slot);
    ++s->events;
  }
  s->cv_work.notify_one();
  delete c;
}

void destroy_slot(Slot* sl) {
  TRACE("destroy slot %p", (void*)sl);
  if (sl->stream) cudaStreamSynchronize(sl->stream);
  if (sl->graph) cudaGraphExecDestroy(sl->graph);
  if (sl->h) hdsr_destroy_tile_splat_compositor(sl->h);
  if (sl->pinned_u) cudaFreeHost(sl->pinned_u);
  if (sl->pinned_ctl) cudaFreeHost(sl->pinned_ctl);
  if (sl->stream) cudaStreamDestroy(sl->stream);
  delete sl;
}

// New slot for a key (no lock held). nullptr with msg on failure.
Slot* create_slot(const Key& k, const hdsr_scene_views& scene, uint64_t capacity, char* msg, size_t msg_len) {
  hdsr_plan_input in{};
  in.viewport_width = k.width;
  in.viewport_height = k.height;
  in.tile_size_px = kTilePx;
  in.splat_count = scene.splat_count;
  hdsr_plan plan{};
  if (hdsr_plan_tile_splat_compositor(&in, &plan) != HDSR_OK) {
    std::snprintf(msg, msg_len, "viewport %ux%u cannot be planned", k.width, k.height);
    return nullptr;
  }
  hdsr_config cfg{};
  cfg.pair_capacity = capacity;
  cfg.color_format = k.color_format;
  Slot* sl = new Slot();
  sl->scene_id = k.scene_id;
  sl->width = k.width;
  sl->height = k.height;
  sl->color_format = k.color_format;
  hdsr_status st = hdsr_create_tile_splat_compositor(&plan, &cfg, &sl->h);
  if (st == HDSR_OK) st = hdsr_bind_scene(sl->h, &scene);
  if (st != HDSR_OK) {
    std::snprintf(msg, msg_len, "slot: %s", sl->h ? hdsr_last_error(sl->h) : "create failed");
    destroy_slot(sl);
    return nullptr;
  }
  if (cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMallocHost(&sl->pinned_u, 256) != cudaSuccess ||
      cudaMallocHost(&sl->pinned_ctl, kCtlWords * sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    std::snprintf(msg, msg_len, "slot: stream or pinned staging could not be created");
    destroy_slot(sl);
    return nullptr;
  }
  sl->bytes = handle_device_bytes(sl->h);
  sl->capacity = handle_args(sl->h)->cap;
  TRACE("create slot %p scene %u %ux%u fmt %u bytes %llu cap %llu", (void*)sl, k.scene_id, k.width, k.height,
        k.color_format, (unsigned long long)sl->bytes, (unsigned long long)sl->capacity);
  return sl;
}

// Queues one frame of `t` on `sl` (no lock held). Returns a status; on
// success a completion callback will arrive.
hdsr_status launch_frame(hdsr_server* s, Slot* sl, Ticket& t) {
  hdsr_compositor* h = sl->h;
  hdsr_status st = hdsr_bind_outputs(h, &t.req.outputs);
  if (st == HDSR_OK) st = hdsr_set_frame_uniforms(h, t.req.uniforms);
  if (st == HDSR_OK) st = (hdsr_status)handle_frame_checks(h);
  if (st != HDSR_OK) {
    server_fail(s, st, hdsr_last_error(h));
    return st;
  }
  // the request's outputs (and anything else the caller queued on the legacy
  // stream before submit) are ready first
  if (t.ready && cudaStreamWaitEvent(sl->stream, t.ready, 0) != cudaSuccess) {
    cudaGetLastError();
    return server_fail(s, HDSR_ERR_CUDA, "wait for the request's inputs");
  }
  std::memcpy(sl->pinned_u, t.req.uniforms, 256);
  st = (hdsr_status)handle_upload_uniforms(h, sl->pinned_u, sl->stream);
  const bool use_graph = !(s->cfg.flags & HDSR_SERVER_NO_GRAPH);
  if (st == HDSR_OK) {
    if (sl->graph) {
      if (cudaGraphLaunch(sl->graph, sl->stream) != cudaSuccess) st = HDSR_ERR_CUDA;
    } else if (use_graph && sl->frames > 0) {
      // the slot's kernels are warm (their launch attributes set): capture
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(sl->stream, cudaStreamCaptureModeThreadLocal);
      hdsr_status cs = e == cudaSuccess ? (hdsr_status)handle_encode_pre_raster(h, sl->stream) : HDSR_ERR_CUDA;
      cudaError_t e2 = cudaStreamEndCapture(sl->stream, &g);
      if (e == cudaSuccess && cs == HDSR_OK && e2 == cudaSuccess && g &&
          cudaGraphInstantiate(&sl->graph, g, 0) == cudaSuccess) {
        std::lock_guard<std::mutex> lock(s->mu);
        ++s->graphs;
      } else {
        sl->graph = nullptr;
      }
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      if (sl->graph) {
        if (cudaGraphLaunch(sl->graph, sl->stream) != cudaSuccess) st = HDSR_ERR_CUDA;
      } else {
        st = (hdsr_status)handle_encode_pre_raster(h, sl->stream);
      }
    } else {
      st = (hdsr_status)handle_encode_pre_raster(h, sl->stream);
    }
  }
  if (st == HDSR_OK) st = (hdsr_status)handle_encode_raster(h, sl->stream);
  if (st == HDSR_OK &&
      cudaMemcpyAsync(sl->pinned_ctl, handle_args(h)->ctl, kCtlWords * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                      sl->stream) != cudaSuccess)
    st = HDSR_ERR_CUDA;
  if (st == HDSR_OK) {
    DoneCtx* c = new DoneCtx{s, sl};
    if (cudaLaunchHostFunc(sl->stream, on_frame_done, c) != cudaSuccess) {
      delete c;
      st = HDSR_ERR_CUDA;
    }
  }
  if (st != HDSR_OK) {
    TRACE("launch failed slot %p status %d cuda %s", (void*)sl, (int)st, cudaGetErrorString(cudaGetLastError()));
    server_fail(s, st, "frame launch failed");
  }
  TRACE("launched slot %p ticket %llu graph %d status %d", (void*)sl, (unsigned long long)sl->ticket,
        sl->graph != nullptr, (int)st);
  return st;
}

void finish_ticket(hdsr_server* s, Ticket& t, hdsr_status st) {
  if (t.ready) {
    cudaEventDestroy(t.ready);  // does not block: a pending event is released when it completes
    t.ready = nullptr;
  }
  t.res.status = st;
  t.done = true;
  if (t.res.done_ms == 0.0) t.res.done_ms = ms_since(s);
  ++s->completed;
}

void dispatcher_main(hdsr_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lock(s->mu);
  for (;;) {
    if (s->stop) break;
    // events seen by this pass: one that arrives while the lock is released
    // below (CUDA calls) still wakes the wait at the end
    const uint64_t seen = s->events;
    bool progress = false;
    // 1. completions: status, overflow re-runs, slot back to idle
    while (!s->completions.empty()) {
      Slot* sl = s->completions.front();
      s->completions.pop_front();
      progress = true;
      auto it = s->tickets.find(sl->ticket);
      const uint32_t flags = sl->pinned_ctl[kCtlFlags];
      const uint64_t pairs = (uint64_t)sl->pinned_ctl[kCtlPairsLo] | ((uint64_t)sl->pinned_ctl[kCtlPairsHi] << 32);
      ++sl->frames;
      --s->in_flight;
      if (it == s->tickets.end()) {
        sl->busy = false;
        continue;
      }
      Ticket& t = it->second;
      t.res.total_pairs = pairs;
      TRACE("done slot %p ticket %llu flags %u pairs %llu in_flight %u", (void*)sl, (unsigned long long)sl->ticket,
            flags, (unsigned long long)pairs, s->in_flight);
      const Key key{sl->scene_id, sl->width, sl->height, sl->color_format};
      uint64_t& learned = s->learned_pairs[key];
      learned = std::max(learned, pairs);
      if ((flags & HDSR_DEV_OVERFLOW) && t.res.reruns == 0) {
        // re-run on this slot, recreated with room for this frame
        ++t.res.reruns;
        ++s->reruns;
        const uint64_t old_bytes = sl->bytes;
        const Scene scene = s->scenes[sl->scene_id];
        lock.unlock();
        if (sl->graph) {
          cudaGraphExecDestroy(sl->graph);
          sl->graph = nullptr;
        }
        hdsr_destroy_tile_splat_compositor(sl->h);
        sl->h = nullptr;
        char msg[160];
        Slot* fresh = create_slot(key, scene.views, pairs + pairs / 4 + 65536, msg, sizeof(msg));
        hdsr_status st = HDSR_ERR_OOM;
        if (fresh) {
          // keep the slot object (its stream and staging); take the new handle
          std::swap(sl->h, fresh->h);
          sl->bytes = handle_device_bytes(sl->h);
          sl->capacity = handle_args(sl->h)->cap;
          sl->frames = 0;
          destroy_slot(fresh);
          st = launch_frame(s, sl, t);
        }
        lock.lock();
        s->slot_bytes = s->slot_bytes - old_bytes + (sl->h ? sl->bytes : 0);
        if (st == HDSR_OK) {
          ++s->in_flight;
        } else {
          if (!fresh) server_fail(s, st, msg);
          finish_ticket(s, t, st);
          sl->busy = false;
          s->cv_done.notify_all();
        }
        continue;
      }
      hdsr_status st = HDSR_OK;
      if (flags & HDSR_DEV_OVERFLOW) st = HDSR_ERR_OVERFLOW;
      else if (flags & HDSR_DEV_TIMEOUT) st = HDSR_ERR_TIMEOUT;
      else if (flags & (HDSR_DEV_COUNT_MISMATCH | HDSR_DEV_BAD_ENTRY)) st = HDSR_ERR_CUDA;
      finish_ticket(s, t, st);
      sl->busy = false;
      sl->last_used = ++s->use_clock;
      s->cv_done.notify_all();
    }
    // 2. dispatch queued requests onto idle (or new) slots, in order, without
    //    letting one key's wait block the others. Only ticket ids are held
    //    across the unlocked stretches (submit() may grow the queue there).
    std::vector<uint64_t> blocked;  // tickets that cannot be placed in this pass
    auto dequeue = [s](uint64_t id) {
      auto q = std::find(s->queue.begin(), s->queue.end(), id);
      if (q != s->queue.end()) s->queue.erase(q);
    };
    while (s->in_flight < s->cfg.max_in_flight) {
      uint64_t id = 0;
      for (uint64_t q : s->queue)
        if (std::find(blocked.begin(), blocked.end(), q) == blocked.end()) {
          id = q;
          break;
        }
      if (id == 0) break;
      Ticket& t = s->tickets[id];
      const uint32_t W = (uint32_t)t.req.uniforms[16], H = (uint32_t)t.req.uniforms[17];
      const Key key{t.req.scene_id, W, H, t.req.color_format};
      Slot* sl = nullptr;
      for (Slot* c : s->slots)
        if (!c->busy && c->scene_id == key.scene_id && c->width == W && c->height == H &&
            c->color_format == key.color_format) {
          sl = c;
          break;
        }
      if (!sl) {
        // a slot of known size that cannot fit even with every idle slot
        // evicted: wait for running frames instead of building it
        if (s->learned_bytes.count(key) && s->in_flight > 0) {
          uint64_t idle_bytes = 0;
          for (Slot* c : s->slots)
            if (!c->busy) idle_bytes += c->bytes;
          if (s->scene_bytes + s->slot_bytes - idle_bytes + s->learned_bytes[key] > s->cfg.hbm_budget_bytes) {
            blocked.push_back(id);
            continue;
          }
        }
        // a new slot, inside the budget: evict idle slots, least recently used first
        const Scene scene = s->scenes[key.scene_id];
        const uint64_t learned = s->learned_pairs.count(key) ? s->learned_pairs[key] : 0;
        lock.unlock();
        char msg[160];
        // headroom over the largest frame seen: another camera of the same
        // key rarely needs more, and a re-run rebuilds the slot
        Slot* fresh = create_slot(key, scene.views, learned ? learned + learned / 2 + 65536 : 0, msg, sizeof(msg));
        lock.lock();
        if (!fresh) {
          finish_ticket(s, t, HDSR_ERR_OOM);
          server_fail(s, HDSR_ERR_OOM, msg);
          dequeue(id);
          s->cv_done.notify_all();
          progress = true;
          continue;
        }
        s->learned_bytes[key] = fresh->bytes;
        std::vector<Slot*> victims;
        uint64_t need = s->scene_bytes + s->slot_bytes + fresh->bytes;
        if (need > s->cfg.hbm_budget_bytes) {
          std::vector<Slot*> idle;
          for (Slot* c : s->slots)
            if (!c->busy) idle.push_back(c);
          std::sort(idle.begin(), idle.end(), [](Slot* a, Slot* b) { return a->last_used < b->last_used; });
          for (Slot* c : idle) {
            if (need <= s->cfg.hbm_budget_bytes) break;
            victims.push_back(c);
            need -= c->bytes;
          }
        }
        if (need > s->cfg.hbm_budget_bytes) {
          // cannot fit now: drop the new slot; wait for running frames, or
          // fail the request when nothing is running that could free room
          lock.unlock();
          destroy_slot(fresh);
          lock.lock();
          if (s->in_flight == 0) {
            finish_ticket(s, t, HDSR_ERR_OOM);
            server_fail(s, HDSR_ERR_OOM, "a slot for this request does not fit in the HBM budget");
            dequeue(id);
            s->cv_done.notify_all();
            progress = true;
          } else {
            TRACE("ticket %llu waits for room", (unsigned long long)id);
            blocked.push_back(id);
          }
          continue;
        }
        for (Slot* v : victims) {
          TRACE("evict slot %p", (void*)v);
          s->slots.erase(std::find(s->slots.begin(), s->slots.end(), v));
          s->slot_bytes -= v->bytes;
          ++s->evictions;
        }
        s->slots.push_back(fresh);
        s->slot_bytes += fresh->bytes;
        sl = fresh;
        if (!victims.empty()) {
          lock.unlock();
          for (Slot* v : victims) destroy_slot(v);
          lock.lock();
        }
      }
      sl->busy = true;
      sl->ticket = id;
      t.res.start_ms = ms_since(s);
      ++s->in_flight;
      dequeue(id);
      progress = true;
      lock.unlock();
      hdsr_status st = launch_frame(s, sl, t);
      lock.lock();
      if (st != HDSR_OK) {
        --s->in_flight;
        sl->busy = false;
        finish_ticket(s, t, st);
        s->cv_done.notify_all();
      }
    }
    if (!progress) s->cv_work.wait(lock, [s, seen] { return s->stop || s->events != seen; });
  }
}

}  // namespace

extern "C" {

hdsr_status hdsr_server_create(const hdsr_server_config* cfg, hdsr_server** out) {
  if (!cfg || !out) return HDSR_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->hbm_budget_bytes == 0 || cfg->max_in_flight == 0 || cfg->max_in_flight > 64) return HDSR_ERR_INVALID_ARG;
  hdsr_server* s = new (std::nothrow) hdsr_server();
  if (!s) return HDSR_ERR_OOM;
  s->cfg = *cfg;
  s->t0 = Clock::now();
  if (cudaGetDevice(&s->device) != cudaSuccess) {
    delete s;
    return HDSR_ERR_CUDA;
  }
  s->dispatcher = std::thread(dispatcher_main, s);
  *out = s;
  return HDSR_OK;
}

void hdsr_server_destroy(hdsr_server* s) {
  if (!s) return;
  {
    std::unique_lock<std::mutex> lock(s->mu);
    // let queued and running frames finish
    s->cv_done.wait(lock, [s] { return s->queue.empty() && s->in_flight == 0; });
    s->stop = true;
    ++s->events;
  }
  s->cv_work.notify_all();
  if (s->dispatcher.joinable()) s->dispatcher.join();
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(s->device);
  for (Slot* sl : s->slots) destroy_slot(sl);
  cudaSetDevice(prev);
  delete s;
}

hdsr_status hdsr_server_add_scene(hdsr_server* s, uint32_t scene_id, const hdsr_scene_views* scene) {
  if (!s) return HDSR_ERR_INVALID_ARG;
  if (!scene) return server_fail(s, HDSR_ERR_INVALID_ARG, "scene views are NULL");
  if (scene->sh_degree > 3) return server_fail(s, HDSR_ERR_INVALID_ARG, "sh_degree must be 0..3");
  if (scene->splat_count &&
      (!scene->positions || !scene->scales || !scene->rotations || !scene->opacities || !scene->material ||
       !scene->sh_data || !scene->sorted_indices))
    return server_fail(s, HDSR_ERR_INVALID_ARG, "a scene array is NULL");
  // the scene's arrays may still be written by work on the legacy stream
  if (cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess) {
    cudaGetLastError();
    return server_fail(s, HDSR_ERR_CUDA, "synchronize before registering the scene");
  }
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->scenes.count(scene_id)) return server_fail(s, HDSR_ERR_INVALID_ARG, "scene id already registered");
  const uint64_t b = scene_device_bytes(*scene);
  if (s->scene_bytes + s->slot_bytes + b > s->cfg.hbm_budget_bytes)
    return server_fail(s, HDSR_ERR_OOM, "the scene does not fit in the HBM budget");
  Scene sc;
  sc.views = *scene;
  sc.bytes = b;
  s->scenes[scene_id] = sc;
  s->scene_bytes += b;
  return HDSR_OK;
}

hdsr_status hdsr_server_submit(hdsr_server* s, const hdsr_request* req, uint64_t* ticket) {
  if (!s) return HDSR_ERR_INVALID_ARG;
  if (!req || !ticket) return server_fail(s, HDSR_ERR_INVALID_ARG, "request or ticket is NULL");
  if (req->color_format > HDSR_COLOR_RGBA32F) return server_fail(s, HDSR_ERR_INVALID_ARG, "unknown color format");
  const float W = req->uniforms[16], H = req->uniforms[17];
  if (!(W >= 1.0f && H >= 1.0f && W <= 4080.0f && H <= 4080.0f) || W != (float)(uint32_t)W ||
      H != (float)(uint32_t)H)
    return server_fail(s, HDSR_ERR_INVALID_ARG, "uniform viewport must be whole pixels in 1..4080");
  if (!req->outputs.color || !req->outputs.depth || !req->outputs.normal || !req->outputs.material)
    return server_fail(s, HDSR_ERR_INVALID_ARG, "an output image is NULL");
  cudaEvent_t ready = nullptr;
  if (cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventRecord(ready, cudaStreamLegacy) != cudaSuccess) {
    cudaGetLastError();
    if (ready) cudaEventDestroy(ready);
    return server_fail(s, HDSR_ERR_CUDA, "record the request's ready event");
  }
  std::lock_guard<std::mutex> lock(s->mu);
  auto sc = s->scenes.find(req->scene_id);
  if (sc == s->scenes.end()) {
    cudaEventDestroy(ready);
    return server_fail(s, HDSR_ERR_INVALID_ARG, "unknown scene id");
  }
  uint32_t n, deg;
  std::memcpy(&n, req->uniforms + 22, 4);
  std::memcpy(&deg, req->uniforms + 25, 4);
  if (n != sc->second.views.splat_count || deg != sc->second.views.sh_degree) {
    cudaEventDestroy(ready);
    return server_fail(s, HDSR_ERR_INVALID_ARG, "uniform splatCount / shDegree differ from the scene");
  }
  const uint64_t id = s->next_ticket++;
  Ticket& t = s->tickets[id];
  t.req = *req;
  t.ready = ready;
  t.res.submit_ms = ms_since(s);
  s->queue.push_back(id);
  ++s->events;
  *ticket = id;
  s->cv_work.notify_one();
  return HDSR_OK;
}

hdsr_status hdsr_server_wait(hdsr_server* s, uint64_t ticket, hdsr_request_result* result) {
  if (!s) return HDSR_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return server_fail(s, HDSR_ERR_INVALID_ARG, "unknown ticket");
  s->cv_done.wait(lock, [&] { return it->second.done; });
  if (result) *result = it->second.res;
  const hdsr_status st = (hdsr_status)it->second.res.status;
  s->tickets.erase(it);
  return st;
}

hdsr_status hdsr_server_query(hdsr_server* s, hdsr_server_stats* st) {
  if (!s || !st) return HDSR_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  std::memset(st, 0, sizeof(*st));
  st->budget_bytes = s->cfg.hbm_budget_bytes;
  st->scene_bytes = s->scene_bytes;
  st->slot_bytes = s->slot_bytes;
  st->scenes = (uint32_t)s->scenes.size();
  st->slots = (uint32_t)s->slots.size();
  st->graphs = s->graphs;
  st->evictions = s->evictions;
  st->completed = s->completed;
  st->reruns = s->reruns;
  return HDSR_OK;
}

const char* hdsr_server_last_error(const hdsr_server* s) { return s ? s->err : "null server"; }

}  // extern "C"
