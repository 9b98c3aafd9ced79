// C ABI of libfgrain_cuda.so: engine lifetime, presets, emulsion transfer and the stage entry
// points.  Every call takes the engine lock, runs on the engine's stream, waits for completion,
// reads the device error word and maps failures to fg_status (error.rs:9-33 for 1-6).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include "fg_internal.h"

namespace fg {
void replay_segments(fg_engine* e, fg_emulsion* em, const fg_exposure_cfg& cfg, uint64_t seed,
                     const fg_segment* segs_host, size_t nseg, uint32_t* offsets_host,
                     uint32_t* ids_host, size_t id_cap, size_t* nhits);
void replay_rays(fg_engine* e, const fg_emulsion* em, const double* org_host,
                 const double* dir_host, size_t nrays, int developed_only, uint32_t* offsets_host,
                 uint32_t* ids_host, size_t id_cap, size_t* nhits, double* chord_host);

void check_error_word(fg_engine* e) {
  uint32_t rec[ERR_WORDS] = {};
  FG_CUDA(cudaMemcpyAsync(rec, e->d_err, sizeof(rec), cudaMemcpyDeviceToHost, e->stream));
  FG_CUDA(cudaStreamSynchronize(e->stream));
  const uint32_t w = rec[0];
  e->timings.error_word = w;
  if (!w) return;
  FG_CUDA(cudaMemsetAsync(e->d_err, 0, sizeof(rec), e->stream));
  FG_CUDA(cudaStreamSynchronize(e->stream));
  std::string m = "device error word " + std::to_string(w) + ":";
  if (w & ERR_BAD_INDEX)
    m += " index check failed at site " + std::to_string(rec[1]) + " (values " + std::to_string(rec[2]) + ", " +
         std::to_string(rec[3]) + "), access skipped;";
  if (w & ERR_HIT_OVERFLOW) m += " hit list overflow;";
  if (w & ERR_STACK_OVERFLOW) m += " traversal stack overflow;";
  if (w & ERR_LIST_OVERFLOW) m += " work list overflow;";
  if (w & ERR_BAD_INPUT) m += " invalid input;";
  if (w & ERR_SPIN_LIMIT) throw Error{FG_ERR_DEVICE_TIMEOUT, m + " bounded wait gave up"};
  throw Error{FG_ERR_DEVICE_OVERFLOW, m};
}

// Starts a call: zeroes the per-call timings and device counters.
void begin_call(fg_engine* e) {
  e->timings = fg_timings{};
  FG_CUDA(cudaMemsetAsync(e->d_stats, 0, 8 * sizeof(unsigned long long), e->stream));
}

void end_call(fg_engine* e) {
  unsigned long long st[8];
  FG_CUDA(cudaMemcpyAsync(st, e->d_stats, sizeof(st), cudaMemcpyDeviceToHost, e->stream));
  FG_CUDA(cudaStreamSynchronize(e->stream));
  e->timings.hits += st[0] + st[2];
  e->timings.fallbacks += st[1];
  check_error_word(e);
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.0f;
  FG_CUDA(cudaEventElapsedTime(&ms, a, b));
  return ms;
}

template <class T>
void to_device(DBuf<T>& d, const T* h, size_t n, cudaStream_t st) {
  d.alloc(n, st);
  if (n) FG_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
}

void alloc_state(fg_emulsion* em, cudaStream_t st) {
  const uint32_t n = em->n;
  em->counts.alloc(std::max<uint32_t>(n, 1), st);
  em->developed.alloc(std::max<uint32_t>(n, 1), st);
  em->exp32.alloc(std::max<uint32_t>(n, 1), st);
  em->exp64.alloc(std::max<uint32_t>(n, 1), st);
  em->clump.alloc(std::max<uint32_t>(n, 1), st);
  FG_CUDA(cudaMemsetAsync(em->counts.p, 0, em->counts.n * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(em->developed.p, 0, em->developed.n, st));
  FG_CUDA(cudaMemsetAsync(em->exp32.p, 0, em->exp32.n * sizeof(float), st));
  FG_CUDA(cudaMemsetAsync(em->exp64.p, 0, em->exp64.n * sizeof(double), st));
  FG_CUDA(cudaMemsetAsync(em->clump.p, 0xff, em->clump.n * sizeof(int64_t), st));
}

}  // namespace fg

using namespace fg;

extern "C" {

const char* fg_status_string(fg_status s) {
  switch (s) {
    case FG_OK: return "ok";
    case FG_ERR_ADAPTER_NOT_FOUND: return "Failed to find suitable GPU adapter";
    case FG_ERR_DEVICE_REQUEST_FAILED: return "Failed to create device";
    case FG_ERR_CHANNEL: return "GPU channel error";
    case FG_ERR_BUFFER_MAP: return "GPU buffer map error";
    case FG_ERR_BUFFER_RANGE: return "GPU buffer range error";
    case FG_ERR_PIPELINE: return "GPU pipeline error";
    case FG_ERR_INVALID_ARG: return "invalid argument";
    case FG_ERR_OOM: return "out of device memory";
    case FG_ERR_DEVICE_TIMEOUT: return "device wait limit reached";
    case FG_ERR_DEVICE_OVERFLOW: return "device capacity exceeded";
  }
  return "unknown status";
}

fg_status fg_set_device_budget(uint64_t bytes) {
  fg::g_dev_budget.store(bytes);
  return FG_OK;
}

fg_status fg_engine_create(int device, fg_engine** out) {
  if (!out) return FG_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return FG_ERR_ADAPTER_NOT_FOUND;
  if (device < 0 || device >= count) return FG_ERR_ADAPTER_NOT_FOUND;
  fg_engine* e = new (std::nothrow) fg_engine();
  if (!e) return FG_ERR_OOM;
  e->device = device;
  try {
    FG_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    FG_CUDA(cudaGetDeviceProperties(&prop, device));
    e->name = prop.name;
    e->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess)
      throw Error{FG_ERR_DEVICE_REQUEST_FAILED, "stream creation failed"};
    cudaMemPool_t pool;
    FG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t thr = UINT64_MAX;
    FG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    FG_CUDA(cudaMalloc(&e->d_err, ERR_WORDS * sizeof(uint32_t)));
    FG_CUDA(cudaMalloc(&e->d_stats, 8 * sizeof(unsigned long long)));
    FG_CUDA(cudaMemset(e->d_err, 0, ERR_WORDS * sizeof(uint32_t)));
    FG_CUDA(cudaMemset(e->d_stats, 0, 8 * sizeof(unsigned long long)));
    e->timer.init();
  } catch (const Error& x) {
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return x.st == FG_ERR_PIPELINE ? FG_ERR_DEVICE_REQUEST_FAILED : x.st;
  }
  *out = e;
  return FG_OK;
}

fg_status fg_engine_destroy(fg_engine* e) {
  if (!e) return FG_ERR_INVALID_ARG;
  {
    std::lock_guard<std::recursive_mutex> lk(e->mu);
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    e->timer.destroy();
    cudaFree(e->d_err);
    cudaFree(e->d_stats);
    cudaStreamDestroy(e->stream);
  }
  delete e;
  return FG_OK;
}

const char* fg_last_error(const fg_engine* e) { return e ? e->err.c_str() : "no engine"; }
const char* fg_engine_device_name(const fg_engine* e) { return e ? e->name.c_str() : ""; }

fg_status fg_engine_timings(const fg_engine* e, fg_timings* out) {
  if (!e || !out) return FG_ERR_INVALID_ARG;
  *out = e->timings;
  return FG_OK;
}

fg_status fg_emulsion_preset(const char* name, double width, double height, fg_emulsion_cfg* c) {
  if (!name || !c) return FG_ERR_INVALID_ARG;
  std::string s(name);
  for (auto& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  *c = fg_emulsion_cfg{};
  c->width = width;
  c->height = height;
  c->optics.refractive_index = 1.534;
  if (s == "t-max" || s == "tmax" || s == "t-max-100") {
    c->depth = 8.0; c->r_min = 0.9; c->mean_crystal_radius = 0.40; c->size_variance = 0.20;
    c->morphology = FG_TABULAR; c->tabular_aspect_ratio = 6.5;
    c->optics.absorption_coeff = 0.002; c->optics.scattering_coeff = 0.035; c->optics.anisotropy_g = 0.85;
    c->optics.antihalation_reflectance = 0.08; c->optics.antihalation_density = 1.10;
    c->base_sensitivity = 0.8;
  } else if (s == "hp5" || s == "hp5-plus") {
    c->depth = 12.5; c->r_min = 1.1; c->mean_crystal_radius = 0.50; c->size_variance = 0.30;
    c->morphology = FG_OCTAHEDRAL; c->tabular_aspect_ratio = 1.0;
    c->optics.absorption_coeff = 0.0025; c->optics.scattering_coeff = 0.045; c->optics.anisotropy_g = 0.82;
    c->optics.antihalation_reflectance = 0.12; c->optics.antihalation_density = 0.85;
    c->base_sensitivity = 1.1;
  } else if (s == "tri-x-1600" || s == "trix-1600" || s == "caffenol") {
    c->depth = 14.5; c->r_min = 1.1; c->mean_crystal_radius = 0.52; c->size_variance = 0.38;
    c->morphology = FG_CUBIC; c->tabular_aspect_ratio = 1.0;
    c->optics.absorption_coeff = 0.0032; c->optics.scattering_coeff = 0.052; c->optics.anisotropy_g = 0.80;
    c->optics.antihalation_reflectance = 0.14; c->optics.antihalation_density = 0.80;
    c->base_sensitivity = 1.35;
  } else if (s == "tri-x" || s == "trix" || s == "tri-x-400") {
    c->depth = 14.0; c->r_min = 1.2; c->mean_crystal_radius = 0.55; c->size_variance = 0.40;
    c->morphology = FG_CUBIC; c->tabular_aspect_ratio = 1.0;
    c->optics.absorption_coeff = 0.003; c->optics.scattering_coeff = 0.050; c->optics.anisotropy_g = 0.80;
    c->optics.antihalation_reflectance = 0.14; c->optics.antihalation_density = 0.80;
    c->base_sensitivity = 1.2;
  } else {
    return FG_ERR_INVALID_ARG;
  }
  return FG_OK;
}

fg_status fg_emulsion_upload(fg_engine* e, const fg_emulsion_cfg* cfg, const fg_crystals_host* c,
                             size_t n, fg_emulsion** out) {
  if (!out) return FG_ERR_INVALID_ARG;
  *out = nullptr;
  return guard(e, [&] {
    FG_REQUIRE(cfg && c, "null config or crystals");
    FG_REQUIRE(n == 0 || (c->pos && c->dims && c->quat && c->sensitivity), "null crystal array");
    FG_REQUIRE(n < 0x7ffffff0u, "too many crystals");
    cudaStream_t st = e->stream;
    begin_call(e);
    std::unique_ptr<fg_emulsion> em(new fg_emulsion());
    em->cfg = *cfg;
    em->n = static_cast<uint32_t>(n);
    em->stream = st;
    em->has64 = true;
    for (size_t i = 0; i < 3 * n; ++i) em->extent = std::max(em->extent, std::fabs(c->pos[i]));
    for (size_t i = 0; i < 3 * n; ++i) em->max_half_dim = std::max(em->max_half_dim, c->dims[i]);
    em->any_cubic = c->morphology ? std::any_of(c->morphology, c->morphology + n, [](int32_t m) { return m == FG_CUBIC; })
                                  : cfg->morphology == FG_CUBIC;
    FG_CUDA(cudaEventRecord(e->timer.ev[0], st));
    if (n) {
      DBuf<double> pos, dims, quat, sens;
      DBuf<int32_t> morph;
      to_device(pos, c->pos, 3 * n, st);
      to_device(dims, c->dims, 3 * n, st);
      to_device(quat, c->quat, 4 * n, st);
      to_device(sens, c->sensitivity, n, st);
      if (c->morphology) to_device(morph, c->morphology, n, st);
      em->a.alloc(n, st); em->q.alloc(n, st); em->d.alloc(n, st);
      em->pos64.alloc(3 * n, st); em->dims64.alloc(3 * n, st);
      em->quat64.alloc(4 * n, st); em->sens64.alloc(n, st);
      em->sorted_to_id.alloc(n, st); em->id_to_sorted.alloc(n, st);
      DBuf<uint64_t> keys;
      DBuf<uint32_t> order;
      morton_order(em.get(), c->pos, pos.p, st, keys, order);
      gather_sorted(em.get(), order.p, pos.p, dims.p, quat.p, sens.p, c->morphology ? morph.p : nullptr,
                    cfg->morphology, st);
      alloc_state(em.get(), st);
      em->h_s2id.resize(n);
      FG_CUDA(cudaMemcpyAsync(em->h_s2id.data(), em->sorted_to_id.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaStreamSynchronize(st));
      DBuf<uint32_t> none;
      build_emulsion_tree(e, em.get(), false, em->rt, none);
    } else {
      alloc_state(em.get(), st);
    }
    FG_CUDA(cudaEventRecord(e->timer.ev[1], st));
    FG_CUDA(cudaStreamSynchronize(st));
    e->timings.bvh_ms = elapsed(e->timer.ev[0], e->timer.ev[1]);
    e->timings.total_ms = e->timings.bvh_ms;
    e->timings.crystals = n;
    end_call(e);
    *out = em.release();
  });
}

fg_status fg_emulsion_destroy(fg_engine* e, fg_emulsion* em) {
  if (!em) return FG_ERR_INVALID_ARG;
  return guard(e, [&] {
    FG_CUDA(cudaStreamSynchronize(e->stream));
    delete em;
    FG_CUDA(cudaStreamSynchronize(e->stream));
  });
}

fg_status fg_emulsion_count(const fg_emulsion* em, size_t* n) {
  if (!em || !n) return FG_ERR_INVALID_ARG;
  *n = em->n;
  return FG_OK;
}

fg_status fg_emulsion_download(fg_engine* e, const fg_emulsion* em, fg_crystals_out* out) {
  return guard(e, [&] {
    FG_REQUIRE(em && out, "null emulsion or output");
    const uint32_t n = em->n;
    if (!n) return;
    cudaStream_t st = e->stream;
    std::vector<float4> a(n), q(n), d(n);
    FG_CUDA(cudaMemcpyAsync(a.data(), em->a.p, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaMemcpyAsync(q.data(), em->q.p, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaMemcpyAsync(d.data(), em->d.p, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
    std::vector<double> p64, d64, q64, s64;
    if (em->has64) {
      p64.resize(3 * n); d64.resize(3 * n); q64.resize(4 * n); s64.resize(n);
      FG_CUDA(cudaMemcpyAsync(p64.data(), em->pos64.p, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaMemcpyAsync(d64.data(), em->dims64.p, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaMemcpyAsync(q64.data(), em->quat64.p, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaMemcpyAsync(s64.data(), em->sens64.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    FG_CUDA(cudaStreamSynchronize(st));
    for (uint32_t s = 0; s < n; ++s) {
      const uint32_t i = em->h_s2id.empty() ? s : em->h_s2id[s];
      if (out->pos)
        for (int j = 0; j < 3; ++j) out->pos[3 * i + j] = em->has64 ? p64[3 * s + j] : (&a[s].x)[j];
      if (out->dims)
        for (int j = 0; j < 3; ++j) out->dims[3 * i + j] = em->has64 ? d64[3 * s + j] : (&d[s].x)[j];
      if (out->quat)
        for (int j = 0; j < 4; ++j) out->quat[4 * i + j] = em->has64 ? q64[4 * s + j] : (&q[s].x)[j];
      if (out->sensitivity) out->sensitivity[i] = em->has64 ? s64[s] : a[s].w;
      if (out->morphology) {
        int32_t mo;
        std::memcpy(&mo, &d[s].w, sizeof(mo));
        out->morphology[i] = mo;
      }
    }
  });
}

fg_status fg_emulsion_get_counts(fg_engine* e, const fg_emulsion* em, uint32_t* counts) {
  return guard(e, [&] {
    FG_REQUIRE(em && counts, "null argument");
    std::vector<uint32_t> v(em->n);
    if (em->n) FG_CUDA(cudaMemcpyAsync(v.data(), em->counts.p, em->n * sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream));
    FG_CUDA(cudaStreamSynchronize(e->stream));
    from_sorted(em, v, counts);
  });
}

fg_status fg_emulsion_set_counts(fg_engine* e, fg_emulsion* em, const uint32_t* counts) {
  return guard(e, [&] {
    FG_REQUIRE(em && counts, "null argument");
    const std::vector<uint32_t> v = to_sorted(em, counts);
    if (em->n) FG_CUDA(cudaMemcpyAsync(em->counts.p, v.data(), em->n * sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
    FG_CUDA(cudaStreamSynchronize(e->stream));
  });
}

fg_status fg_emulsion_get_development(fg_engine* e, const fg_emulsion* em, uint8_t* developed,
                                      int64_t* clump, double* expansion) {
  return guard(e, [&] {
    FG_REQUIRE(em, "null emulsion");
    const uint32_t n = em->n;
    std::vector<uint8_t> dv(n);
    std::vector<double> ex(n);
    if (n) {
      FG_CUDA(cudaMemcpyAsync(dv.data(), em->developed.p, n, cudaMemcpyDeviceToHost, e->stream));
      FG_CUDA(cudaMemcpyAsync(ex.data(), em->exp64.p, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
      if (clump) FG_CUDA(cudaMemcpyAsync(clump, em->clump.p, n * sizeof(int64_t), cudaMemcpyDeviceToHost, e->stream));
    }
    FG_CUDA(cudaStreamSynchronize(e->stream));
    if (developed) from_sorted(em, dv, developed);
    if (expansion) from_sorted(em, ex, expansion);
  });
}

fg_status fg_emulsion_set_development(fg_engine* e, fg_emulsion* em, const uint8_t* developed,
                                      const double* expansion) {
  return guard(e, [&] {
    FG_REQUIRE(em && developed && expansion, "null argument");
    const uint32_t n = em->n;
    const std::vector<uint8_t> dv = to_sorted(em, developed);
    const std::vector<double> ex = to_sorted(em, expansion);
    std::vector<float> ex32(n);
    for (uint32_t s = 0; s < n; ++s) ex32[s] = static_cast<float>(ex[s]);
    if (n) {
      FG_CUDA(cudaMemcpyAsync(em->developed.p, dv.data(), n, cudaMemcpyHostToDevice, e->stream));
      FG_CUDA(cudaMemcpyAsync(em->exp64.p, ex.data(), n * sizeof(double), cudaMemcpyHostToDevice, e->stream));
      FG_CUDA(cudaMemcpyAsync(em->exp32.p, ex32.data(), n * sizeof(float), cudaMemcpyHostToDevice, e->stream));
      FG_CUDA(cudaMemsetAsync(em->clump.p, 0xff, n * sizeof(int64_t), e->stream));
    }
    FG_CUDA(cudaStreamSynchronize(e->stream));
  });
}

fg_status fg_expose_emulsion(fg_engine* e, fg_emulsion* em, const float* tile, uint32_t tw,
                             uint32_t th, const fg_exposure_cfg* cfg, uint64_t seed) {
  return guard(e, [&] {
    FG_REQUIRE(em && tile && cfg, "null argument");
    FG_REQUIRE(tw > 0 && th > 0, "tile size must be positive");
    cudaStream_t st = e->stream;
    begin_call(e);
    DBuf<float> t;
    to_device(t, tile, static_cast<size_t>(tw) * th, st);
    FG_CUDA(cudaEventRecord(e->timer.ev[0], st));
    unsigned long long P = 0;
    expose(e, em, t.p, tw, th, *cfg, seed, &P);
    FG_CUDA(cudaEventRecord(e->timer.ev[1], st));
    FG_CUDA(cudaStreamSynchronize(st));
    e->timings.transport_ms = elapsed(e->timer.ev[0], e->timer.ev[1]);
    e->timings.total_ms = e->timings.transport_ms;
    e->timings.photons = P;
    e->timings.crystals = em->n;
    e->timings.kernel_launches = P ? 1 : 0;
    end_call(e);
  });
}

fg_status fg_develop_emulsion(fg_engine* e, fg_emulsion* em, const fg_dev_cfg* cfg,
                              fg_dev_report* report) {
  return guard(e, [&] {
    FG_REQUIRE(em && cfg, "null argument");
    begin_call(e);
    FG_CUDA(cudaEventRecord(e->timer.ev[0], e->stream));
    develop(e, em, *cfg, report);
    FG_CUDA(cudaEventRecord(e->timer.ev[1], e->stream));
    FG_CUDA(cudaStreamSynchronize(e->stream));
    e->timings.develop_ms = elapsed(e->timer.ev[0], e->timer.ev[1]);
    e->timings.total_ms = e->timings.develop_ms;
    e->timings.crystals = em->n;
    end_call(e);
  });
}

static void run_scan(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg, uint64_t seed,
                     const float* sigma, float* out, uint8_t* image8, uint16_t* ray_hits) {
  FG_REQUIRE(em && cfg, "null argument");
  cudaStream_t st = e->stream;
  begin_call(e);
  const size_t npx = static_cast<size_t>(cfg->width_px) * cfg->height_px;
  const uint32_t spp = std::max<uint32_t>(cfg->samples_per_pixel, 1);
  const uint32_t g = static_cast<uint32_t>(std::lround(std::sqrt(static_cast<double>(spp))));
  const size_t a = std::max<uint32_t>(g * g, 1);
  DBuf<float> d_out, d_sig;
  DBuf<uint8_t> d_img;
  DBuf<uint16_t> d_hits;
  ScanOut so;
  if (out) { d_out.alloc(npx, st); so.out = d_out.p; }
  if (image8) { d_img.alloc(npx, st); so.image8 = d_img.p; }
  if (ray_hits) { d_hits.alloc(npx * a, st); so.ray_hits = d_hits.p; }
  if (sigma) {
    const std::vector<float> sv = to_sorted(em, sigma);
    to_device(d_sig, sv.data(), sv.size(), st);
  }
  FG_CUDA(cudaEventRecord(e->timer.ev[0], st));
  scan(e, em, *cfg, seed, sigma ? d_sig.p : nullptr, so);
  FG_CUDA(cudaEventRecord(e->timer.ev[1], st));
  if (out) FG_CUDA(cudaMemcpyAsync(out, d_out.p, npx * sizeof(float), cudaMemcpyDeviceToHost, st));
  if (image8) FG_CUDA(cudaMemcpyAsync(image8, d_img.p, npx, cudaMemcpyDeviceToHost, st));
  if (ray_hits) FG_CUDA(cudaMemcpyAsync(ray_hits, d_hits.p, npx * a * sizeof(uint16_t), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  e->timings.scan_ms = elapsed(e->timer.ev[0], e->timer.ev[1]);
  e->timings.total_ms = e->timings.scan_ms;
  e->timings.rays = npx * a;
  e->timings.crystals = em->n;
  end_call(e);
}

fg_status fg_scan_emulsion(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg,
                           uint64_t seed, const float* sigma_per_crystal, float* out,
                           uint8_t* image8) {
  return guard(e, [&] { run_scan(e, em, cfg, seed, sigma_per_crystal, out, image8, nullptr); });
}

fg_status fg_scan_ray_hits(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg,
                           uint64_t seed, uint16_t* ray_hits) {
  return guard(e, [&] {
    FG_REQUIRE(ray_hits, "null output");
    run_scan(e, em, cfg, seed, nullptr, nullptr, nullptr, ray_hits);
  });
}

fg_status fg_replay_segments(fg_engine* e, fg_emulsion* em, const fg_exposure_cfg* cfg,
                             uint64_t seed, const fg_segment* segs, size_t nseg,
                             uint32_t* offsets, uint32_t* ids, size_t id_cap, size_t* nhits) {
  return guard(e, [&] {
    FG_REQUIRE(em && cfg && (segs || nseg == 0), "null argument");
    begin_call(e);
    replay_segments(e, em, *cfg, seed, segs, nseg, offsets, ids, id_cap, nhits);
    end_call(e);
  });
}

fg_status fg_replay_rays(fg_engine* e, const fg_emulsion* em, const double* origins,
                         const double* dirs, size_t nrays, int developed_only, uint32_t* offsets,
                         uint32_t* ids, size_t id_cap, size_t* nhits, double* chord_sum) {
  return guard(e, [&] {
    FG_REQUIRE(em && ((origins && dirs) || nrays == 0), "null argument");
    begin_call(e);
    replay_rays(e, em, origins, dirs, nrays, developed_only, offsets, ids, id_cap, nhits, chord_sum);
    end_call(e);
  });
}

}  // extern "C"
