// or3_gpu_path_tracer.hpp -- C++ host mirror of the reference's PathTracer over
// the C ABI in include/or3.h (header-only; link libor3.so).
//
// Same constructors, setters and Renderer methods as
// OmochiRenderer::PathTracer (src/renderer/PathTracer.h:18-88,
// src/renderer/Renderer.h:10-23), taking the flattened scene (or3_scene_desc)
// instead of a Scene object.  Errors never abort: RenderScene returns the
// C ABI status and the message stays available through LastError(), and, as
// the reference does, it is also written to stderr.
#pragma once

#include <atomic>
#include <cstdio>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "or3.h"

namespace or3 {

class GpuPathTracer {
 public:
  // PathTracer::RenderingFinishCallbackFunction (src/renderer/PathTracer.h:21)
  typedef std::function<void(int samples, const double *result, size_t width, size_t height,
                             double accumulatedRenderingTime)>
      RenderingFinishCallbackFunction;

  GpuPathTracer(const or3_camera &camera, int samples, int supersamples, int device = 0)
      : GpuPathTracer(camera, samples, samples, 1, supersamples, nullptr, device) {}

  GpuPathTracer(const or3_camera &camera, int min_samples, int max_samples, int step, int supersamples,
                RenderingFinishCallbackFunction callback, int device = 0)
      : camera_(camera), callback_(callback) {
    params_.min_samples = min_samples;
    params_.max_samples = max_samples;
    params_.step_samples = step;
    params_.supersamples = supersamples;
    params_.next_event_estimation = 0;
    params_.rr_min_depth = 5;  // PathTracer.cpp:177
    params_.max_depth = 0;
    params_.output_layout = OR3_LAYOUT_REFERENCE;
    params_.seed = 0;
    params_.wave_paths = 0;
    params_.flags = 0;
    params_.tuning = 0;
    status_ = or3_context_create(device, &ctx_);
    if (status_ != OR3_OK) report("cannot create a CUDA context");
  }

  ~GpuPathTracer() {
    if (ctx_) {
      if (scene_ >= 0) or3_scene_release(ctx_, scene_);
      or3_context_destroy(ctx_);
    }
  }

  GpuPathTracer(const GpuPathTracer &) = delete;
  GpuPathTracer &operator=(const GpuPathTracer &) = delete;

  void EnableNextEventEstimation(bool enable = true) { params_.next_event_estimation = enable ? 1 : 0; }
  // Host threads do not apply to the GPU path; kept for interface parity.
  void SetMaxThreadCount(size_t count) { threads_ = count == 0 ? 1 : count; }
  // Depth policy (not in the reference): RR for depth > rr_min_depth, no ray at depth >= max_depth (0 = none).
  void SetDepthLimits(int rr_min_depth, int max_depth) {
    params_.rr_min_depth = rr_min_depth;
    params_.max_depth = max_depth;
  }
  void SetSeed(uint64_t seed) { params_.seed = seed; }

  // Renderer::RenderScene: uploads (flattens) the scene, then runs every pass,
  // calling the callback after each one.  Blocking.
  int RenderScene(const or3_scene_desc &scene) {
    if (!ctx_) return status_;
    if (scene_ >= 0) {
      or3_scene_release(ctx_, scene_);
      scene_ = -1;
    }
    status_ = or3_scene_upload(ctx_, &scene, &scene_);
    if (status_ != OR3_OK) return report("scene upload failed");
    enabled_.store(true);
    or3_reset_stop(ctx_);
    status_ = or3_render(ctx_, scene_, &camera_, &params_, &GpuPathTracer::on_frame, this);
    if (status_ != OR3_OK) return report("render failed");
    return OR3_OK;
  }

  // Renderer::GetResult: the last completed frame, 2W x H RGB doubles with
  // the image in the left viewport and rows top-down (ScreenPixels layout).
  // Safe to call from other threads while RenderScene runs.
  std::shared_ptr<const std::vector<double>> GetResult() const {
    std::lock_guard<std::mutex> lk(mu_);
    return result_;
  }
  size_t CalcScreenWidth() const { return 2 * (size_t)camera_.width; }
  size_t CalcScreenHeight() const { return camera_.height; }

  int GetCurrentSampleCount() const { return current_.load(); }

  std::string GetCurrentRenderingInfo() const {
    or3_render_stats s{};
    if (ctx_) or3_get_stats(ctx_, &s);
    char buf[256];
    std::snprintf(buf, sizeof(buf), "(width, height) = (%u, %u)\nsamples / pixel = %dx(%dx%d)\nextension rays = %llu\n",
                  camera_.width, camera_.height, current_.load(), params_.supersamples, params_.supersamples,
                  (unsigned long long)s.extension_rays);
    return buf;
  }

  // Renderer::StopRendering; may be called from any thread.
  void StopRendering() {
    enabled_.store(false);
    if (ctx_) or3_stop(ctx_);
  }

  int LastStatus() const { return status_; }
  std::string LastError() const { return ctx_ ? or3_last_error(ctx_) : "no CUDA context"; }

 private:
  static void on_frame(void *user, int32_t samples, const double *rgb, size_t w, size_t h, double minutes) {
    GpuPathTracer *self = static_cast<GpuPathTracer *>(user);
    auto frame = std::make_shared<std::vector<double>>(rgb, rgb + w * h * 3);
    {
      std::lock_guard<std::mutex> lk(self->mu_);
      self->result_ = frame;
    }
    self->current_.store(samples);
    if (self->callback_) self->callback_(samples, frame->data(), w, h, minutes);
  }

  int report(const char *what) {
    std::fprintf(stderr, "GpuPathTracer: %s: %s (status %d)\n", what, LastError().c_str(), status_);
    return status_;
  }

  or3_camera camera_;
  or3_render_params params_{};
  RenderingFinishCallbackFunction callback_;
  or3_context *ctx_ = nullptr;
  int32_t scene_ = -1;
  int status_ = OR3_OK;
  size_t threads_ = 1;
  std::atomic<bool> enabled_{true};
  std::atomic<int> current_{0};
  mutable std::mutex mu_;
  std::shared_ptr<const std::vector<double>> result_;
};

}  // namespace or3
