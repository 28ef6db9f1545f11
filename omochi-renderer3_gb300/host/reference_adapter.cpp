// reference_adapter.cpp -- the drop-in for omochi-renderer3's render call.
//
// Compiled inside the reference's own build (include path = its src/), this
// translation unit provides OmochiRenderer::GpuPathTracerAdapter, a
// `Renderer` (src/renderer/Renderer.h:10-23) with PathTracer's constructor
// (src/renderer/PathTracer.h:25-37).  main.cpp changes by one line:
//     std::make_shared<PathTracer>(camera, start, end, step, ss, callback)
//  -> std::make_shared<GpuPathTracerAdapter>(camera, start, end, step, ss, callback)
// (src/main.cpp:103-104).  RenderScene flattens the reference Scene into an
// or3_scene_desc and renders it on the GPU through libor3.so; GetResult
// returns a reference ScreenPixels with the same 2W x H layout.
//
// The reference keeps Scene's object lists protected and Polygon's geometry
// private (src/scenes/Scene.h:110-118, src/renderer/Polygon.h:108-111); this TU
// alone reads them by compiling the reference headers with `private` and
// `protected` redefined after the standard headers are in (class layouts are
// unchanged; no reference file is edited).
#include <algorithm>
#include <atomic>
#include <cassert>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <ctime>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stack>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#define private public
#define protected public
#include "stdafx.h"
#include "renderer/AxisAlignedPlane.h"
#include "renderer/Camera.h"
#include "renderer/IBL.h"
#include "renderer/InfiniteFloor.h"
#include "renderer/Polygon.h"
#include "renderer/Renderer.h"
#include "renderer/ScreenPixels.hpp"
#include "renderer/Sphere.h"
#include "renderer/SphereLight.h"
#include "scenes/Scene.h"
#include "tools/ImageHandler.h"
#undef private
#undef protected

#include "or3.h"
#include "or3_gpu_path_tracer.hpp"
#include "reference_flatten.hpp"

namespace OmochiRenderer {

class GpuPathTracerAdapter : public Renderer {
 public:
  typedef std::function<void(int samples, const Color *result, size_t width, size_t height, double minutes)>
      RenderingFinishCallbackFunction;

  GpuPathTracerAdapter(const Camera &camera, int min_samples, int max_samples, int step, int supersamples,
                       RenderingFinishCallbackFunction callback)
      : camera_(camera), callback_(callback),
        gpu_(to_or3(camera), min_samples, max_samples, step, supersamples,
             [this](int s, const double *rgb, size_t w, size_t h, double minutes) { on_frame(s, rgb, w, h, minutes); }) {
    for (ScreenPixels &r : result_) r.InitializePixels(camera.GetScreenWidth(), camera.GetScreenHeight(), 2, 1);
  }

  void EnableNextEventEstimation(bool enable = true) { gpu_.EnableNextEventEstimation(enable); }
  void SetMaxThreadCount(size_t count) { gpu_.SetMaxThreadCount(count); }

  void RenderScene(const Scene &scene) override {
    // A stopped renderer stays stopped, as the reference's does: its pass
    // loop tests m_enableRendering, which nothing sets back (PathTracer.cpp:70).
    if (!m_enableRendering) return;
    FlatScene flat(scene);
    const or3_scene_desc d = flat.desc();
    // The stop watch forwards Renderer::StopRendering (a plain bool set by a
    // timer thread) to the GPU render.  It runs for this call only: the guard
    // ends and joins it on every way out, exceptions included.
    struct WatchGuard {
      GpuPathTracerAdapter *a;
      ~WatchGuard() {
        a->done_.store(true);
        if (a->stop_watch_.joinable()) a->stop_watch_.join();
      }
    } guard{this};
    done_.store(false);
    stop_watch_ = std::thread([this]() {
      while (!done_.load()) {
        if (!m_enableRendering) gpu_.StopRendering();
        std::this_thread::sleep_for(std::chrono::milliseconds(20));
      }
    });
    gpu_.RenderScene(d);
  }

  // The last completed frame.  Frames are double-buffered: a pass writes the
  // buffer readers were not given, then publishes it, so a reader that
  // finishes with the pointer before the next pass ends never sees a frame
  // being written (the reference's savers read it from timer threads,
  // src/tools/FileSaverCallerWithTimer.cpp:59-66).
  const ScreenPixels *GetResult() const override { return &result_[front_.load(std::memory_order_acquire)]; }
  const int GetCurrentSampleCount() const override { return gpu_.GetCurrentSampleCount(); }
  std::string GetCurrentRenderingInfo() const override { return gpu_.GetCurrentRenderingInfo(); }

 private:
  void on_frame(int samples, const double *rgb, size_t w, size_t h, double minutes) {
    const int back = 1 - front_.load(std::memory_order_relaxed);
    Color *px = result_[back].m_pixels;
    for (size_t i = 0; i < w * h; i++) px[i] = Color(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    front_.store(back, std::memory_order_release);
    if (callback_) callback_(samples, result_[back].GetScreen(), w, h, minutes);
  }

  Camera camera_;
  RenderingFinishCallbackFunction callback_;
  ScreenPixels result_[2];
  std::atomic<int> front_{0};
  or3::GpuPathTracer gpu_;
  std::thread stop_watch_;
  std::atomic<bool> done_{false};
};

// Factory used by main.cpp's one-line change (returns the Renderer base).
std::shared_ptr<Renderer> MakeGpuPathTracer(const Camera &camera, int min_samples, int max_samples, int step,
                                            int supersamples,
                                            GpuPathTracerAdapter::RenderingFinishCallbackFunction callback,
                                            bool next_event_estimation) {
  auto r = std::make_shared<GpuPathTracerAdapter>(camera, min_samples, max_samples, step, supersamples, callback);
  r->EnableNextEventEstimation(next_event_estimation);
  return r;
}

}  // namespace OmochiRenderer
