// threads_main.cpp -- TEST INFRASTRUCTURE: the drop-in adapter
// (reference_adapter.cpp) driven as the reference's main() and its timer
// threads drive a Renderer (src/main.cpp:98-151,
// src/tools/StopRendererWithTimer.cpp:38-40, src/tools/FileSaverCallerWithTimer.cpp:59-66),
// linked with tests/adapter/fake_or3.cpp instead of libor3.so.  Checks:
//   1. a full render delivers every pass;
//   2. a second RenderScene on the same renderer still honours StopRendering
//      sent from another thread;
//   3. after a stop the renderer renders nothing, as the reference's does;
//   4. GetResult() readers polling from another thread never see a frame that
//      is being written (every pixel of a frame holds the same count);
//   5. an exception thrown by the frame callback leaves RenderScene with the
//      stop watch joined (no std::terminate), and the renderer renders again.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <stdexcept>
#include <thread>

#include "stdafx.h"
#include "renderer/Camera.h"
#include "renderer/Renderer.h"
#include "renderer/ScreenPixels.hpp"
#include "scenes/CornellBoxScene.h"

namespace OmochiRenderer {
std::shared_ptr<Renderer> MakeGpuPathTracer(
    const Camera &camera, int min_samples, int max_samples, int step, int supersamples,
    std::function<void(int, const Color *, size_t, size_t, double)> callback, bool nee);
}

using namespace OmochiRenderer;

static int fails = 0;
#define CHECK(c)                                              \
  do {                                                        \
    if (!(c)) {                                               \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
      fails++;                                                \
    }                                                         \
  } while (0)

int main() {
  Camera camera(64, 48, Vector3(50, 55, 230), Vector3(0.00001, -0.15, -1.0), Vector3(0, 1, 0), 30.0, 40.0, 300);
  CornellBoxScene scene;
  const int kMax = 60;  // passes of 5 ms
  std::atomic<int> frames(0);
  auto r = MakeGpuPathTracer(camera, 1, kMax, 1, 2,
                             [&frames](int, const Color *, size_t, size_t, double) { frames++; }, false);

  // a reader polling GetResult() while the renders run.  Double buffering
  // promises whole frames to a reader that is done before the next pass
  // completes (a pass takes 5 ms here); a read the scheduler stretched past
  // 2 ms is not counted.
  std::atomic<bool> reading(true);
  std::atomic<long> reads(0), torn(0), slow(0);
  std::thread reader([&]() {
    while (reading.load()) {
      const auto t0 = std::chrono::steady_clock::now();
      const ScreenPixels *px = r->GetResult();
      const Color *c = px->GetScreen();
      const size_t n = px->CalcScreenWidth() * px->CalcScreenHeight();
      const double v = c[0].x;
      bool whole = true;
      for (size_t i = 1; i < n; i++)
        if (c[i].x != v || c[i].z != v) {
          whole = false;
          break;
        }
      if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(2)) {
        slow++;
        continue;
      }
      if (!whole) torn++;
      reads++;
    }
  });

  // 1. a full render
  r->RenderScene(scene);
  CHECK(r->GetCurrentSampleCount() == kMax);
  CHECK(frames.load() == kMax);

  // 2. the same renderer again, stopped from a timer thread after ~80 ms
  frames = 0;
  std::thread timer([&]() {
    std::this_thread::sleep_for(std::chrono::milliseconds(80));
    r->StopRendering();
  });
  const auto t0 = std::chrono::steady_clock::now();
  r->RenderScene(scene);
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  timer.join();
  CHECK(frames.load() > 0);
  CHECK(frames.load() < kMax);
  CHECK(ms < kMax * 5 * 0.8);

  // 3. a stopped renderer stays stopped
  frames = 0;
  r->RenderScene(scene);
  CHECK(frames.load() == 0);

  reading = false;
  reader.join();
  CHECK(reads.load() > 0);
  CHECK(torn.load() == 0);

  // 5. an exception from the frame callback
  std::atomic<int> throws(1);
  auto r2 = MakeGpuPathTracer(camera, 1, 10, 1, 2,
                              [&throws](int s, const Color *, size_t, size_t, double) {
                                if (s == 3 && throws-- > 0) throw std::runtime_error("saver failed");
                              },
                              false);
  bool threw = false;
  try {
    r2->RenderScene(scene);
  } catch (const std::runtime_error &) {
    threw = true;
  }
  CHECK(threw);
  CHECK(r2->GetCurrentSampleCount() == 3);
  r2->RenderScene(scene);  // and it renders again
  CHECK(r2->GetCurrentSampleCount() == 10);

  std::printf("reads %ld torn %ld (slow reads not counted %ld) stopped after %.1f ms, fails %d\n", reads.load(),
              torn.load(), slow.load(), ms, fails);
  return fails ? 1 : 0;
}
