// adapter_main.cpp -- links the drop-in adapter into a program that uses the
// reference's own scene and camera classes, exactly as its main.cpp would.
// Built by tests/test_reference_adapter.py; run only where a GPU exists.
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

int main() {
  Camera camera(64, 48, Vector3(50, 55, 230), Vector3(0.00001, -0.15, -1.0), Vector3(0, 1, 0), 30.0, 40.0, 300);
  CornellBoxScene scene;
  int frames = 0;
  auto r = MakeGpuPathTracer(camera, 1, 3, 1, 2,
                             [&frames](int, const Color *, size_t w, size_t h, double) { frames += (w == 128 && h == 48); },
                             false);
  r->RenderScene(scene);
  const ScreenPixels *px = r->GetResult();
  double sum = 0;
  for (size_t i = 0; i < px->CalcScreenWidth() * px->CalcScreenHeight(); i++) sum += px->GetScreen()[i].x;
  printf("frames %d samples %d mean %.6f\n", frames, r->GetCurrentSampleCount(), sum / (64 * 48));
  return (frames == 3 && r->GetCurrentSampleCount() == 3 && sum > 0) ? 0 : 1;
}
