// flatten_probe.cpp -- TEST INFRASTRUCTURE: the drop-in adapter's scene
// flattener (omochi-renderer3_gb300/host/reference_flatten.hpp) run on scenes
// the reference itself builds, so a test can compare its or3_scene_desc with
// the native scene-file reader's and with the Python scene builders.
// Built by tests/test_reference_adapter.py against the reference's objects.
#include <algorithm>
#include <atomic>
#include <cassert>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
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
#include "renderer/Sphere.h"
#include "renderer/SphereLight.h"
#include "scenes/CornellBoxScene.h"
#include "scenes/Scene.h"
#include "scenes/SceneFromExternalFile.h"
#include "tools/ImageHandler.h"
#undef private
#undef protected

#include "or3.h"
#include "reference_flatten.hpp"

using namespace OmochiRenderer;

extern "C" {

// The reference's SceneFromExternalFile(path) flattened; NULL if it rejects the file.
void *flat_scene_file(const char *path, or3_scene_desc *out) {
  SceneFromExternalFile scene(path);
  if (!scene.IsValid()) return nullptr;
  FlatScene *f = new FlatScene(scene);
  *out = f->desc();
  return f;
}

// The reference's built-in CornellBoxScene (src/scenes/CornellBoxScene.cpp) flattened.
void *flat_cornell(or3_scene_desc *out) {
  CornellBoxScene scene;
  FlatScene *f = new FlatScene(scene);
  *out = f->desc();
  return f;
}

void flat_free(void *p) { delete static_cast<FlatScene *>(p); }

}  // extern "C"
