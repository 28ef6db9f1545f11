// fake_or3.cpp -- TEST INFRASTRUCTURE: a CPU stand-in for the part of
// libor3.so that the drop-in adapter calls (context, scene upload, or3_render
// with its per-pass frame callback, or3_stop), so the adapter's threading can
// be tested where no GPU exists.  or3_render sleeps `pass_ms` per pass and
// delivers frames whose every pixel holds the pass's sample count (a torn
// frame shows two counts); it checks the stop flag between passes as the real
// library does between waves and passes.
#include <atomic>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "or3.h"

struct or3_context {
  std::atomic<bool> stop{false};
  int renders = 0;
};

extern "C" {

int fake_pass_ms = 5;

int or3_context_create(int, or3_context **out) {
  *out = new or3_context();
  return OR3_OK;
}
int or3_context_destroy(or3_context *ctx) {
  delete ctx;
  return OR3_OK;
}
const char *or3_last_error(const or3_context *) { return ""; }
int or3_scene_upload(or3_context *, const or3_scene_desc *d, int32_t *scene_out) {
  if (!d || d->num_triangles + d->num_spheres + d->num_planes == 0) return OR3_ERR_INVALID_ARGUMENT;
  *scene_out = 1;
  return OR3_OK;
}
int or3_scene_release(or3_context *, int32_t) { return OR3_OK; }
int or3_stop(or3_context *ctx) {
  ctx->stop.store(true);
  return OR3_OK;
}
int or3_reset_stop(or3_context *ctx) {
  ctx->stop.store(false);
  return OR3_OK;
}
int or3_get_stats(or3_context *, or3_render_stats *s) {
  std::memset(s, 0, sizeof(*s));
  return OR3_OK;
}
int or3_render(or3_context *ctx, int32_t, const or3_camera *cam, const or3_render_params *p, or3_frame_callback cb,
               void *user) {
  const size_t w = 2 * (size_t)cam->width, h = cam->height;
  std::vector<double> frame(w * h * 3);
  ctx->renders++;
  for (int next = p->min_samples; next <= p->max_samples; next += p->step_samples) {
    if (ctx->stop.load()) break;
    std::this_thread::sleep_for(std::chrono::milliseconds(fake_pass_ms));
    for (double &v : frame) v = (double)next;
    if (cb) cb(user, next, frame.data(), w, h, 0.0);
  }
  return OR3_OK;
}

}  // extern "C"
