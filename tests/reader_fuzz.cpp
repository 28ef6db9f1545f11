// reader_fuzz.cpp -- seeded mutation run of the host-side file readers
// (or3_read_hdr, or3_mesh_load_obj through or3_scene_load_file), built by
// tests/test_reader_fuzz.py with AddressSanitizer and UndefinedBehaviorSanitizer
// so that any read past a buffer, use after free or undefined arithmetic on a
// malformed file aborts the run.  Every mutated input must load or fail with a
// status.
//
//   reader_fuzz <staged scene dir> <rle.hdr> <flat.hdr> <scene iterations> <hdr iterations>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "or3.h"

namespace {

std::string slurp(const std::string &p) {
  std::ifstream f(p, std::ios::binary);
  std::stringstream s;
  s << f.rdbuf();
  return s.str();
}

void spit(const std::string &p, const std::string &t) {
  std::ofstream f(p, std::ios::binary);
  f << t;
}

std::string mutate_text(const std::string &t, std::mt19937 &rng) {
  static const char kChars[] = "{}:,#/ \n0123456789.-e";
  std::string s = t;
  const int m = 1 + (int)(rng() % 4);
  for (int i = 0; i < m && !s.empty(); i++) {
    const size_t j = rng() % s.size();
    switch (rng() % 5) {
      case 0: s.erase(j, 1 + rng() % 40); break;
      case 1: s.insert(j, 1, kChars[rng() % (sizeof(kChars) - 1)]); break;
      case 2: s[j] = kChars[rng() % (sizeof(kChars) - 1)]; break;
      case 3: s.resize(j); break;
      default: s.insert(j, s.substr(rng() % s.size(), 1 + rng() % 60)); break;
    }
  }
  return s;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 6) return 2;
  const std::string dir = argv[1];
  const int scene_iters = std::atoi(argv[4]), hdr_iters = std::atoi(argv[5]);
  std::mt19937 rng(11);
  int ok = 0, failed = 0;

  const std::string scene = slurp(dir + "/full.scene"), obj = slurp(dir + "/obj/mesh.obj"),
                    mtl = slurp(dir + "/obj/mesh.mtl");
  for (int k = 0; k < scene_iters; k++) {
    const int which = (int)(rng() % 3);
    spit(dir + "/m.scene", which == 0 ? mutate_text(scene, rng) : scene);
    spit(dir + "/obj/mesh.obj", which == 1 ? mutate_text(obj, rng) : obj);
    spit(dir + "/obj/mesh.mtl", which == 2 ? mutate_text(mtl, rng) : mtl);
    or3_scene_file *sf = nullptr;
    char err[256];
    const int rc = or3_scene_load_file((dir + "/m.scene").c_str(), 1 + rng() % 4, &sf, err, sizeof(err));
    if (rc == OR3_OK) {
      ok++;
      or3_scene_file_free(sf);
    } else if (rc == OR3_ERR_INVALID_ARGUMENT || rc == OR3_ERR_NOT_FOUND) {
      failed++;
    } else {
      std::printf("unexpected status %d\n", rc);
      return 1;
    }
  }

  for (int f = 2; f <= 3; f++) {
    const std::string s = slurp(argv[f]);
    const std::vector<uint8_t> base(s.begin(), s.end());
    for (int k = 0; k < hdr_iters; k++) {
      std::vector<uint8_t> b = base;
      switch (rng() % 3) {
        case 0: b.resize(rng() % b.size()); break;
        case 1:
          for (int i = 0, m = 1 + (int)(rng() % 8); i < m; i++) b[rng() % b.size()] = (uint8_t)rng();
          break;
        default: {
          std::vector<uint8_t> ins(1 + rng() % 64);
          for (auto &x : ins) x = (uint8_t)rng();
          b.insert(b.begin() + (long)(rng() % b.size()), ins.begin(), ins.end());
        }
      }
      // an exact-size heap copy: a read one byte past the end is reported
      uint8_t *buf = static_cast<uint8_t *>(std::malloc(b.size() ? b.size() : 1));
      if (!b.empty()) std::memcpy(buf, b.data(), b.size());
      uint32_t w = 0, h = 0;
      int rc = or3_read_hdr(buf, b.size(), &w, &h, nullptr, 0);
      if (rc == OR3_OK) {
        std::vector<uint8_t> out(4ull * w * h);
        rc = or3_read_hdr(buf, b.size(), &w, &h, out.data(), out.size());
      }
      std::free(buf);
      (rc == OR3_OK ? ok : failed)++;
    }
  }
  std::printf("ok %d failed %d\n", ok, failed);
  return 0;
}
