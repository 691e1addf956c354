// vt_cli.cpp — a C++ host of the renderer that uses nothing but the C ABI
// (include/vt.h, include/vt_diag.h), the way the reference application's
// Renderer would after the switch.
//
//   vt_cli vox FILE.vox OUT.pfm [WIDTH HEIGHT SPP]
//       MagicaVoxel file -> scene (interior emitters pruned), orbit camera
//       framing the volume, SPP progressive passes, the average image
//       written as a colour PFM (Renderer::loadVoxFile + render +
//       saveImage, src/renderer/renderer.h:54-72).  Prints the path rate.
//
//   vt_cli frame DIR
//       Renders one sample of a frame described by raw files in DIR and
//       writes its per-sample radiance and first hits next to them:
//         meta.txt      rx ry rz width height sample n_palette n_emissive env_w env_h
//         voxels.u8     rx*ry*rz palette entries, x fastest
//         palette.f32   n_palette records {type, emission[3], albedo[3], roughness}
//         emissive.i32  n_emissive linear voxel indices
//         env.f32       env_h*env_w*3 floats (absent when env_w == 0)
//         camera.bin    one vt_camera,  settings.bin  one vt_render_settings
//       -> rgba.f32 (height*width*4 floats), hits.i32 (height*width*4 ints).
//
// Exit status 0 on success, 1 on a library error (its message on stderr),
// 2 on bad arguments or unreadable files.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "vt.h"
#include "vt_diag.h"

namespace {

int die(const char* what) {
  std::fprintf(stderr, "vt_cli: %s: %s\n", what, vt_last_error());
  return 1;
}

#define CHECK(call)                  \
  do {                               \
    if ((call) != VT_OK) return die(#call); \
  } while (0)

bool read_file(const std::string& path, std::vector<uint8_t>& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return true;
}

template <class T>
bool read_array(const std::string& path, std::vector<T>& out, size_t count) {
  std::vector<uint8_t> bytes;
  if (!read_file(path, bytes) || bytes.size() != count * sizeof(T)) return false;
  out.resize(count);
  if (count) std::memcpy(out.data(), bytes.data(), bytes.size());
  return true;
}

bool write_file(const std::string& path, const void* data, size_t size) {
  std::ofstream f(path, std::ios::binary);
  f.write(static_cast<const char*>(data), (std::streamsize)size);
  return (bool)f;
}

int cmd_vox(int argc, char** argv) {
  if (argc != 4 && argc != 7) return 2;
  const int32_t w = argc == 7 ? std::atoi(argv[4]) : 512;
  const int32_t h = argc == 7 ? std::atoi(argv[5]) : 512;
  const int32_t spp = argc == 7 ? std::atoi(argv[6]) : 64;
  if (w <= 0 || h <= 0 || spp <= 0) return 2;
  std::vector<uint8_t> vox;
  if (!read_file(argv[2], vox)) {
    std::fprintf(stderr, "vt_cli: cannot read %s\n", argv[2]);
    return 2;
  }
  vt_context* ctx = nullptr;
  CHECK(vt_create(nullptr, &ctx));
  vt_scene* scene = nullptr;
  CHECK(vt_scene_create_from_vox(ctx, vox.data(), vox.size(), VT_SCENE_PRUNE_EMISSIVE, &scene));
  vt_scene_info info;
  CHECK(vt_scene_get_info(scene, &info));
  vt_camera cam;
  CHECK(vt_camera_default(&cam));
  CHECK(vt_camera_focus_on_bounds(&cam, info.bounds_min, info.bounds_max));
  vt_render_settings set;
  CHECK(vt_settings_default(&set));
  set.max_samples = spp;
  vt_job* job = nullptr;
  CHECK(vt_job_create(ctx, scene, nullptr, &cam, &set, w, h, &job));
  const auto t0 = std::chrono::steady_clock::now();
  int32_t result = VT_SAMPLES_PENDING;
  CHECK(vt_job_render(job, spp, &result));
  CHECK(vt_job_synchronize(job));
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::vector<float> rgba((size_t)w * h * 4);
  CHECK(vt_job_readback(job, rgba.data(), rgba.size() * sizeof(float), 0));
  size_t size = 0;
  CHECK(vt_image_encode_pfm(rgba.data(), w, h, 4, nullptr, 0, &size));
  std::vector<uint8_t> pfm(size);
  CHECK(vt_image_encode_pfm(rgba.data(), w, h, 4, pfm.data(), pfm.size(), &size));
  if (!write_file(argv[3], pfm.data(), size)) {
    std::fprintf(stderr, "vt_cli: cannot write %s\n", argv[3]);
    return 2;
  }
  std::printf("%d x %d x %d spp of a %d x %d x %d volume in %.3f s: %.1f Mpaths/s\n", w, h, spp,
              info.resolution[0], info.resolution[1], info.resolution[2], secs, (double)w * h * spp / secs / 1e6);
  vt_job_destroy(job);
  vt_scene_destroy(scene);
  vt_destroy(ctx);
  return 0;
}

int cmd_frame(int argc, char** argv) {
  if (argc != 3) return 2;
  const std::string dir = std::string(argv[2]) + "/";
  int32_t rx, ry, rz, w, h, sample, n_pal, env_w, env_h;
  long long n_em;
  {
    std::ifstream meta(dir + "meta.txt");
    if (!(meta >> rx >> ry >> rz >> w >> h >> sample >> n_pal >> n_em >> env_w >> env_h)) return 2;
  }
  std::vector<uint8_t> voxels;
  std::vector<float> pal_f, env_rgb;
  std::vector<int32_t> emissive;
  std::vector<uint8_t> cam_b, set_b;
  if (!read_array(dir + "voxels.u8", voxels, (size_t)rx * ry * rz) ||
      !read_array(dir + "palette.f32", pal_f, (size_t)n_pal * 8) ||
      !read_array(dir + "emissive.i32", emissive, (size_t)n_em) ||
      (env_w > 0 && !read_array(dir + "env.f32", env_rgb, (size_t)env_w * env_h * 3)) ||
      !read_array(dir + "camera.bin", cam_b, sizeof(vt_camera)) ||
      !read_array(dir + "settings.bin", set_b, sizeof(vt_render_settings))) {
    std::fprintf(stderr, "vt_cli: missing or mis-sized input in %s\n", dir.c_str());
    return 2;
  }
  std::vector<vt_material> palette((size_t)n_pal);
  for (int32_t i = 0; i < n_pal; ++i) {
    const float* r = &pal_f[(size_t)i * 8];
    palette[i].type = (int32_t)r[0];
    for (int c = 0; c < 3; ++c) { palette[i].emission[c] = r[1 + c]; palette[i].albedo[c] = r[4 + c]; }
    palette[i].roughness = r[7];
  }
  vt_camera cam;
  vt_render_settings set;
  std::memcpy(&cam, cam_b.data(), sizeof(cam));
  std::memcpy(&set, set_b.data(), sizeof(set));
  vt_context* ctx = nullptr;
  CHECK(vt_create(nullptr, &ctx));
  vt_scene* scene = nullptr;
  CHECK(vt_scene_create(ctx, rx, ry, rz, voxels.data(), palette.data(), n_pal, emissive.data(), n_em, 0, &scene));
  vt_env* env = nullptr;
  if (env_w > 0) CHECK(vt_env_create_image(ctx, env_rgb.data(), env_w, env_h, &env));
  vt_job* job = nullptr;
  CHECK(vt_job_create(ctx, scene, env, &cam, &set, w, h, &job));
  std::vector<float> rgba((size_t)w * h * 4);
  std::vector<int32_t> hits((size_t)w * h * 4);
  std::vector<uint64_t> counters(VT_DIAG_NUM_COUNTERS);
  CHECK(vt_diag_samples(job, sample, rgba.data(), hits.data(), counters.data()));
  if (!write_file(dir + "rgba.f32", rgba.data(), rgba.size() * sizeof(float)) ||
      !write_file(dir + "hits.i32", hits.data(), hits.size() * sizeof(int32_t)))
    return 2;
  vt_job_destroy(job);
  if (env) vt_env_destroy(env);
  vt_scene_destroy(scene);
  vt_destroy(ctx);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  int rc = 2;
  if (argc >= 2 && std::strcmp(argv[1], "vox") == 0) rc = cmd_vox(argc, argv);
  else if (argc >= 2 && std::strcmp(argv[1], "frame") == 0) rc = cmd_frame(argc, argv);
  if (rc == 2)
    std::fprintf(stderr, "usage: vt_cli vox FILE.vox OUT.pfm [WIDTH HEIGHT SPP]\n       vt_cli frame DIR\n");
  return rc;
}
