// A C++ host of the C ABI, as a reference user would write it: generate a
// seeded scene (parameters and camera read as raw structs from files, so
// that the Python test can render the same frame), create the scene, render
// one tensor-core frame into host buffers, and write rgb, depth and opacity
// as raw float32 to the output file.
//
//   render_host <params.bin> <camera.bin> <out.bin>
#include <cstdio>
#include <vector>

#include "snisr.h"

namespace {

template <class T>
bool read_struct(const char* path, T* out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  const size_t got = std::fread(out, 1, sizeof(T), f);
  std::fclose(f);
  return got == sizeof(T);
}

int fail(const char* what) {
  std::fprintf(stderr, "%s: %s\n", what, snisr_last_error_string());
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s params.bin camera.bin out.bin\n", argv[0]);
    return 2;
  }
  snisr_synth_params params{};
  snisr_camera cam{};
  if (!read_struct(argv[1], &params) || !read_struct(argv[2], &cam)) {
    std::fprintf(stderr, "cannot read the parameter files\n");
    return 2;
  }
  snisr_synth_scene* synth = nullptr;
  snisr_scene_desc desc{};
  if (snisr_synth_create(&params, &synth, &desc) != SNISR_OK) return fail("synth_create");
  desc.max_pixels = cam.width * cam.height;
  desc.max_samples_per_ray = 48;
  snisr_scene* scene = nullptr;
  if (snisr_scene_create(&desc, 0, &scene) != SNISR_OK) return fail("scene_create");
  const size_t n = (size_t)cam.width * cam.height;
  std::vector<float> rgb(3 * n), depth(n), opacity(n);
  if (snisr_render_host(scene, &cam, SNISR_FORM_TC, rgb.data(), depth.data(), opacity.data(), nullptr) != SNISR_OK)
    return fail("render_host");
  if (snisr_scene_check(scene, nullptr) != SNISR_OK) return fail("scene_check");
  FILE* f = std::fopen(argv[3], "wb");
  if (!f) return 2;
  std::fwrite(rgb.data(), sizeof(float), rgb.size(), f);
  std::fwrite(depth.data(), sizeof(float), depth.size(), f);
  std::fwrite(opacity.data(), sizeof(float), opacity.size(), f);
  std::fclose(f);
  snisr_scene_destroy(scene);
  snisr_synth_destroy(synth);
  std::printf("rendered %dx%d\n", cam.width, cam.height);
  return 0;
}
