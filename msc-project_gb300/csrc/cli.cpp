// msc-gpu: headless command line equivalent of the reference's batch mode
// (src/main.cpp:18-81 options, :195-215 render once and write an RGBA half
// EXR).  The interactive OpenGL window of the reference (src/framebuffer/) is
// a display only and is not part of this build.
//
//   msc-gpu [-o out.exr|out.pfm] [-n iterations] [--mean] scene.yaml
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>

#include "msc_gpu.h"

static void usage(FILE* f) {
  fprintf(f, "usage: msc-gpu [options] scene_file.yaml\noptions:\n"
             "  -h [ --help ]          produce help message\n"
             "  -o [ --output ] arg    output as file (.exr or .pfm)\n"
             "  -n [ --iterations ] N  render N iterations (default 1)\n"
             "  --mean                 divide the accumulated image by the iteration count\n");
}

int main(int argc, char** argv) {
  std::string input, output = "output.exr";
  int iterations = 1;
  bool mean = false;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-h" || a == "--help") { usage(stdout); return EXIT_SUCCESS; }
    if ((a == "-o" || a == "--output") && i + 1 < argc) { output = argv[++i]; continue; }
    if ((a == "-n" || a == "--iterations") && i + 1 < argc) { iterations = atoi(argv[++i]); continue; }
    if (a == "--mean") { mean = true; continue; }
    if (!a.empty() && a[0] == '-') {
      fprintf(stderr, "error: unknown option %s\n\n", a.c_str());
      usage(stderr);
      return EXIT_FAILURE;
    }
    input = a;
  }
  struct stat st;
  if (input.empty()) {
    fprintf(stderr, "error: a scene file is required but missing\n\n");
    usage(stderr);
    return EXIT_FAILURE;
  }
  if (stat(input.c_str(), &st) != 0) {
    fprintf(stderr, "error: the scene file does not exist\n\n");
    usage(stderr);
    return EXIT_FAILURE;
  }
  msc_handle* h = nullptr;
  if (msc_create(input.c_str(), &h) != MSC_OK) {
    fprintf(stderr, "error: %s\n", msc_last_error(nullptr));
    return EXIT_FAILURE;
  }
  int it = 0;
  for (int k = 0; k < iterations; ++k) {
    if (msc_process(h, &it) != MSC_OK) {
      fprintf(stderr, "error: %s\n", msc_last_error(h));
      msc_destroy(h);
      return EXIT_FAILURE;
    }
    msc_stats s;
    msc_get_stats(h, &s);
    printf("Iteration %d is complete (%.1f ms, %.1f Mrays/s).\n", it, s.process_ms,
           (double)(s.closest_queries + s.shadow_queries) / (s.process_ms * 1e3));
  }
  if (msc_save_image(h, output.c_str(), mean ? 1 : 0) != MSC_OK) {
    fprintf(stderr, "error: %s\n", msc_last_error(h));
    msc_destroy(h);
    return EXIT_FAILURE;
  }
  printf("Output file named \"%s\" written.\n", output.c_str());
  msc_destroy(h);
  return EXIT_SUCCESS;
}
