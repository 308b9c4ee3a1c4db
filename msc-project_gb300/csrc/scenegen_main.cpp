// msc-scenegen: writes one of the seeded synthetic scenes (YAML + OBJ files)
// without loading the CUDA library, for callers that only read scene files:
// the CPU renderer that the benchmark times beside the GPU, or a user preparing
// inputs on a machine without a GPU.  Same generator as msc_generate_scene().
//
//   msc-scenegen <config> <seed> <scale> <out_dir>    prints the YAML path
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>

namespace mscg {
bool generate_scene(int config, uint32_t seed, double scale, const std::string& dir, std::string* yaml,
                    std::string* err);
}

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: msc-scenegen <config 0|1|2|100> <seed> <scale in (0,1]> <out_dir>\n");
    return 2;
  }
  std::string yaml, err;
  const int config = std::atoi(argv[1]);
  const uint32_t seed = (uint32_t)std::strtoul(argv[2], nullptr, 10);
  const double scale = std::strtod(argv[3], nullptr);
  if (!mscg::generate_scene(config, seed, scale, argv[4], &yaml, &err)) {
    std::fprintf(stderr, "msc-scenegen: %s\n", err.c_str());
    return 1;
  }
  std::printf("%s\n", yaml.c_str());
  return 0;
}
