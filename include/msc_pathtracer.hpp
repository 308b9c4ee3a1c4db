// msc_pathtracer.hpp - header-only C++ drop-in for the reference engine class
// msc::Pathtracer (include/core/Pathtracer.h:36-110 of joshbainbridge/msc-project),
// implemented over the C ABI of msc_gpu.h.  Same names, same argument meaning:
//   Pathtracer(const std::string& scene_yaml)   // throws std::runtime_error on a bad scene
//   void image(float** pixels, int* width, int* height)
//   void clear(); bool active(); void terminate(); int process();
// The reference's constructor throws (yaml-cpp exceptions) on malformed input;
// this one throws std::runtime_error with the loader's message.
#ifndef MSC_PATHTRACER_HPP_
#define MSC_PATHTRACER_HPP_

#include <stdexcept>
#include <string>

#include "msc_gpu.h"

namespace msc {

class Pathtracer {
 public:
  explicit Pathtracer(const std::string& filename) {
    if (msc_create(filename.c_str(), &handle_) != MSC_OK) throw std::runtime_error(msc_last_error(nullptr));
  }
  ~Pathtracer() {
    if (handle_) msc_destroy(handle_);
  }
  Pathtracer(const Pathtracer&) = delete;
  Pathtracer& operator=(const Pathtracer&) = delete;

  // Accumulated image, row-major, 3 floats per pixel; owned by the object.
  void image(float** pixels, int* width, int* height) {
    const float* p = nullptr;
    check(msc_image(handle_, &p, width, height));
    *pixels = const_cast<float*>(p);
  }
  void clear() { check(msc_clear(handle_)); }
  bool active() {
    int a = 0;
    check(msc_active(handle_, &a));
    return a != 0;
  }
  void terminate() { check(msc_terminate(handle_)); }
  int process() {
    int it = 0;
    check(msc_process(handle_, &it));
    return it;
  }

  msc_handle* handle() { return handle_; }

 private:
  void check(int rc) {
    if (rc != MSC_OK) throw std::runtime_error(msc_last_error(handle_));
  }
  msc_handle* handle_ = nullptr;
};

}  // namespace msc

#endif  // MSC_PATHTRACER_HPP_
