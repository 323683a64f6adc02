// Test double for the reference's xromm::Volume (libautoscoper/src/Volume.hpp):
// the reference reads TIFF stacks; this builds the same object from memory.
// The "filename" is "mem:<address>:<width>:<height>:<depth>:<bps>".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include "Volume.hpp"

namespace xromm {
Volume::Volume(const std::string& filename)
  : name_(filename), width_(0), height_(0), depth_(0), bps_(0), data_(0), scaleX_(1.f), scaleY_(1.f), scaleZ_(1.f),
    flipX_(false), flipY_(false), flipZ_(false)
{
  unsigned long long addr = 0;
  size_t w = 0, h = 0, d = 0, b = 0;
  if (sscanf(filename.c_str(), "mem:%llx:%zu:%zu:%zu:%zu", &addr, &w, &h, &d, &b) != 5) return;
  width_ = w; height_ = h; depth_ = d; bps_ = b;
  size_t n = w * h * d * (b / 8);
  data_ = malloc(n);
  memcpy(data_, (const void*)addr, n);
}
Volume::~Volume() { free(data_); }
} // namespace xromm
