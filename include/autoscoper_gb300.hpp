// autoscoper_gb300.hpp -- the reference's C++ operator interfaces
// (namespace xromm::gpu, CUDA backend) as header-only classes over the C ABI
// in autoscoper_gb300.h.  Code written against libautoscoper/src/gpu/cuda
// (Tracker, View, the GUI widgets) compiles against these unchanged; errors
// that the reference turned into exit() raise std::runtime_error instead.
//
//   RayCaster            libautoscoper/src/gpu/cuda/RayCaster.hpp:51-104
//   RadRenderer          libautoscoper/src/gpu/cuda/RadRenderer.hpp:52-85
//   BackgroundRenderer   libautoscoper/src/gpu/cuda/BackgroundRenderer.hpp:52-79
//   Filter + 4 filters   libautoscoper/src/Filter.hpp:56-93, gpu/cuda/*Filter.hpp
//   VolumeDescription    libautoscoper/src/VolumeDescription.hpp:56-84
//   ncc/hdist/multiply/merge/composite/fill/drr_background/cudaMallocWrap
//                        gpu/cuda/*_kernels.h, gpu/cuda/CudaWrap.hpp
#ifndef AUTOSCOPER_GB300_HPP
#define AUTOSCOPER_GB300_HPP

#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "autoscoper_gb300.h"

namespace xromm {
namespace gpu {

inline void asc_check(int status, const char* what)
{
  if (status != ASC_OK) {
    std::ostringstream s;
    s << what << ": " << asc_status_string(status);
    const char* e = asc_last_error();
    if (e && *e) s << " (" << e << ")";
    throw std::runtime_error(s.str());
  }
}

// ---- VolumeDescription (VolumeDescription.cpp:152-305) ----
class VolumeDescription
{
public:
  // Any type with xromm::Volume's accessors (Volume.hpp:56-110).
  template <class V>
  explicit VolumeDescription(const V& volume, int storage = ASC_STORE_U16)
  {
    double scale[3] = {volume.scaleX(), volume.scaleY(), volume.scaleZ()};
    int flip[3] = {volume.flipX() ? 1 : 0, volume.flipY() ? 1 : 0, volume.flipZ() ? 1 : 0};
    init(volume.data(), (int)volume.width(), (int)volume.height(), (int)volume.depth(), (int)volume.bps(), scale,
         flip, storage);
  }
  VolumeDescription(const void* data, int width, int height, int depth, int bps, const double scale[3],
                    const int flip[3], int storage = ASC_STORE_U16)
  {
    init(data, width, height, depth, bps, scale, flip, storage);
  }
  ~VolumeDescription() { asc_volume_destroy(vol_); }
  VolumeDescription(const VolumeDescription&) = delete;
  VolumeDescription& operator=(const VolumeDescription&) = delete;

  const float* invScale() const { return invScale_; }
  const float* invTrans() const { return invTrans_; }
  const double* transCenter() const { return transCenter_; }
  float minValue() const { return minValue_; }
  float maxValue() const { return maxValue_; }
  asc_volume image() const { return vol_; }

private:
  void init(const void* data, int w, int h, int d, int bps, const double* scale, const int* flip, int storage)
  {
    asc_check(asc_volume_create(data, w, h, d, bps, scale, flip, storage, &vol_), "VolumeDescription");
    asc_check(asc_volume_info(vol_, invScale_, invTrans_, transCenter_, &minValue_, &maxValue_, dims_),
              "VolumeDescription");
  }
  asc_volume vol_ = nullptr;
  float invScale_[3], invTrans_[3], minValue_ = 0, maxValue_ = 1;
  double transCenter_[3];
  int dims_[3];
};

// ---- RayCaster (RayCaster.cpp:57-143) ----
class RayCaster
{
public:
  RayCaster()
  {
    static int count = 0;
    name_ = "DrrRenderer" + std::to_string(++count);
  }
  void setVolume(VolumeDescription& volume) { volume_ = &volume; }
  void setInvModelView(const double* invModelView)
  {
    if (!volume_) throw std::runtime_error("RayCaster: ERROR: Unable to calculate matrix.");
    for (int i = 0; i < 16; ++i) imv_[i] = invModelView[i];
  }
  void setViewport(float x, float y, float width, float height)
  {
    viewport_[0] = x; viewport_[1] = y; viewport_[2] = width; viewport_[3] = height;
  }
  void render(float* buffer, size_t width, size_t height, void* stream = nullptr)
  {
    if (!volume_) return;  // the reference prints a warning and returns
    asc_check(asc_raycast(volume_->image(), imv_, viewport_, sampleDistance_, rayIntensity_, cutoff_, visible_ ? 1 : 0,
                          buffer, (int)width, (int)height, stream),
              "RayCaster::render");
  }
  float getSampleDistance() const { return sampleDistance_; }
  void setSampleDistance(float d) { sampleDistance_ = d; }
  float getRayIntensity() const { return rayIntensity_; }
  void setRayIntensity(float i) { rayIntensity_ = i; }
  float getCutoff() const { return cutoff_; }
  float getMinCutoff() const { return volume_->minValue(); }
  float getMaxCutoff() const { return volume_->maxValue(); }
  void setCutoff(float c) { cutoff_ = c; }
  const std::string& getName() const { return name_; }
  void setName(const std::string& n) { name_ = n; }
  void setVisible(bool v) { visible_ = v; }

private:
  VolumeDescription* volume_ = nullptr;
  double imv_[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  float viewport_[4] = {-1.0f, -1.0f, 2.0f, 2.0f};
  float sampleDistance_ = 0.5f, rayIntensity_ = 10.0f, cutoff_ = 0.0f;
  bool visible_ = true;
  std::string name_;
};

// ---- RadRenderer (RadRenderer.cpp:54-142) ----
class RadRenderer
{
public:
  RadRenderer()
  {
    static int count = 0;
    name_ = "RadRenderer" + std::to_string(++count);
  }
  ~RadRenderer()
  {
    if (img_) asc_image_destroy(img_);
  }
  void set_rad(const void* data, size_t width, size_t height, size_t bps)
  {
    if (img_ && (size_t)w_ == width && (size_t)h_ == height && (size_t)bps_ == bps) {
      asc_check(asc_image_update(img_, data, nullptr), "RadRenderer::set_rad");
      return;
    }
    if (img_) asc_image_destroy(img_);
    img_ = nullptr;
    asc_check(asc_image_create(data, (int)width, (int)height, (int)bps, &img_), "RadRenderer::set_rad");
    w_ = (int)width; h_ = (int)height; bps_ = (int)bps;
  }
  void set_image_plane(float x, float y, float width, float height)
  {
    ip_[0] = x; ip_[1] = y; ip_[2] = width; ip_[3] = height;
  }
  void set_viewport(float x, float y, float width, float height)
  {
    vp_[0] = x; vp_[1] = y; vp_[2] = width; vp_[3] = height;
  }
  void render(float* buffer, size_t width, size_t height, void* stream = nullptr) const
  {
    asc_check(asc_rad_render(img_, ip_, vp_, buffer, (int)width, (int)height, stream), "RadRenderer::render");
  }
  const std::string& getName() const { return name_; }
  void setName(const std::string& n) { name_ = n; }
  asc_image image() const { return img_; }

private:
  asc_image img_ = nullptr;
  int w_ = 0, h_ = 0, bps_ = 0;
  float ip_[4] = {-1.0f, -1.0f, 2.0f, 2.0f}, vp_[4] = {-1.0f, -1.0f, 2.0f, 2.0f};
  std::string name_;
};

// ---- BackgroundRenderer (BackgroundRenderer.cpp:54-124) ----
class BackgroundRenderer
{
public:
  ~BackgroundRenderer()
  {
    if (img_) asc_image_destroy(img_);
  }
  void set_back(const void* data, size_t width, size_t height)
  {
    if (img_) asc_image_destroy(img_);
    img_ = nullptr;
    asc_check(asc_image_create(data, (int)width, (int)height, 32, &img_), "BackgroundRenderer::set_back");
  }
  void set_image_plane(float x, float y, float width, float height)
  {
    ip_[0] = x; ip_[1] = y; ip_[2] = width; ip_[3] = height;
  }
  void set_viewport(float x, float y, float width, float height)
  {
    vp_[0] = x; vp_[1] = y; vp_[2] = width; vp_[3] = height;
  }
  void render(float* buffer, size_t width, size_t height, float threshold, void* stream = nullptr) const
  {
    asc_check(asc_background_render(img_, ip_, vp_, threshold, buffer, (int)width, (int)height, stream),
              "BackgroundRenderer::render");
  }

private:
  asc_image img_ = nullptr;
  float ip_[4] = {-1.0f, -1.0f, 2.0f, 2.0f}, vp_[4] = {-1.0f, -1.0f, 2.0f, 2.0f};
};

// ---- filters (Filter.hpp:56-93) ----
class Filter
{
public:
  enum { XROMM_GPU_CONTRAST_FILTER, XROMM_GPU_SOBEL_FILTER, XROMM_GPU_MEDIAN_FILTER, XROMM_GPU_GAUSSIAN_FILTER,
         XROMM_GPU_SHARPEN_FILTER };
  Filter(int type, const std::string& name) : type_(type), name_(name) {}
  virtual ~Filter() {}
  virtual void apply(const float* input, float* output, int width, int height) = 0;
  int type() const { return type_; }
  const std::string& name() const { return name_; }
  void set_name(const std::string& n) { name_ = n; }
  bool enabled() const { return enabled_; }
  void set_enabled(bool e) { enabled_ = e; }

protected:
  int type_;
  std::string name_;
  bool enabled_ = true;
};

class SobelFilter : public Filter
{
public:
  SobelFilter() : Filter(XROMM_GPU_SOBEL_FILTER, "SobelFilter") {}
  void apply(const float* in, float* out, int w, int h) override
  {
    asc_check(asc_sobel(in, out, w, h, scale_, blend_, nullptr), "SobelFilter::apply");
  }
  float getScale() const { return scale_; }
  void setScale(float s) { scale_ = s; }
  float getBlend() const { return blend_; }
  void setBlend(float b) { blend_ = b; }

private:
  float scale_ = 1.0f, blend_ = 0.5f;
};

class ContrastFilter : public Filter
{
public:
  ContrastFilter() : Filter(XROMM_GPU_CONTRAST_FILTER, "ContrastFilter") {}
  void apply(const float* in, float* out, int w, int h) override
  {
    asc_check(asc_contrast(in, out, w, h, alpha_, beta_, size_, nullptr), "ContrastFilter::apply");
  }
  float alpha() const { return alpha_; }
  void set_alpha(float a) { alpha_ = a; }
  float beta() const { return beta_; }
  void set_beta(float b) { beta_ = b; }

private:
  float alpha_ = 1.0f, beta_ = 1.0f;
  int size_ = 3;
};

class GaussianFilter : public Filter
{
public:
  GaussianFilter() : Filter(XROMM_GPU_GAUSSIAN_FILTER, "GaussianFilter") {}
  void apply(const float* in, float* out, int w, int h) override
  {
    asc_check(asc_gaussian(in, out, w, h, radius_, nullptr), "GaussianFilter::apply");
  }
  float radius() const { return radius_; }
  void set_radius(float r) { radius_ = r < 0 ? 0 : r; }

private:
  float radius_ = 1.0f;
};

class SharpenFilter : public Filter
{
public:
  SharpenFilter() : Filter(XROMM_GPU_SHARPEN_FILTER, "SharpenFilter") {}
  void apply(const float* in, float* out, int w, int h) override
  {
    asc_check(asc_sharpen(in, out, w, h, radius_, contrast_, threshold_, nullptr), "SharpenFilter::apply");
  }
  float radius() const { return radius_; }
  void set_radius(float r) { radius_ = r < 0 ? 0 : r; }
  float contrast() const { return contrast_; }
  void set_contrast(float c) { contrast_ = c < 1 ? 1 : c; }
  float threshold() const { return threshold_; }
  void set_threshold(float t) { threshold_ = t; }

private:
  float radius_ = 1.0f, contrast_ = 1.0f, threshold_ = 0.0f;
};

// ---- free functions (gpu/cuda/*_kernels.h, CudaWrap.hpp) ----
inline void cudaMallocWrap(float*& p, size_t bytes) { asc_check(asc_malloc((void**)&p, bytes), "cudaMallocWrap"); }
inline void ncc_init(unsigned max_n, unsigned = 256) { asc_check(asc_ncc_init(max_n), "ncc_init"); }
inline void ncc_deinit() { asc_ncc_init(0); }
inline float ncc(float* f, float* g, float* mask, unsigned n, int coverage = ASC_SUM_TREE)
{
  double r = 0;
  asc_check(asc_ncc_host(f, g, mask, n, coverage, &r, nullptr), "ncc");
  return (float)r;
}
inline void hdist_init(unsigned max_n, unsigned = 256) { asc_check(asc_ncc_init(max_n), "hdist_init"); }
inline void hdist_deinit() {}
inline float hdist(float* f, float* g, float* mask, unsigned n, int coverage = ASC_SUM_TREE)
{
  double r = 0;
  asc_check(asc_hdist_host(f, g, mask, n, coverage, &r, nullptr), "hdist");
  return (float)r;
}
inline void multiply(float* a, float* b, float* d, size_t w, size_t h)
{
  asc_check(asc_multiply(a, b, d, (int)w, (int)h, nullptr), "multiply");
}
inline void merge(float* a, float* b, float* d, size_t w, size_t h)
{
  asc_check(asc_merge(a, b, d, (int)w, (int)h, nullptr), "merge");
}
inline void composite(float* a, float* b, float* c, float* e, float* d, size_t w, size_t h)
{
  asc_check(asc_composite(a, b, c, e, d, (int)w, (int)h, nullptr), "composite");
}
inline void fill(float* p, unsigned size, float val) { asc_check(asc_fill(p, size, val, nullptr), "fill"); }
inline void drr_background(float* src, float* dst, size_t w, size_t h)
{
  asc_check(asc_drr_background(src, dst, (int)w, (int)h, nullptr), "drr_background");
}

}  // namespace gpu
}  // namespace xromm

#endif
