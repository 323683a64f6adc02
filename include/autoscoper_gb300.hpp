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
//   View                 libautoscoper/src/View.hpp:68-154 (CUDA backend,
//                        without the OpenGL pixel-buffer members)
#ifndef AUTOSCOPER_GB300_HPP
#define AUTOSCOPER_GB300_HPP

#include <algorithm>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "autoscoper_gb300.h"

namespace xromm {
// The caller's camera class (libautoscoper/src/Camera.hpp); a View only
// keeps a pointer to it, as the reference's does.
class Camera;

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

// ---- View (View.cpp:81-555, CUDA backend) ----
// One camera's renderers and filter lists, with the view's device scratch
// (maxWidth x maxHeight floats per buffer, allocated on first use as
// View::init does).  The OpenGL members (renderDrr(pbo), render(pbo)) are
// left out: render() writes the RGB composite into a device buffer instead.
class View
{
public:
  explicit View(Camera& camera) : camera_(&camera), radRenderer_(new RadRenderer()),
                                  backgroundRenderer_(new BackgroundRenderer())
  {
  }
  ~View()
  {
    for (Filter* f : drrFilters_) delete f;
    for (Filter* f : radFilters_) delete f;
    for (float* b : drrBuffer_) asc_free(b);
    for (float* b : {filterBuffer_, drrBufferMerged_, drrFilterBuffer_, radBuffer_, radFilterBuffer_,
                     backgroundmask_, drr_mask_})
      asc_free(b);
    for (RayCaster* r : drrRenderer_) delete r;
    delete radRenderer_;
    delete backgroundRenderer_;
  }
  View(const View&) = delete;
  View& operator=(const View&) = delete;

  Camera* camera() { return camera_; }
  const Camera* camera() const { return camera_; }
  RayCaster* drrRenderer(int idx) { return drrRenderer_[idx]; }
  const RayCaster* drrRenderer(int idx) const { return drrRenderer_[idx]; }
  RadRenderer* radRenderer() { return radRenderer_; }
  const RadRenderer* radRenderer() const { return radRenderer_; }
  std::vector<Filter*>& drrFilters() { return drrFilters_; }
  const std::vector<Filter*>& drrFilters() const { return drrFilters_; }
  std::vector<Filter*>& radFilters() { return radFilters_; }
  const std::vector<Filter*>& radFilters() const { return radFilters_; }
  BackgroundRenderer* backgroundRenderer() { return backgroundRenderer_; }
  unsigned int nbDrrRenderer() const { return (unsigned)drrRenderer_.size(); }

  void addDrrRenderer()
  {
    drrRenderer_.push_back(new RayCaster());
    drrBuffer_.push_back(nullptr);
  }

  // RadRenderer into the view's buffer, then the radiograph filters (View.cpp:147-169)
  void renderRad(float* buffer, unsigned width, unsigned height)
  {
    init();
    clamp_size(width, height, "renderRad");
    radRenderer_->render(radBuffer_, width, height);
    filter(radFilters_, radBuffer_, buffer, width, height);
  }

  // The background mask, or nothing while the threshold is negative (View.cpp:171-194)
  void renderBackground(float* buffer, unsigned width, unsigned height)
  {
    if (backgroundThreshold_ < 0.0f) return;
    init();
    clamp_size(width, height, "renderBackground");
    backgroundRenderer_->render(buffer, width, height, backgroundThreshold_);
  }

  // mask = filtered DRR != 0 (View.cpp:196-199)
  void renderDRRMask(float* in_buffer, float* out_buffer, unsigned width, unsigned height)
  {
    drr_background(in_buffer, out_buffer, width, height);
  }

  // Every volume's DRR, merged (sum clamped to 1), then the DRR filters (View.cpp:201-231)
  void renderDrr(float* buffer, unsigned width, unsigned height)
  {
    init();
    clamp_size(width, height, "renderDrr");
    asc_check(asc_memset(drrBufferMerged_, 0, (size_t)width * height * sizeof(float), nullptr), "View::renderDrr");
    for (size_t i = 0; i < drrRenderer_.size(); ++i) {
      drrRenderer_[i]->render(drr_buffer(i), width, height);
      merge(drrBufferMerged_, drrBuffer_[i], drrBufferMerged_, width, height);
    }
    filter(drrFilters_, drrBufferMerged_, buffer, width, height);
  }

  // One volume's DRR, then the DRR filters (View.cpp:233-256)
  void renderDrrSingle(int volume, float* buffer, unsigned width, unsigned height)
  {
    init();
    clamp_size(width, height, "renderDrrSingle");
    drrRenderer_[volume]->render(drr_buffer(volume), width, height);
    filter(drrFilters_, drrBuffer_[volume], buffer, width, height);
  }

  // The display composite (View.cpp:352-380) into a device buffer of
  // 3 x width x height floats: R = DRR, G = mask (DRR + rad) / 2, B = rad.
  void render(float* rgb, unsigned width, unsigned height)
  {
    init();
    clamp_size(width, height, "render");
    const size_t bytes = (size_t)width * height * sizeof(float);
    if (drr_enabled)
      renderDrr(drrFilterBuffer_, width, height);
    else
      asc_check(asc_memset(drrFilterBuffer_, 0, bytes, nullptr), "View::render");
    if (rad_enabled)
      renderRad(radFilterBuffer_, width, height);
    else
      asc_check(asc_memset(radFilterBuffer_, 0, bytes, nullptr), "View::render");
    renderBackground(backgroundmask_, width, height);
    renderDRRMask(drrFilterBuffer_, drr_mask_, width, height);
    composite(drrFilterBuffer_, radFilterBuffer_, backgroundmask_, drr_mask_, rgb, width, height);
  }

  // The merged, filtered DRR as an ASCII PGM, 255 (1 - value), rows bottom
  // up (View.cpp:258-334)
  void saveImage(const std::string& filename, int width, int height)
  {
    unsigned w = (unsigned)width, h = (unsigned)height;
    init();
    clamp_size(w, h, "saveImage");
    renderDrr(drrFilterBuffer_, w, h);
    std::vector<float> img((size_t)w * h);
    asc_check(asc_memcpy_d2h(img.data(), drrFilterBuffer_, img.size() * sizeof(float), nullptr), "View::saveImage");
    std::ofstream file(filename.c_str(), std::ios::out);
    file << "P2" << std::endl << w << " " << h << std::endl << 255 << std::endl;
    for (unsigned y = 0; y < h; ++y)
      for (unsigned x = 0; x < w; ++x)
        file << (int)(unsigned char)(int)(255 * (1.0 - img[(size_t)(h - y - 1) * w + x])) << " ";
  }

  // BackgroundRenderer::set_back with a host float image (View.cpp:423-426)
  void updateBackground(const float* buffer, unsigned width, unsigned height)
  {
    backgroundRenderer_->set_back(buffer, width, height);
  }
  void setBackgroundThreshold(float threshold) { backgroundThreshold_ = threshold; }

  bool drr_enabled = true;
  bool rad_enabled = true;

private:
  // View::init (View.cpp:428-445): the view's scratch, masks filled with 1
  void init()
  {
    if (filterBuffer_) return;
    const size_t bytes = maxWidth_ * maxHeight_ * sizeof(float);
    for (float** p : {&filterBuffer_, &drrBufferMerged_, &drrFilterBuffer_, &radBuffer_, &radFilterBuffer_,
                      &backgroundmask_, &drr_mask_})
      cudaMallocWrap(*p, bytes);
    fill(backgroundmask_, (unsigned)(maxWidth_ * maxHeight_), 1.0f);
    fill(drr_mask_, (unsigned)(maxWidth_ * maxHeight_), 1.0f);
  }

  // A volume's DRR buffer (a renderer added after init gets one on first use)
  float* drr_buffer(size_t i)
  {
    if (!drrBuffer_[i]) cudaMallocWrap(drrBuffer_[i], maxWidth_ * maxHeight_ * sizeof(float));
    return drrBuffer_[i];
  }

  void clamp_size(unsigned& width, unsigned& height, const char* who) const
  {
    if (width > maxWidth_ || height > maxHeight_)
      std::cerr << "View::" << who << "(): ERROR: Buffer too large." << std::endl;
    width = std::min<unsigned>(width, (unsigned)maxWidth_);
    height = std::min<unsigned>(height, (unsigned)maxHeight_);
  }

  // View::filter (View.cpp:475-518): the enabled filters in order, ping-pong
  // between `output` and the view's filter buffer so that the last one
  // writes `output`; a disabled filter copies, an empty list copies.
  void filter(const std::vector<Filter*>& filters, const float* input, float* output, unsigned width,
              unsigned height)
  {
    const size_t bytes = (size_t)width * height * sizeof(float);
    if (filters.empty()) {
      asc_check(asc_memcpy_d2d(output, input, bytes, nullptr), "View::filter");
      return;
    }
    float* b1 = filters.size() % 2 ? output : filterBuffer_;
    float* b2 = filters.size() % 2 ? filterBuffer_ : output;
    if (filters[0]->enabled())
      filters[0]->apply(input, b1, (int)width, (int)height);
    else
      asc_check(asc_memcpy_d2d(b1, input, bytes, nullptr), "View::filter");
    for (size_t i = 1; i < filters.size(); ++i) {
      if (filters[i]->enabled())
        filters[i]->apply(b1, b2, (int)width, (int)height);
      else
        asc_check(asc_memcpy_d2d(b2, b1, bytes, nullptr), "View::filter");
      std::swap(b1, b2);
    }
  }

  Camera* camera_;
  std::vector<RayCaster*> drrRenderer_;
  RadRenderer* radRenderer_;
  BackgroundRenderer* backgroundRenderer_;
  std::vector<Filter*> drrFilters_, radFilters_;
  size_t maxWidth_ = 3000, maxHeight_ = 3000;
  std::vector<float*> drrBuffer_;
  float* drrBufferMerged_ = nullptr;
  float* drrFilterBuffer_ = nullptr;
  float* radBuffer_ = nullptr;
  float* radFilterBuffer_ = nullptr;
  float* filterBuffer_ = nullptr;
  float* backgroundmask_ = nullptr;
  float* drr_mask_ = nullptr;
  float backgroundThreshold_ = -1.0f;
};

}  // namespace gpu
}  // namespace xromm

#endif
