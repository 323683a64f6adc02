// One view of Tracker::trackFrame (Tracker.cpp:603-770) as the reference
// writes it, through xromm::gpu::View (View.hpp:68-154): the view's DRR
// renderer, radiograph renderer, background renderer and filter lists set up
// as Tracker::load does (Tracker.cpp:244-335), then per pose renderDrrSingle,
// renderRad, renderBackground, renderDRRMask, the three multiplies and ncc.
// Compiled against autoscoper_gb300.hpp: the drop-in check for View.
//
// usage: dropin_view <spec.txt> <out.bin>
// spec: W H D bps sx sy sz volume.raw | imv[16] | vp[4] | step intensity cutoff |
//       RW RH rbps rad.raw | ip[4] | w h | BW BH bg.raw (BW = 0: none) threshold |
//       n_drr (kind enabled p0 p1 p2)... | n_rad (kind enabled p0 p1 p2)...
// out:  w*h float DRR (masked), w*h float radiograph (masked), w*h float mask,
//       double 1 - NCC
#include <fstream>
#include <iostream>
#include <vector>

#include "autoscoper_gb300.hpp"

namespace xromm {
// Stands in for libautoscoper's Camera (Camera.hpp): a View only keeps it.
class Camera
{
};
}  // namespace xromm

using namespace xromm::gpu;

static std::vector<char> slurp(const std::string& p)
{
  std::ifstream f(p, std::ios::binary);
  return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

// A filter of the reference's kinds (Filter.hpp:59-66) with its setters.
static Filter* make_filter(std::istream& in)
{
  int kind, enabled;
  float p0, p1, p2;
  in >> kind >> enabled >> p0 >> p1 >> p2;
  Filter* f = nullptr;
  if (kind == Filter::XROMM_GPU_CONTRAST_FILTER) {
    ContrastFilter* c = new ContrastFilter();
    c->set_alpha(p0);
    c->set_beta(p1);
    f = c;
  } else if (kind == Filter::XROMM_GPU_SOBEL_FILTER) {
    SobelFilter* s = new SobelFilter();
    s->setScale(p0);
    s->setBlend(p1);
    f = s;
  } else if (kind == Filter::XROMM_GPU_GAUSSIAN_FILTER) {
    GaussianFilter* g = new GaussianFilter();
    g->set_radius(p0);
    f = g;
  } else if (kind == Filter::XROMM_GPU_SHARPEN_FILTER) {
    SharpenFilter* s = new SharpenFilter();
    s->set_radius(p0);
    s->set_contrast(p1);
    s->set_threshold(p2);
    f = s;
  } else {
    throw std::runtime_error("unknown filter kind");
  }
  f->set_enabled(enabled != 0);
  return f;
}

int main(int argc, char** argv)
{
  if (argc != 3) return 2;
  std::ifstream in(argv[1]);
  int W, H, D, bps, RW, RH, rbps, w, h, BW, BH;
  double scale[3], imv[16];
  float vp[4], ip[4], step, intensity, cutoff, threshold;
  std::string vpath, rpath, bpath;
  in >> W >> H >> D >> bps >> scale[0] >> scale[1] >> scale[2] >> vpath;
  for (double& x : imv) in >> x;
  for (float& x : vp) in >> x;
  in >> step >> intensity >> cutoff >> RW >> RH >> rbps >> rpath;
  for (float& x : ip) in >> x;
  in >> w >> h >> BW >> BH >> bpath >> threshold;
  if (!in) return 3;
  std::vector<char> vol = slurp(vpath), rad = slurp(rpath), bg;
  if (BW > 0) bg = slurp(bpath);
  int flip[3] = {0, 0, 0};
  try {
    xromm::Camera camera;
    VolumeDescription vd(vol.data(), W, H, D, bps, scale, flip);
    View view(camera);
    // Tracker::load: one DRR renderer per volume, the radiograph, the
    // background image and threshold, the filter lists (Tracker.cpp:244-335)
    view.addDrrRenderer();
    view.drrRenderer(0)->setVolume(vd);
    view.drrRenderer(0)->setSampleDistance(step);
    view.drrRenderer(0)->setRayIntensity(intensity);
    view.drrRenderer(0)->setCutoff(cutoff);
    view.radRenderer()->set_rad(rad.data(), RW, RH, rbps);
    view.radRenderer()->set_image_plane(ip[0], ip[1], ip[2], ip[3]);
    view.backgroundRenderer()->set_image_plane(ip[0], ip[1], ip[2], ip[3]);
    if (BW > 0) view.updateBackground((const float*)bg.data(), BW, BH);
    view.setBackgroundThreshold(threshold);
    int n;
    in >> n;
    for (int i = 0; i < n; ++i) view.drrFilters().push_back(make_filter(in));
    in >> n;
    for (int i = 0; i < n; ++i) view.radFilters().push_back(make_filter(in));
    if (!in) return 3;
    const size_t px = (size_t)w * h;
    float *rendered_drr, *rendered_rad, *drr_mask, *background_mask;
    for (float** p : {&rendered_drr, &rendered_rad, &drr_mask, &background_mask}) cudaMallocWrap(*p, px * sizeof(float));
    fill(background_mask, (unsigned)px, 1.0f);  // Tracker.cpp:298
    ncc_init((unsigned)px);
    // trackFrame, one view (Tracker.cpp:603-770)
    view.drrRenderer(0)->setInvModelView(imv);
    view.drrRenderer(0)->setViewport(vp[0], vp[1], vp[2], vp[3]);
    view.radRenderer()->set_viewport(vp[0], vp[1], vp[2], vp[3]);
    view.renderDrrSingle(0, rendered_drr, w, h);
    view.renderRad(rendered_rad, w, h);
    view.backgroundRenderer()->set_viewport(vp[0], vp[1], vp[2], vp[3]);
    view.renderBackground(background_mask, w, h);
    view.renderDRRMask(rendered_drr, drr_mask, w, h);
    multiply(background_mask, drr_mask, drr_mask, w, h);
    multiply(rendered_rad, drr_mask, rendered_rad, w, h);
    multiply(rendered_drr, drr_mask, rendered_drr, w, h);
    double cost = 1.0 - ncc(rendered_drr, rendered_rad, drr_mask, (unsigned)px);
    std::vector<float> a(px), b(px), m(px);
    asc_check(asc_memcpy_d2h(a.data(), rendered_drr, px * sizeof(float), nullptr), "copy");
    asc_check(asc_memcpy_d2h(b.data(), rendered_rad, px * sizeof(float), nullptr), "copy");
    asc_check(asc_memcpy_d2h(m.data(), drr_mask, px * sizeof(float), nullptr), "copy");
    std::ofstream out(argv[2], std::ios::binary);
    out.write((const char*)a.data(), px * sizeof(float));
    out.write((const char*)b.data(), px * sizeof(float));
    out.write((const char*)m.data(), px * sizeof(float));
    out.write((const char*)&cost, sizeof cost);
    for (float* p : {rendered_drr, rendered_rad, drr_mask, background_mask}) asc_free(p);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
