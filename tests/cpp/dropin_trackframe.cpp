// One view of Tracker::trackFrame (Tracker.cpp:603-770) written against the
// reference's C++ operator classes, compiled against autoscoper_gb300.hpp:
// the drop-in check that code using xromm::gpu builds and runs unchanged.
//
// usage: dropin_trackframe <spec.txt> <out.bin>
// spec: W H D bps sx sy sz volume.raw | imv[16] | vp[4] | step intensity cutoff |
//       RW RH rbps rad.raw | ip[4] | w h | sobel_scale sobel_blend
// out:  w*h float DRR (masked), w*h float radiograph (masked), double 1-NCC
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "autoscoper_gb300.hpp"

using namespace xromm::gpu;

static std::vector<char> slurp(const std::string& p)
{
  std::ifstream f(p, std::ios::binary);
  return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

int main(int argc, char** argv)
{
  if (argc != 3) return 2;
  std::ifstream in(argv[1]);
  int W, H, D, bps, RW, RH, rbps, w, h;
  double scale[3], imv[16];
  float vp[4], ip[4], step, intensity, cutoff, sscale, sblend;
  std::string vpath, rpath;
  in >> W >> H >> D >> bps >> scale[0] >> scale[1] >> scale[2] >> vpath;
  for (double& x : imv) in >> x;
  for (float& x : vp) in >> x;
  in >> step >> intensity >> cutoff >> RW >> RH >> rbps >> rpath;
  for (float& x : ip) in >> x;
  in >> w >> h >> sscale >> sblend;
  if (!in) return 3;
  std::vector<char> vol = slurp(vpath), rad = slurp(rpath);
  int flip[3] = {0, 0, 0};
  try {
    VolumeDescription vd(vol.data(), W, H, D, bps, scale, flip);
    RayCaster rc;
    rc.setVolume(vd);
    rc.setInvModelView(imv);
    rc.setViewport(vp[0], vp[1], vp[2], vp[3]);
    rc.setSampleDistance(step);
    rc.setRayIntensity(intensity);
    rc.setCutoff(cutoff);
    RadRenderer rr;
    rr.set_rad(rad.data(), RW, RH, rbps);
    rr.set_image_plane(ip[0], ip[1], ip[2], ip[3]);
    rr.set_viewport(vp[0], vp[1], vp[2], vp[3]);
    SobelFilter sobel;
    sobel.setScale(sscale);
    sobel.setBlend(sblend);
    float *drr, *drr_f, *rad_b, *rad_f, *mask, *bg;
    size_t n = (size_t)w * h;
    for (float** p : {&drr, &drr_f, &rad_b, &rad_f, &mask, &bg}) cudaMallocWrap(*p, n * sizeof(float));
    fill(bg, (unsigned)n, 1.0f);
    ncc_init((unsigned)n);
    rc.render(drr, w, h);                   // View::renderDrrSingle
    sobel.apply(drr, drr_f, w, h);          //   + View::filter
    rr.render(rad_b, w, h);                 // View::renderRad
    sobel.apply(rad_b, rad_f, w, h);
    drr_background(drr_f, mask, w, h);      // View::renderDRRMask
    multiply(bg, mask, mask, w, h);         // (1f)
    multiply(rad_f, mask, rad_f, w, h);
    multiply(drr_f, mask, drr_f, w, h);
    double cost = 1.0 - ncc(drr_f, rad_f, mask, (unsigned)n);
    std::vector<float> a(n), b(n);
    asc_check(asc_memcpy_d2h(a.data(), drr_f, n * sizeof(float), nullptr), "copy");
    asc_check(asc_memcpy_d2h(b.data(), rad_f, n * sizeof(float), nullptr), "copy");
    std::ofstream out(argv[2], std::ios::binary);
    out.write((const char*)a.data(), n * sizeof(float));
    out.write((const char*)b.data(), n * sizeof(float));
    out.write((const char*)&cost, sizeof cost);
    for (float* p : {drr, drr_f, rad_b, rad_f, mask, bg}) asc_free(p);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
