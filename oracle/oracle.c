/*
 * oracle.c -- FP64 CPU restatement of Autoscoper's registration cost path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product
 * path in autoscoper_gb300/csrc: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py load it.  Nothing in the product links it.
 *
 * Every function restates, in double precision, one piece of the reference
 * (BrownBiomechanics/Autoscoper, CUDA backend); the file:line it follows is
 * given above each function (paths relative to the reference project root).
 *
 * Parity pin: tests/test_oracle_pin.py compares this oracle against the
 * reference's own sources compiled for the CPU (oracle/build_ref.sh ->
 * oracle/_ref/libascref.so) and against fixtures in tests/golden/ that were
 * generated from that build (tests/golden/make_golden.py).
 *
 * Conventions shared with the reference:
 *  - a rigid frame is double[12]: rotation r[0..8] stored as three columns
 *    (r[0..2] = image of the x axis, ...) followed by translation t[0..2];
 *    see libautoscoper/src/CoordFrame.cpp:356-370 (point_to_world_space);
 *  - images are row-major float/double arrays with row stride = width;
 *  - texture reads use normalized coordinates, texel centres at (i+0.5)/N,
 *    linear filtering and clamp-to-edge addressing
 *    (libautoscoper/src/gpu/cuda/cutil/cutil_create_tex_obj.h:6-28).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define ORC_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------ */
/* Rigid frames (libautoscoper/src/CoordFrame.cpp)                     */
/* ------------------------------------------------------------------ */

ORC_EXPORT void orc_frame_identity(double f[12])
{
  memset(f, 0, 12 * sizeof(double));
  f[0] = f[4] = f[8] = 1.0;
}

/* CoordFrame::rotate, CoordFrame.cpp:262-320 (angle in degrees). */
ORC_EXPORT void orc_frame_rotate(double f[12], const double caxis[3], double angle)
{
  double a[3] = {caxis[0], caxis[1], caxis[2]};
  double c = cos(M_PI * angle / 180.0);
  double s = sin(M_PI * angle / 180.0);
  double mag = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  if (mag == 0) return;
  a[0] /= mag; a[1] /= mag; a[2] /= mag;
  double xx = a[0] * a[0], yy = a[1] * a[1], zz = a[2] * a[2];
  double xy = a[0] * a[1], xz = a[0] * a[2], yz = a[1] * a[2];
  double sx = s * a[0], sy = s * a[1], sz = s * a[2];
  double oc = 1.0 - c;
  double R[9] = {oc * xx + c,  oc * xy + sz, oc * xz - sy,
                 oc * xy - sz, oc * yy + c,  oc * yz + sx,
                 oc * xz + sy, oc * yz - sx, oc * zz + c};
  double *M = f, t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      t[3 * i + j] = M[3 * i + 0] * R[j] + M[3 * i + 1] * R[3 + j] + M[3 * i + 2] * R[6 + j];
  memcpy(f, t, 9 * sizeof(double));
}

/* CoordFrame::from_xyzypr, CoordFrame.cpp:100-108. */
ORC_EXPORT void orc_frame_from_xyzypr(const double v[6], double f[12])
{
  orc_frame_identity(f);
  double ax[3];
  memcpy(ax, f + 6, sizeof ax); orc_frame_rotate(f, ax, v[3]);
  memcpy(ax, f + 3, sizeof ax); orc_frame_rotate(f, ax, v[4]);
  memcpy(ax, f + 0, sizeof ax); orc_frame_rotate(f, ax, v[5]);
  f[9] += v[0]; f[10] += v[1]; f[11] += v[2];
}

/* CoordFrame::from_xyzAxis_angle, CoordFrame.cpp:163-175. */
ORC_EXPORT void orc_frame_from_axis_angle(const double v[6], double f[12])
{
  orc_frame_identity(f);
  double angle = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
  if (angle != 0) orc_frame_rotate(f, v + 3, angle);
  f[9] += v[0]; f[10] += v[1]; f[11] += v[2];
}

/* CoordFrame::to_xyzypr, CoordFrame.cpp:177-189. */
ORC_EXPORT void orc_frame_to_xyzypr(const double f[12], double v[6])
{
  v[0] = f[9]; v[1] = f[10]; v[2] = f[11];
  v[3] = 180.0 * atan2(f[1], f[0]) / M_PI;
  v[4] = 180.0 * atan2(-f[2], sqrt(f[5] * f[5] + f[8] * f[8])) / M_PI;
  v[5] = 180.0 * atan2(f[5], f[8]) / M_PI;
}

/* CoordFrame::operator*, CoordFrame.cpp:478-528. */
ORC_EXPORT void orc_frame_mul(const double a[12], const double b[12], double out[12])
{
  double r[12];
  for (int c = 0; c < 3; ++c)
    for (int i = 0; i < 3; ++i)
      r[3 * c + i] = a[i] * b[3 * c] + a[3 + i] * b[3 * c + 1] + a[6 + i] * b[3 * c + 2];
  for (int i = 0; i < 3; ++i)
    r[9 + i] = a[i] * b[9] + a[3 + i] * b[10] + a[6 + i] * b[11] + a[9 + i];
  memcpy(out, r, sizeof r);
}

/* CoordFrame::inverse, CoordFrame.cpp:335-353. */
ORC_EXPORT void orc_frame_inverse(const double a[12], double out[12])
{
  double r[12] = {a[0], a[3], a[6], a[1], a[4], a[7], a[2], a[5], a[8]};
  r[9] = -(r[0] * a[9] + r[3] * a[10] + r[6] * a[11]);
  r[10] = -(r[1] * a[9] + r[4] * a[10] + r[7] * a[11]);
  r[11] = -(r[2] * a[9] + r[5] * a[10] + r[8] * a[11]);
  memcpy(out, r, sizeof r);
}

/* CoordFrame::point_to_world_space, CoordFrame.cpp:356-370. */
ORC_EXPORT void orc_frame_point(const double f[12], const double p[3], double q[3])
{
  double r[3];
  for (int i = 0; i < 3; ++i) r[i] = f[i] * p[0] + f[3 + i] * p[1] + f[6 + i] * p[2] + f[9 + i];
  memcpy(q, r, sizeof r);
}

/* CoordFrame::to_matrix_row_order, CoordFrame.cpp:223-241. */
ORC_EXPORT void orc_frame_row_matrix(const double f[12], double m[16])
{
  double t[16] = {f[0], f[3], f[6], f[9], f[1], f[4], f[7], f[10], f[2], f[5], f[8], f[11], 0, 0, 0, 1};
  memcpy(m, t, sizeof t);
}

/* CoordFrame::linear_extrap, CoordFrame.cpp:419-476 (this = a, x = b). */
ORC_EXPORT void orc_frame_linear_extrap(const double a[12], const double b[12], double out[12])
{
  const double t = 2.0;
  double trans[3] = {t * (b[9] - a[9]), t * (b[10] - a[10]), t * (b[11] - a[11])};
  double A[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      A[3 * r + c] = b[c] * a[r] + b[3 + c] * a[3 + r] + b[6 + c] * a[6 + r];
  double axis[3] = {1.0, 0.0, 0.0};
  double trace = A[0] + A[4] + A[8];
  double ang = acos((trace - 1.0) / 2.0);
  if (ang > 0.0 && ang < M_PI) {
    axis[0] = A[5] - A[7];
    axis[1] = A[6] - A[2];
    axis[2] = A[1] - A[3];
  }
  double x3[12];
  memcpy(x3, a, sizeof x3);
  orc_frame_rotate(x3, axis, t * 180.0 * ang / M_PI);
  x3[9] += trans[0]; x3[10] += trans[1]; x3[11] += trans[2];
  memcpy(out, x3, sizeof x3);
}

/* A pose as Tracker::optimize stores it in the trial's key curves and reads
 * it back (Tracker.cpp:422-438): x, y, z as float; the rotation as a float
 * quaternion from (yaw, pitch, roll) (Quaternion.hpp:80-94), read back as
 * Euler angles (Quaternion.hpp:220-243).  Float math throughout, as there. */
/* Quat<float>(yaw, pitch, roll), Quaternion.hpp:80-94: q = (w, x, y, z). */
ORC_EXPORT void orc_quat_from_ypr(float yaw, float pitch, float roll, float q[4])
{
  const float pi = (float)M_PI;
  const float cr = cosf(roll * pi / 360.0f), sr = sinf(roll * pi / 360.0f);
  const float cp = cosf(pitch * pi / 360.0f), sp = sinf(pitch * pi / 360.0f);
  const float cy = cosf(yaw * pi / 360.0f), sy = sinf(yaw * pi / 360.0f);
  q[0] = cr * cp * cy + sr * sp * sy;
  q[1] = sr * cp * cy - cr * sp * sy;
  q[2] = cr * sp * cy + sr * cp * sy;
  q[3] = cr * cp * sy - sr * sp * cy;
}

/* Quat<float>::toEuler, Quaternion.hpp:220-243, read as (yaw, pitch, roll)
   = (e.z, e.y, e.x) in degrees. */
ORC_EXPORT void orc_quat_to_ypr(const float q[4], double ypr[3])
{
  const float pi = (float)M_PI;
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  const float r_x = atan2f(2.0f * (w * x + y * z), 1.0f - 2.0f * (x * x + y * y));
  const float sp2 = sqrtf(1.0f + 2.0f * (w * y - x * z)), cp2 = sqrtf(1.0f - 2.0f * (w * y - x * z));
  const float r_y = 2.0f * atan2f(sp2, cp2) - pi / 2.0f;
  const float r_z = atan2f(2.0f * (w * z + x * y), 1.0f - 2.0f * (y * y + z * z));
  ypr[0] = r_z * (180.0f / pi);
  ypr[1] = r_y * (180.0f / pi);
  ypr[2] = r_x * (180.0f / pi);
}

ORC_EXPORT void orc_keycurve_store(const double in[6], double out[6])
{
  float q[4];
  orc_quat_from_ypr((float)in[3], (float)in[4], (float)in[5], q);
  out[0] = (float)in[0];
  out[1] = (float)in[1];
  out[2] = (float)in[2];
  orc_quat_to_ypr(q, out + 3);
}

/* KeyCurve<float>::operator() (KeyCurve.hpp:334-359) over keys (times
   ascending, float values), every key SMOOTH: the tangent of key i is
   (v[i+1] - v[i-1]) / (t[i+1] - t[i-1]) with the neighbours clamped to the
   ends (update_curve, KeyCurve.hpp:403-426), and the segment from key i is
   the cubic a + b s + c s^2 + d s^3 with D1 = tan_i (t[i+1] - t[i]),
   D2 = tan_{i+1} (t[i+1] - t[i]) (KeyCurve.hpp:428-441).  Here every
   tangent and segment is computed afresh from the final keys. */
static float curve_tangent(int n, const int *t, const float *v, int i)
{
  const int p = i > 0 ? i - 1 : i, q = i < n - 1 ? i + 1 : i;
  return (v[q] - v[p]) / (float)(t[q] - t[p]);
}

ORC_EXPORT float orc_curve_eval(int n, const int *t, const float *v, int frame)
{
  if (n == 0) return 0.0f;
  int j = 0; /* first key after frame */
  while (j < n && t[j] <= frame) ++j;
  if (j == 0) return v[0];
  if (j == n) return v[n - 1];
  const int i = j - 1;
  const float ti = (float)t[i], dt = (float)t[j] - ti;
  const float D1 = curve_tangent(n, t, v, i) * dt, D2 = curve_tangent(n, t, v, j) * dt;
  const float a = v[i], b = D1;
  const float c = 3.0f * (v[j] - v[i]) - 2.0f * D1 - D2;
  const float d = 2.0f * (v[i] - v[j]) + D1 + D2;
  const float s = ((float)frame - ti) / (float)(t[j] - t[i]);
  return a + s * b + s * s * c + s * s * s * d;
}

static float q4_dot(const float *p, const float *q) { return p[0] * q[0] + p[1] * q[1] + p[2] * q[2] + p[3] * q[3]; }
static void q4_unit(const float *q, float *o)
{
  const float l = sqrtf(q4_dot(q, q));
  for (int k = 0; k < 4; ++k) o[k] = q[k] / l;
}

/* KeyCurve<Quatf>::operator(): slerp (Quaternion.hpp:380-396) between the
   keys around frame, nlerp (:400-403) for nearly equal ones; q: 4 floats
   (w, x, y, z) per key. */
ORC_EXPORT void orc_quat_curve_eval(int n, const int *t, const float *q, int frame, float out[4])
{
  if (n == 0) {
    out[0] = 1.0f;
    out[1] = out[2] = out[3] = 0.0f;
    return;
  }
  int j = 0;
  while (j < n && t[j] <= frame) ++j;
  const float *src = j == 0 ? q : q + 4 * (j - 1);
  if (j == 0 || j == n) {
    for (int k = 0; k < 4; ++k) out[k] = src[k];
    return;
  }
  const float *p0 = q + 4 * (j - 1), *p1 = q + 4 * j;
  const float s = ((float)frame - (float)t[j - 1]) / (float)(t[j] - t[j - 1]);
  float r[4], u0[4], u1[4];
  if (s < FLT_EPSILON) {
    for (int k = 0; k < 4; ++k) out[k] = p0[k];
    return;
  }
  if (s > 1.0f - FLT_EPSILON) {
    for (int k = 0; k < 4; ++k) out[k] = p1[k];
    return;
  }
  q4_unit(p0, u0);
  q4_unit(p1, u1);
  const float cr = q4_dot(u0, u1);
  float rad = acosf(cr);
  if (rad < FLT_EPSILON) {
    if (q4_dot(p0, p1) > 0.0f)
      for (int k = 0; k < 4; ++k) r[k] = p0[k] + s * (p1[k] - p0[k]);
    else
      for (int k = 0; k < 4; ++k) r[k] = p0[k] - s * (p1[k] + p0[k]);
  } else if (cr > 0.0f) {
    const float a = sinf(rad * (1.0f - s)), b = sinf(rad * s);
    for (int k = 0; k < 4; ++k) r[k] = a * p0[k] + b * p1[k];
  } else {
    rad = (float)(M_PI - (double)rad);
    const float a = sinf(rad * (1.0f - s)), b = sinf(rad * s);
    for (int k = 0; k < 4; ++k) r[k] = a * p0[k] - b * p1[k];
  }
  q4_unit(r, out);
}

/* ------------------------------------------------------------------ */
/* Camera (libautoscoper/src/Camera.cpp:424-484)                       */
/* ------------------------------------------------------------------ */

/* Camera::calculateViewport, Camera.cpp:424-438. Returns -1 if fx or fy is 0. */
ORC_EXPORT int orc_camera_viewport(double cx, double cy, double fx, double fy, double W, double H, double vp[4])
{
  if (fx == 0 || fy == 0) return -1;
  vp[0] = -(2.0 * cx - W) / fx;
  vp[1] = -(2.0 * cy - H) / fy;
  vp[2] = 2.0 * W / fx;
  vp[3] = 2.0 * H / fy;
  return 0;
}

/* Camera::calculateImagePlane, Camera.cpp:440-484. */
ORC_EXPORT void orc_camera_image_plane(const double cam[12], double cx, double cy, double z, double W, double H,
                                       double ip[12])
{
  double dist = sqrt(cam[9] * cam[9] + cam[10] * cam[10] + cam[11] * cam[11]);
  double scale = -1.5 * dist / z;
  double tr[3] = {scale * (W / 2.0 - cx), scale * (H / 2.0 - cy), scale * z};
  double c[3];
  orc_frame_point(cam, tr, c);
  double hw = scale * W / 2.0, hh = scale * H / 2.0;
  const double *right = cam, *up = cam + 3;
  for (int i = 0; i < 3; ++i) {
    ip[0 + i] = c[i] - hw * right[i] + hh * up[i];
    ip[3 + i] = c[i] - hw * right[i] - hh * up[i];
    ip[6 + i] = c[i] + hw * right[i] - hh * up[i];
    ip[9 + i] = c[i] + hw * right[i] + hh * up[i];
  }
}

/* Tracker::calculate_viewport, Tracker.cpp:923-1032.  Returns 1 when the
 * projected volume box overlaps the image, 0 when it is out of view or NaN. */
ORC_EXPORT int orc_calculate_viewport(const double mv[12], const double cam[12], const double ip[12],
                                      const float inv_scale[3], const float inv_trans[3], double vp[4])
{
  double mm[4] = {1.0, 1.0, -1.0, -1.0};
  static const double corners[24] = {0, 0, -1, 0, 0, 0, 0, 1, -1, 0, 1, 0, 1, 0, -1, 1, 0, 0, 1, 1, -1, 1, 1, 0};
  for (int j = 0; j < 8; ++j) {
    double p[3], q[3];
    for (int k = 0; k < 3; ++k) p[k] = (corners[3 * j + k] - (double)inv_trans[k]) / (double)inv_scale[k];
    orc_frame_point(mv, p, q);
    double fx = -2 * q[0] / q[2], fy = -2 * q[1] / q[2];
    if (mm[0] > fx) mm[0] = fx;
    if (mm[1] > fy) mm[1] = fy;
    if (mm[2] < fx) mm[2] = fx;
    if (mm[3] < fy) mm[3] = fy;
  }
  double ci[12], a[3], b[3];
  orc_frame_inverse(cam, ci);
  orc_frame_point(ci, ip + 3, a);
  orc_frame_point(ci, ip + 9, b);
  double rf[4] = {-2 * a[0] / a[2], -2 * a[1] / a[2], -2 * b[0] / b[2], -2 * b[1] / b[2]};
  if (mm[0] > rf[2] && mm[2] > rf[2]) return 0;
  if (mm[1] > rf[3] && mm[3] > rf[3]) return 0;
  if (mm[0] < rf[0] && mm[2] < rf[0]) return 0;
  if (mm[1] < rf[1] && mm[3] < rf[1]) return 0;
  if (mm[0] == 1.0 && mm[1] == 1.0 && mm[2] == -1.0 && mm[3] == -1.0) return 0;
  if (mm[0] < rf[0]) mm[0] = rf[0];
  if (mm[1] < rf[1]) mm[1] = rf[1];
  if (mm[2] > rf[2]) mm[2] = rf[2];
  if (mm[3] > rf[3]) mm[3] = rf[3];
  vp[0] = mm[0];
  vp[1] = mm[1];
  vp[2] = mm[2] - mm[0];
  vp[3] = mm[3] - mm[1];
  return 1;
}

/* RayCaster::setInvModelView, RayCaster.cpp:88-114: folds the volume's
 * normalisation into the camera->volume matrix.  Returns the 3x4 rows. */
ORC_EXPORT void orc_fold_inv_model_view(const double imv[16], const float inv_scale[3], const float inv_trans[3],
                                        double m[12])
{
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) m[4 * r + c] = imv[4 * r + c] * (double)inv_scale[r] + imv[12 + c] * (double)inv_trans[r];
}

/* ------------------------------------------------------------------ */
/* Volume description (libautoscoper/src/VolumeDescription.cpp:59-252) */
/* ------------------------------------------------------------------ */

/* Flip (:59-74), crop to the non-zero box (:76-120), copy with min/max
 * (:122-148) and the normalisation constants (:240-252).  `out` must hold
 * W*H*D voxels.  Returns -1 for an unsupported bit depth, -2 for an empty
 * volume (the reference calls exit(0) in both cases). */
ORC_EXPORT int orc_volume_describe(const void *data, int W, int H, int D, int bps, const double scale[3],
                                   const int flip[3], void *out, int dims[3], float inv_scale[3], float inv_trans[3],
                                   double trans_center[3], float *min_value, float *max_value)
{
  if (bps != 8 && bps != 16) return -1;
  size_t n = (size_t)W * H * D, bytes = (size_t)bps / 8;
  unsigned char *fl = (unsigned char *)malloc(n * bytes);
  for (int k = 0; k < D; ++k)
    for (int i = 0; i < H; ++i)
      for (int j = 0; j < W; ++j) {
        int x = flip[0] ? W - 1 - j : j, y = flip[1] ? H - 1 - i : i, z = flip[2] ? D - 1 - k : k;
        memcpy(fl + ((size_t)z * W * H + (size_t)y * W + x) * bytes, (const unsigned char *)data + ((size_t)k * W * H + (size_t)i * W + j) * bytes, bytes);
      }
#define VOX(p) (bps == 8 ? (unsigned)((const uint8_t *)fl)[p] : (unsigned)((const uint16_t *)fl)[p])
  int mn[3] = {W, H, D}, mx[3] = {0, 0, 0};
  size_t p = 0;
  for (int k = 0; k < D; ++k) {
    int col = 0;
    for (int i = 0; i < H; ++i) {
      int row = 0;
      for (int j = 0; j < W; ++j, ++p)
        if (VOX(p) != 0) {
          if (j < mn[0]) mn[0] = j;
          if (j > mx[0]) mx[0] = j;
          row = 1;
        }
      if (row) {
        if (i < mn[1]) mn[1] = i;
        if (i > mx[1]) mx[1] = i;
        col = 1;
      }
    }
    if (col) {
      if (k < mn[2]) mn[2] = k;
      if (k > mx[2]) mx[2] = k;
    }
  }
  if (mn[0] > mx[0] || mn[1] > mx[1] || mn[2] > mx[2]) {
    free(fl);
    return -2;
  }
  for (int a = 0; a < 3; ++a) dims[a] = mx[a] - mn[a] + 1;
  unsigned vmin = bps == 8 ? 255u : 65535u, vmax = 0;
  size_t q = 0;
  for (int k = mn[2]; k <= mx[2]; ++k)
    for (int i = mn[1]; i <= mx[1]; ++i)
      for (int j = mn[0]; j <= mx[0]; ++j, ++q) {
        size_t s = (size_t)k * W * H + (size_t)i * W + j;
        unsigned v = VOX(s);
        if (v < vmin) vmin = v;
        if (v > vmax) vmax = v;
        memcpy((unsigned char *)out + q * bytes, fl + s * bytes, bytes);
      }
#undef VOX
  float norm = bps == 8 ? 255.0f : 65535.0f;
  *min_value = vmin / norm;
  *max_value = vmax / norm;
  float sc[3] = {(float)scale[0], (float)scale[1], (float)scale[2]};
  trans_center[0] = -sc[0] * 0.5 * (mn[0] + mx[0]);
  trans_center[1] = -sc[1] * 0.5 * (mn[1] + mx[1]);
  trans_center[2] = sc[2] * 0.5 * (mn[2] + mx[2]);
  for (int a = 0; a < 3; ++a) inv_scale[a] = 1.0f / (float)(sc[a] * dims[a]);
  inv_trans[0] = -mn[0] / (float)dims[0];
  inv_trans[1] = -((H - mx[1] - 1) / (float)dims[1]);
  inv_trans[2] = mn[2] / (float)dims[2];
  free(fl);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Texture sampling                                                     */
/* ------------------------------------------------------------------ */

/* vtype: 8 = u8 normalized by 255, 16 = u16 normalized by 65535,
 * 32 = float32 read as stored (cudaReadModeElementType). */
static inline double texel(const void *d, int vtype, size_t i)
{
  if (vtype == 16) return ((const uint16_t *)d)[i] / 65535.0;
  if (vtype == 8) return ((const uint8_t *)d)[i] / 255.0;
  return (double)((const float *)d)[i];
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* 1-D linear filter set-up with clamp-to-edge for normalized coordinate u. */
static inline void lin_setup(double u, int n, int *i0, int *i1, double *a)
{
  double x = u * n - 0.5;
  double fl = floor(x);
  *a = x - fl;
  /* Clamp the coordinate before converting so that huge values stay defined. */
  if (fl < -1.0) fl = -1.0;
  if (fl > (double)n) fl = (double)n;
  int i = (int)fl;
  *i0 = clampi(i, 0, n - 1);
  *i1 = clampi(i + 1, 0, n - 1);
}

static double tex3d(const void *d, int vtype, int nx, int ny, int nz, double x, double y, double z)
{
  int x0, x1, y0, y1, z0, z1;
  double ax, ay, az;
  lin_setup(x, nx, &x0, &x1, &ax);
  lin_setup(y, ny, &y0, &y1, &ay);
  lin_setup(z, nz, &z0, &z1, &az);
  size_t sxy = (size_t)nx * ny;
#define T(i, j, k) texel(d, vtype, (size_t)(k) * sxy + (size_t)(j) * nx + (i))
  double c00 = T(x0, y0, z0) * (1 - ax) + T(x1, y0, z0) * ax;
  double c10 = T(x0, y1, z0) * (1 - ax) + T(x1, y1, z0) * ax;
  double c01 = T(x0, y0, z1) * (1 - ax) + T(x1, y0, z1) * ax;
  double c11 = T(x0, y1, z1) * (1 - ax) + T(x1, y1, z1) * ax;
#undef T
  double c0 = c00 * (1 - ay) + c10 * ay;
  double c1 = c01 * (1 - ay) + c11 * ay;
  return c0 * (1 - az) + c1 * az;
}

static double tex2d(const void *d, int vtype, int nx, int ny, double x, double y)
{
  int x0, x1, y0, y1;
  double ax, ay;
  lin_setup(x, nx, &x0, &x1, &ax);
  lin_setup(y, ny, &y0, &y1, &ay);
#define T(i, j) texel(d, vtype, (size_t)(j) * nx + (i))
  double c0 = T(x0, y0) * (1 - ax) + T(x1, y0) * ax;
  double c1 = T(x0, y1) * (1 - ax) + T(x1, y1) * ax;
#undef T
  return c0 * (1 - ay) + c1 * ay;
}

ORC_EXPORT double orc_tex3d(const void *d, int vtype, int nx, int ny, int nz, double x, double y, double z)
{
  return tex3d(d, vtype, nx, ny, nz, x, y, z);
}

ORC_EXPORT double orc_tex2d(const void *d, int vtype, int nx, int ny, double x, double y)
{
  return tex2d(d, vtype, nx, ny, x, y);
}

/* ------------------------------------------------------------------ */
/* Renderers                                                            */
/* ------------------------------------------------------------------ */

/* cuda_volume_render_kernel, RayCaster_kernels.cu:113-195.
 * m: folded 3x4 camera->volume matrix (row-major), vp: viewport.
 * Writes the DRR (w*h) and, if `nsamples` is non-NULL, the number of
 * trilinear samples taken per pixel. */
ORC_EXPORT void orc_raycast(const void *vol, int vtype, int nx, int ny, int nz, const double m[12], const double vp[4],
                            double step, double intensity, double cutoff, double *out, int w, int h,
                            int32_t *nsamples)
{
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      double u = vp[0] + vp[2] * (x / (double)w);
      double v = vp[1] + vp[3] * (y / (double)h);
      double len = sqrt(u * u + v * v + 4.0);
      double l[3] = {step * u / len, step * v / len, step * -2.0 / len};
      double o[3] = {m[3], m[7], m[11]};
      double dir[3];
      for (int r = 0; r < 3; ++r) dir[r] = m[4 * r] * l[0] + m[4 * r + 1] * l[1] + m[4 * r + 2] * l[2];
      static const double bmin[3] = {0.0, 0.0, -1.0}, bmax[3] = {1.0, 1.0, 0.0};
      double tn = -INFINITY, tf = INFINITY;
      for (int r = 0; r < 3; ++r) {
        double inv = 1.0 / dir[r];
        double tb = inv * (bmin[r] - o[r]), tt = inv * (bmax[r] - o[r]);
        double lo = fmin(tt, tb), hi = fmax(tt, tb);
        tn = r == 0 ? lo : fmax(tn, lo);
        tf = r == 0 ? hi : fmin(tf, hi);
      }
      size_t px = (size_t)y * w + x;
      if (!(tf > tn)) {
        out[px] = 0.0;
        if (nsamples) nsamples[px] = 0;
        continue;
      }
      if (tn < 0.0) tn = 0.0;
      double t = tf, density = 0.0;
      int32_t cnt = 0;
      while (t > tn) {
        double p0 = o[0] + t * dir[0], p1 = o[1] + t * dir[1], p2 = o[2] + t * dir[2];
        double s = tex3d(vol, vtype, nx, ny, nz, p0, 1.0 - p1, -p2);
        density += s > cutoff ? step * s : 0.0;
        t -= 1.0;
        ++cnt;
      }
      double r = density / intensity;
      out[px] = r < 0.0 ? 0.0 : (r > 1.0 ? 1.0 : r);
      if (nsamples) nsamples[px] = cnt;
    }
  }
}

/* image_render_kernel, RadRenderer_kernels.cu:85-116 (mode 0) and
 * background_render_kernel, BackgroundRenderer_kernels.cu:88-120 (mode 1).
 * ip = image plane (u0, v0, u1, v1) = the camera viewport; vp = viewport. */
ORC_EXPORT void orc_image_render(const void *img, int vtype, int W, int H, const double ip[4], const double vp[4],
                                 int mode, double threshold, double *out, int w, int h)
{
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      double u = vp[0] + vp[2] * (x / (double)w);
      double v = vp[1] + vp[3] * (y / (double)h);
      double s = (u - ip[0]) / ip[2] + 0.5;
      double t = 0.5 - (v - ip[1]) / ip[3];
      double r;
      if (s < 0.0 || t < 0.0 || s > 1.0 || t > 1.0)
        r = 0.0;
      else if (mode == 0)
        r = 1.0 - tex2d(img, vtype, W, H, s, t);
      else
        r = (threshold <= tex2d(img, vtype, W, H, s, t)) ? 1.0 : 0.0;
      out[(size_t)y * w + x] = r;
    }
}

/* drr_background_kernel, DRRBackground_kernels.cu:62-75. */
ORC_EXPORT void orc_drr_background(const double *src, double *dst, size_t n)
{
  for (size_t i = 0; i < n; ++i) dst[i] = src[i] != 0.0 ? 1.0 : 0.0;
}

/* mult_kernel, Mult_kernels.cu:64-77. */
ORC_EXPORT void orc_multiply(const double *a, const double *b, double *dst, size_t n)
{
  for (size_t i = 0; i < n; ++i) dst[i] = a[i] * b[i];
}

/* merge_kernel, Merger_kernels.cu:62-75. */
ORC_EXPORT void orc_merge(const double *a, const double *b, double *dst, size_t n)
{
  for (size_t i = 0; i < n; ++i) dst[i] = fmin(a[i] + b[i], 1.0);
}

/* composite_kernel, Compositor_kernels.cu:72-88 (src4 is unused there too). */
ORC_EXPORT void orc_composite(const double *s1, const double *s2, const double *s3, double *dst, size_t n)
{
  for (size_t i = 0; i < n; ++i) {
    double multi = s3[i] < 0.5 ? 0.0 : 1.0;
    dst[3 * i + 0] = s1[i];
    dst[3 * i + 1] = multi * (s1[i] / 2.0 + s2[i] / 2.0);
    dst[3 * i + 2] = s2[i];
  }
}

/* ------------------------------------------------------------------ */
/* Filters                                                              */
/* ------------------------------------------------------------------ */

/* sobel_filter_kernel, SobelFilter_kernels.cu:63-113. */
ORC_EXPORT void orc_sobel(const double *in, double *out, int w, int h, double scale, double blend)
{
#pragma omp parallel for schedule(static)
  for (int y1 = 0; y1 < h; ++y1)
    for (int x1 = 0; x1 < w; ++x1) {
      int x0 = x1 > 0 ? x1 - 1 : 0, y0 = y1 > 0 ? y1 - 1 : 0;
      int x2 = x1 < w - 1 ? x1 + 1 : w - 1, y2 = y1 < h - 1 ? y1 + 1 : h - 1;
#define P(yy, xx) in[(size_t)(yy) * w + (xx)]
      double p00 = P(y0, x0), p01 = P(y0, x1), p02 = P(y0, x2);
      double p10 = P(y1, x0), p11 = P(y1, x1), p12 = P(y1, x2);
      double p20 = P(y2, x0), p21 = P(y2, x1), p22 = P(y2, x2);
#undef P
      double horz = p02 + 2 * p12 + p22 - p00 - 2 * p10 - p20;
      double vert = p00 + 2 * p01 + p02 - p20 - 2 * p21 - p22;
      double grad = sqrt(horz * horz + vert * vert);
      double sum = blend < 0.5 ? scale * grad + 2.0 * blend * p11 : 2.0 * (1.0 - blend) * scale * grad + p11;
      out[(size_t)y1 * w + x1] = sum < 0.0 ? 0.0 : (sum > 1.0 ? 1.0 : sum);
    }
}

/* contrast_filter_kernel + average, ContrastFilter_kernels.cu:62-96. */
ORC_EXPORT void orc_contrast(const double *in, double *out, int w, int h, double alpha, double beta, int size)
{
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      int i0 = y - size / 2 > 0 ? y - size / 2 : 0, i1 = y + (size + 1) / 2 < h ? y + (size + 1) / 2 : h;
      int j0 = x - size / 2 > 0 ? x - size / 2 : 0, j1 = x + (size + 1) / 2 < w ? x + (size + 1) / 2 : w;
      double n = 0, s = 0;
      for (int i = i0; i < i1; ++i)
        for (int j = j0; j < j1; ++j) {
          n += 1.0;
          s += in[(size_t)i * w + j];
        }
      double axy = s / n, fxy = in[(size_t)y * w + x];
      out[(size_t)y * w + x] = axy > 0.01 ? pow(axy, alpha - beta) * pow(fxy, beta) : 0.0;
    }
}

/* Gaussian weights of GaussianFilter::set_radius (GaussianFilter.cpp:73-121)
 * and SharpenFilter::makeFilter (SharpenFilter.cpp:102-145): K = 2*floor(3r)+1,
 * w(i,j) = 2.71828^(-((i-R)^2+(j-R)^2)/(2r)), normalised to sum 1.
 * Writes K*K weights into `wts` (capacity `cap`) and returns K (1 = identity). */
ORC_EXPORT int orc_gauss_weights(double radius, double *wts, int cap)
{
  if (radius < 0) radius = 0;
  int R = (int)(3 * (float)radius);
  int K = 2 * R + 1;
  if (K == 1 || K * K > cap) return K;
  double sum = 0;
  for (int i = 0; i < K; ++i)
    for (int j = 0; j < K; ++j) {
      double e = -(pow((double)(i - R), 2) + pow((double)(j - R), 2)) / (2 * radius);
      wts[i * K + j] = pow(2.71828, e);
      sum += wts[i * K + j];
    }
  for (int i = 0; i < K * K; ++i) wts[i] /= sum;
  return K;
}

/* filterConvolution, GaussianFilter_kernels.cu:66-89 / SharpenFilter_kernels.cu:82-104:
 * out-of-image taps are skipped (not renormalised). */
static double convolve(const double *in, int w, int h, int x, int y, const double *wts, int K)
{
  int R = (K - 1) / 2;
  double c = 0;
  for (int i = 0; i < K; ++i)
    for (int j = 0; j < K; ++j) {
      int a = x - R + i, b = y - R + j;
      if (!(a < 0 || a >= w || b < 0 || b >= h)) c += wts[i * K + j] * in[(size_t)b * w + a];
    }
  return c;
}

/* filter_kernel, GaussianFilter_kernels.cu:61-97 (result clamped to [0,1]).
 * K == 1 copies the image (the reference comment's intent; its
 * GaussianFilter.cpp:130-131 copies a single float). */
ORC_EXPORT void orc_gaussian(const double *in, double *out, int w, int h, const double *wts, int K)
{
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t p = (size_t)y * w + x;
      if (K == 1) {
        out[p] = in[p];
        continue;
      }
      double c = convolve(in, w, h, x, y, wts, K);
      out[p] = c > 1 ? 1 : (c < 0 ? 0 : c);
    }
}

/* sharpen_filter_kernel, SharpenFilter_kernels.cu:106-129. */
ORC_EXPORT void orc_sharpen(const double *in, double *out, int w, int h, const double *wts, int K, double contrast,
                            double threshold)
{
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t p = (size_t)y * w + x;
      if (K == 1) {
        out[p] = in[p];
        continue;
      }
      double blur = convolve(in, w, h, x, y, wts, K);
      double f = in[p];
      if (fabs(f - blur) > threshold) {
        double o = f + contrast * (f - blur);
        out[p] = o > 1 ? 1 : (o < 0 ? 0 : o);
      } else {
        out[p] = f;
      }
    }
}

/* ------------------------------------------------------------------ */
/* Cost reductions                                                      */
/* ------------------------------------------------------------------ */

/* Inclusion of element i in the reference's multi-level sum() of n floats
 * (Ncc_kernels.cu:137-187, HDist_kernels.cu same): each level launches
 * ceil(n_l/T_l) blocks of T_l = min(n_l, 256) threads and folds shared memory
 * with s = T_l/2, T_l/4, ...; for a T_l that is not a power of two the fold
 * never reads the slots at or above 2s, so those partials are dropped.
 * Returns 1 if element i reaches the final sum. */
ORC_EXPORT int orc_tree_keep(size_t i, size_t n)
{
  size_t idx = i;
  while (n > 1) {
    size_t T = n < 256 ? n : 256;
    size_t t = idx % T;
    for (size_t s = T >> 1; s > 0; s >>= 1) {
      if (t >= 2 * s) return 0;
      if (t >= s) t -= s;
    }
    idx /= T;
    n = (n + T - 1) / T;
  }
  return 1;
}

/* gpu::ncc, Ncc_kernels.cu:116-134 with cuda_ncc_kernel :189-213.
 * tree = 1 reproduces the reference's sum() coverage (orc_tree_keep);
 * tree = 0 sums every element. */
ORC_EXPORT double orc_ncc(const double *f, const double *g, const double *mask, size_t n, int tree)
{
  double sm = 0, sf = 0, sg = 0;
  for (size_t i = 0; i < n; ++i) {
    if (tree && !orc_tree_keep(i, n)) continue;
    sm += mask[i];
    sf += f[i];
    sg += g[i];
  }
  double mf = sf / sm, mg = sg / sm, num = 0, d1 = 0, d2 = 0;
  for (size_t i = 0; i < n; ++i)
    if (mask[i] > 0.5 && (!tree || orc_tree_keep(i, n))) {
      double a = f[i] - mf, b = g[i] - mg;
      num += a * b;
      d1 += a * a;
      d2 += b * b;
    }
  double den = sqrt(d1 * d2);
  if (den < 1e-5) return 1e5;
  return num / den;
}

/* gpu::hdist, HDist_kernels.cu:111-134 with cuda_hdist_kernel :189-203. */
ORC_EXPORT double orc_hdist(const double *f, const double *g, const double *mask, size_t n, int tree)
{
  double sm = 0, sf = 0, sg = 0;
  for (size_t i = 0; i < n; ++i) {
    if (tree && !orc_tree_keep(i, n)) continue;
    sm += mask[i];
    sf += f[i];
    sg += g[i];
  }
  double mf = sf / sm, mg = sg / sm, s = 0;
  for (size_t i = 0; i < n; ++i)
    if (mask[i] > 0.5 && (!tree || orc_tree_keep(i, n))) s += fabs((f[i] - mf) - (g[i] - mg));
  return s;
}
