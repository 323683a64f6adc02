// Pose key curves of a trial: per volume, x, y and z as KeyCurve<float>
// (cubic Bezier segments with SMOOTH tangents, KeyCurve.hpp:231-446) and the
// rotation as KeyCurve<Quatf> (slerp between keys, Quaternion.hpp:380-403).
// Host arithmetic only, in float as the reference stores and evaluates them;
// the library is built with -ffp-contract=off so no product is fused.
#include <cfloat>
#include <cmath>
#include <map>

#include "asc_internal.cuh"

using namespace asc;

namespace {

// KeyCurve<float> with every key SMOOTH, tangents bound and unlocked (what
// KeyCurve::insert creates, KeyCurve.hpp:262-296).
class ScalarCurve {
  struct Key {
    float value = 0.f, in_t = 0.f, out_t = 0.f, a = 0.f, b = 0.f, c = 0.f, d = 0.f;
  };
  using It = std::map<int, Key>::iterator;
  std::map<int, Key> keys_;

  It next_of(It p) { return (p != keys_.end() && p != std::prev(keys_.end())) ? std::next(p) : p; }
  It prev_of(It p) { return p != keys_.begin() ? std::prev(p) : p; }

  // update_curve (KeyCurve.hpp:403-444): the key's SMOOTH tangent from its
  // neighbours, then its cubic segment to the next key.
  void update(It p)
  {
    const float t = (float)p->first;
    Key& k = p->second;
    It prv = prev_of(p), nxt = next_of(p);
    const float nv = nxt->second.value, pv = prv->second.value;
    k.in_t = (nv - pv) / (float)(nxt->first - prv->first);
    k.out_t = (nv - pv) / (float)(nxt->first - prv->first);
    if (nxt != p) {
      const float D1 = k.out_t * ((float)nxt->first - t);
      const float D2 = nxt->second.in_t * ((float)nxt->first - t);
      k.a = k.value;
      k.b = D1;
      k.c = 3.0f * (nv - k.value) - 2.0f * D1 - D2;
      k.d = 2.0f * (k.value - nv) + D1 + D2;
    }
  }

  // key_changed (KeyCurve.hpp:368-401): next, the key, previous, the one
  // before, in that order.
  void changed(It p)
  {
    It nxt = next_of(p), prv = prev_of(p), pp = prev_of(prv);
    if (nxt != p) update(nxt);
    update(p);
    if (prv != p) update(prv);
    if (pp != prv) update(pp);
  }

 public:
  void clear() { keys_.clear(); }
  bool has(int f) const { return keys_.count(f) != 0; }

  void insert(int f, float v)
  {
    keys_[f].value = v;  // a replaced key keeps nothing else that matters: its tangents are recomputed
    changed(keys_.find(f));
  }

  void erase(int f)
  {
    It p = keys_.find(f);
    if (p == keys_.end()) return;
    if (p == keys_.begin()) {
      keys_.erase(p);
      if (!keys_.empty()) changed(keys_.begin());
    } else {
      It q = std::prev(p);
      keys_.erase(p);
      changed(q);
    }
  }

  // operator() (KeyCurve.hpp:334-359)
  float eval(int f) const
  {
    if (keys_.empty()) return 0.f;
    auto p1 = keys_.upper_bound(f);
    if (p1 == keys_.begin()) return p1->second.value;
    auto p0 = std::prev(p1);
    if (p1 == keys_.end()) return p0->second.value;
    const float t = ((float)f - (float)p0->first) / (float)(p1->first - p0->first);
    const Key& k = p0->second;
    return k.a + t * k.b + t * t * k.c + t * t * t * k.d;
  }
};

QuatF qscale(float s, const QuatF& q) { return {s * q.w, s * q.x, s * q.y, s * q.z}; }
QuatF qadd(const QuatF& p, const QuatF& q) { return {p.w + q.w, p.x + q.x, p.y + q.y, p.z + q.z}; }
QuatF qsub(const QuatF& p, const QuatF& q) { return {p.w - q.w, p.x - q.x, p.y - q.y, p.z - q.z}; }
float qdot(const QuatF& p, const QuatF& q) { return p.w * q.w + p.x * q.x + p.y * q.y + p.z * q.z; }
QuatF qunit(const QuatF& q)
{
  const float l = sqrtf(qdot(q, q));
  return {q.w / l, q.x / l, q.y / l, q.z / l};
}

// nlerp and slerp (Quaternion.hpp:380-403).  Note that for nearly equal
// keys the dot of the unit quaternions can round above 1, where acos gives
// NaN and so does the interpolation, as in the reference.
QuatF nlerp(const QuatF& p, const QuatF& q, float t)
{
  return qdot(p, q) > 0.f ? qunit(qadd(p, qscale(t, qsub(q, p)))) : qunit(qsub(p, qscale(t, qadd(q, p))));
}

QuatF slerp(const QuatF& p, const QuatF& q, float t)
{
  if (t < FLT_EPSILON) return p;
  if (t > 1.0f - FLT_EPSILON) return q;
  const float cr = qdot(qunit(p), qunit(q));
  float rad = acosf(cr);
  if (rad < FLT_EPSILON) return nlerp(p, q, t);
  if (cr > 0.f) return qunit(qadd(qscale(sinf(rad * (1.0f - t)), p), qscale(sinf(rad * t), q)));
  rad = (float)(3.14159265358979323846 - (double)rad);
  return qunit(qsub(qscale(sinf(rad * (1.0f - t)), p), qscale(sinf(rad * t), q)));
}

class QuatCurve {
  std::map<int, QuatF> keys_;

 public:
  void clear() { keys_.clear(); }
  bool has(int f) const { return keys_.count(f) != 0; }
  void insert(int f, const QuatF& q) { keys_[f] = q; }
  void erase(int f) { keys_.erase(f); }
  QuatF eval(int f) const
  {
    if (keys_.empty()) return {1.f, 0.f, 0.f, 0.f};  // Quat() is the identity
    auto p1 = keys_.upper_bound(f);
    if (p1 == keys_.begin()) return p1->second;
    auto p0 = std::prev(p1);
    if (p1 == keys_.end()) return p0->second;
    const float t = ((float)f - (float)p0->first) / (float)(p1->first - p0->first);
    return slerp(p0->second, p1->second, t);
  }
};

}  // namespace

struct asc_pose_curve_s {
  ScalarCurve x, y, z;
  QuatCurve q;
};

ASC_API int asc_pose_curve_create(asc_pose_curve* out)
{
  if (!out) return ASC_ERR_ARG;
  *out = new asc_pose_curve_s();
  return ASC_OK;
}

ASC_API int asc_pose_curve_destroy(asc_pose_curve c)
{
  if (!c) return ASC_ERR_ARG;
  delete c;
  return ASC_OK;
}

ASC_API int asc_pose_curve_clear(asc_pose_curve c)
{
  if (!c) return ASC_ERR_ARG;
  c->x.clear();
  c->y.clear();
  c->z.clear();
  c->q.clear();
  return ASC_OK;
}

ASC_API int asc_pose_curve_insert(asc_pose_curve c, int frame, const double xyzypr[6], int mask)
{
  if (!c || !xyzypr || (mask & ~ASC_CURVE_ALL)) return ASC_ERR_ARG;
  if (mask & ASC_CURVE_X) c->x.insert(frame, (float)xyzypr[0]);
  if (mask & ASC_CURVE_Y) c->y.insert(frame, (float)xyzypr[1]);
  if (mask & ASC_CURVE_Z) c->z.insert(frame, (float)xyzypr[2]);
  if (mask & ASC_CURVE_ROT) c->q.insert(frame, quat_from_ypr((float)xyzypr[3], (float)xyzypr[4], (float)xyzypr[5]));
  return ASC_OK;
}

ASC_API int asc_pose_curve_erase(asc_pose_curve c, int frame, int mask)
{
  if (!c || (mask & ~ASC_CURVE_ALL)) return ASC_ERR_ARG;
  if (mask & ASC_CURVE_X) c->x.erase(frame);
  if (mask & ASC_CURVE_Y) c->y.erase(frame);
  if (mask & ASC_CURVE_Z) c->z.erase(frame);
  if (mask & ASC_CURVE_ROT) c->q.erase(frame);
  return ASC_OK;
}

ASC_API int asc_pose_curve_keys(asc_pose_curve c, int frame, int* mask)
{
  if (!c || !mask) return ASC_ERR_ARG;
  *mask = (c->x.has(frame) ? ASC_CURVE_X : 0) | (c->y.has(frame) ? ASC_CURVE_Y : 0) |
          (c->z.has(frame) ? ASC_CURVE_Z : 0) | (c->q.has(frame) ? ASC_CURVE_ROT : 0);
  return ASC_OK;
}

ASC_API int asc_pose_curve_eval(asc_pose_curve c, int frame, double xyzypr[6])
{
  if (!c || !xyzypr) return ASC_ERR_ARG;
  xyzypr[0] = c->x.eval(frame);
  xyzypr[1] = c->y.eval(frame);
  xyzypr[2] = c->z.eval(frame);
  quat_to_ypr(c->q.eval(frame), xyzypr + 3);
  return ASC_OK;
}

// The 4 x 4 column-major matrix of a pose (CoordFrame::from_xyzypr then
// to_matrix, CoordFrame.cpp:100-108, :203-221) and back (from_matrix then
// to_xyzypr, :191-201, :177-189): the tracking-file conversions.
ASC_API int asc_pose_to_matrix(const double xyzypr[6], double m[16])
{
  if (!xyzypr || !m) return ASC_ERR_ARG;
  double f[12];
  frame_from_xyzypr(xyzypr, f);
  for (int c = 0; c < 3; ++c) {
    for (int r = 0; r < 3; ++r) m[4 * c + r] = f[3 * c + r];
    m[4 * c + 3] = 0.0;
  }
  for (int r = 0; r < 3; ++r) m[12 + r] = f[9 + r];
  m[15] = 1.0;
  return ASC_OK;
}

ASC_API int asc_pose_from_matrix(const double m[16], double xyzypr[6])
{
  if (!xyzypr || !m) return ASC_ERR_ARG;
  double f[12];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) f[3 * c + r] = m[4 * c + r];
  for (int r = 0; r < 3; ++r) f[9 + r] = m[12 + r];
  frame_to_xyzypr(f, xyzypr);
  return ASC_OK;
}
