// Host-side optimizers with the reference's exact semantics, for callers that
// want the reference trajectory rather than the batched device swarm:
// pso() (PSO.cpp:198-295) and AMOEBA (DownhillSimplex.cpp:39-172).
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "asc_internal.cuh"

namespace {

float rand_clamped() { return (float)rand() / (float)RAND_MAX; }  // PSO.cpp:156-159

struct Particle {
  float ncc = FLT_MAX;
  float pos[6] = {0, 0, 0, 0, 0, 0};
  float vel[6] = {0, 0, 0, 0, 0, 0};
};

}  // namespace

ASC_API int asc_pso_sequential(asc_cost_fn cost, void* ctx, int np, float lo, float hi, unsigned max_epochs,
                               unsigned max_stall, unsigned seed, float best_pos[6], float* best_cost)
{
  if (!cost || np < 1 || !best_pos || !best_cost) return ASC_ERR_ARG;
  const float c1 = 1.5f, c2 = 1.5f;  // PSO.hpp:19-20
  srand(seed);
  std::vector<Particle> p(np);
  for (int i = 1; i < np; ++i)
    for (int d = 0; d < 6; ++d) p[i].pos[d] = lo + rand_clamped() * (hi - lo);
  std::vector<Particle> pb = p;
  Particle g;
  float omega = 0.8f;
  int stall = 0;
  unsigned counter = 0;
  bool go = true;
  while (go) {
    if (counter >= max_epochs) go = false;
    Particle cur = g;
    for (int i = 0; i < np; ++i) {
      for (int d = 0; d < 6; ++d) {
        float rp = rand_clamped(), rg = rand_clamped();
        p[i].vel[d] = omega * p[i].vel[d] + c1 * rp * (pb[i].pos[d] - p[i].pos[d]) + c2 * rg * (g.pos[d] - p[i].pos[d]);
        p[i].pos[d] += p[i].vel[d];
      }
      double x[6];
      for (int d = 0; d < 6; ++d) x[d] = (double)p[i].pos[d];
      p[i].ncc = (float)cost(x, ctx);
      if (p[i].ncc < pb[i].ncc) pb[i] = p[i];
      if (p[i].ncc < g.ncc) g = p[i];
    }
    omega = omega * 0.9f;
    float dd = fabsf(g.ncc - cur.ncc);
    if (dd < 1e-4f)
      stall++;
    else if (dd > 0.001f)
      stall = 0;
    if ((unsigned)stall == max_stall) go = false;
    counter++;
  }
  for (int d = 0; d < 6; ++d) best_pos[d] = g.pos[d];
  *best_cost = g.ncc;
  return ASC_OK;
}

ASC_API int asc_amoeba(asc_cost_fn cost, void* ctx, double* P, double* Y, int ndim, double ftol, int* iterations)
{
  if (!cost || !P || !Y || ndim < 1 || ndim > 20) return ASC_ERR_ARG;
  const int ITMAX = 1000, mpts = ndim + 1;
  const double ALPHA = 1.0, BETA = 0.5, GAMMA = 2.0;
  std::vector<double> pr(ndim), prr(ndim), pbar(ndim), cent(ndim);
  int iter = 0;
  for (;;) {
    int ilo = 0, ihi, inhi;
    if (Y[0] > Y[1]) { ihi = 0; inhi = 1; } else { ihi = 1; inhi = 0; }
    for (int i = 0; i < mpts; ++i) {
      if (Y[i] < Y[ilo]) ilo = i;
      if (Y[i] > Y[ihi]) { inhi = ihi; ihi = i; }
      else if (Y[i] > Y[inhi] && i != ihi) inhi = i;
    }
    for (int j = 0; j < ndim; ++j) {
      cent[j] = 0;
      for (int i = 0; i < mpts; ++i) cent[j] += P[i * ndim + j];
      cent[j] /= mpts;
    }
    double rtol = 0;
    for (int i = 0; i < mpts; ++i) {
      double ss = 0;
      for (int j = 0; j < ndim; ++j) ss += (cent[j] - P[i * ndim + j]) * (cent[j] - P[i * ndim + j]);
      rtol += sqrt(ss);
    }
    rtol /= mpts;
    if (rtol < ftol || iter == ITMAX) break;
    ++iter;
    for (int j = 0; j < ndim; ++j) pbar[j] = 0.0;
    for (int i = 0; i < mpts; ++i)
      if (i != ihi)
        for (int j = 0; j < ndim; ++j) pbar[j] += P[i * ndim + j];
    for (int j = 0; j < ndim; ++j) {
      pbar[j] /= 1.0 * ndim;
      pr[j] = (1.0 + ALPHA) * pbar[j] - ALPHA * P[ihi * ndim + j];
    }
    double ypr = cost(pr.data(), ctx);
    if (ypr <= Y[ilo]) {
      for (int j = 0; j < ndim; ++j) prr[j] = GAMMA * pr[j] + (1.0 - GAMMA) * pbar[j];
      double yprr = cost(prr.data(), ctx);
      if (yprr < Y[ilo]) {
        for (int j = 0; j < ndim; ++j) P[ihi * ndim + j] = prr[j];
        Y[ihi] = yprr;
      } else {
        for (int j = 0; j < ndim; ++j) P[ihi * ndim + j] = pr[j];
        Y[ihi] = ypr;
      }
    } else if (ypr >= Y[inhi]) {
      if (ypr < Y[ihi]) {
        for (int j = 0; j < ndim; ++j) P[ihi * ndim + j] = pr[j];
        Y[ihi] = ypr;
      }
      for (int j = 0; j < ndim; ++j) prr[j] = BETA * P[ihi * ndim + j] + (1.0 - BETA) * pbar[j];
      double yprr = cost(prr.data(), ctx);
      if (yprr < Y[ihi]) {
        for (int j = 0; j < ndim; ++j) P[ihi * ndim + j] = prr[j];
        Y[ihi] = yprr;
      } else {
        for (int i = 0; i < mpts; ++i)
          if (i != ilo) {
            for (int j = 0; j < ndim; ++j) {
              pr[j] = 0.5 * (P[i * ndim + j] + P[ilo * ndim + j]);
              P[i * ndim + j] = pr[j];
            }
            Y[i] = cost(pr.data(), ctx);
          }
      }
    } else {
      for (int j = 0; j < ndim; ++j) P[ihi * ndim + j] = pr[j];
      Y[ihi] = ypr;
    }
  }
  if (iterations) *iterations = iter;
  return ASC_OK;
}
