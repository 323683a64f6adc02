// Frame optimisation on top of the batched engine: Tracker::optimize
// (Tracker.cpp:337-580) for every bone of a frame at once.
//
// asc_amoeba_batch runs many Nelder-Mead simplices (AMOEBA,
// DownhillSimplex.cpp:39-172) in lock-step.  Each iteration asks, per
// simplex, for the reflection and — speculatively — the expansion and both
// possible contraction points in one batch, then applies AMOEBA's decision
// rules to the values it needs; a shrink asks for its NDIM points in the next
// batch.  The cost is deterministic, so every simplex follows exactly the
// trajectory of the sequential AMOEBA.
#include <cmath>
#include <cstring>
#include <vector>

#include "asc_internal.cuh"

namespace {

struct Simplex {
  int phase = 0;  // 0 start of an iteration, 1 candidates pending, 2 shrink pending, 3 done
  int iter = 0;
  int ilo = 0, ihi = 0, inhi = 0;
  std::vector<double> pbar, pr, pe, pco, pci;  // reflection, expansion, contraction out / in
};

const int ITMAX = 1000;                        // DownhillSimplex.cpp:62
const double ALPHA = 1.0, BETA = 0.5, GAMMA = 2.0;

}  // namespace

ASC_API int asc_amoeba_batch(asc_batch_cost_fn cost, void* ctx, int ns, double* P, double* Y, int ndim, double ftol,
                             int* iterations)
{
  if (!cost || ns < 1 || !P || !Y || ndim < 1 || ndim > 20) return ASC_ERR_ARG;
  const int mp = ndim + 1;
  std::vector<Simplex> S(ns);
  for (auto& s : S) {
    s.pbar.assign(ndim, 0.0);
    s.pr.assign(ndim, 0.0);
    s.pe.assign(ndim, 0.0);
    s.pco.assign(ndim, 0.0);
    s.pci.assign(ndim, 0.0);
  }
  std::vector<int> who;
  std::vector<double> xs, ys;
  for (;;) {
    who.clear();
    xs.clear();
    // ---- issue requests
    for (int k = 0; k < ns; ++k) {
      Simplex& s = S[k];
      double* p = P + (size_t)k * mp * ndim;
      double* y = Y + (size_t)k * mp;
      if (s.phase == 0) {
        int ilo = 0, ihi, inhi;
        if (y[0] > y[1]) { ihi = 0; inhi = 1; } else { ihi = 1; inhi = 0; }
        for (int i = 0; i < mp; ++i) {
          if (y[i] < y[ilo]) ilo = i;
          if (y[i] > y[ihi]) { inhi = ihi; ihi = i; }
          else if (y[i] > y[inhi] && i != ihi) inhi = i;
        }
        std::vector<double> cent(ndim, 0.0);
        for (int j = 0; j < ndim; ++j) {
          for (int i = 0; i < mp; ++i) cent[j] += p[i * ndim + j];
          cent[j] /= mp;
        }
        double rtol = 0;
        for (int i = 0; i < mp; ++i) {
          double ss = 0;
          for (int j = 0; j < ndim; ++j) ss += (cent[j] - p[i * ndim + j]) * (cent[j] - p[i * ndim + j]);
          rtol += sqrt(ss);
        }
        rtol /= mp;
        if (rtol < ftol || s.iter == ITMAX) {
          s.phase = 3;
          continue;
        }
        s.iter++;
        s.ilo = ilo;
        s.ihi = ihi;
        s.inhi = inhi;
        for (int j = 0; j < ndim; ++j) s.pbar[j] = 0.0;
        for (int i = 0; i < mp; ++i)
          if (i != ihi)
            for (int j = 0; j < ndim; ++j) s.pbar[j] += p[i * ndim + j];
        for (int j = 0; j < ndim; ++j) {
          s.pbar[j] /= 1.0 * ndim;
          s.pr[j] = (1.0 + ALPHA) * s.pbar[j] - ALPHA * p[ihi * ndim + j];
        }
        for (int j = 0; j < ndim; ++j) {
          s.pe[j] = GAMMA * s.pr[j] + (1.0 - GAMMA) * s.pbar[j];
          s.pco[j] = BETA * s.pr[j] + (1.0 - BETA) * s.pbar[j];
          s.pci[j] = BETA * p[ihi * ndim + j] + (1.0 - BETA) * s.pbar[j];
        }
        for (const std::vector<double>* v : {&s.pr, &s.pe, &s.pco, &s.pci}) {
          who.push_back(k);
          xs.insert(xs.end(), v->begin(), v->end());
        }
        s.phase = 1;
      } else if (s.phase == 2) {
        for (int i = 0; i < mp; ++i)
          if (i != s.ilo) {
            who.push_back(k);
            xs.insert(xs.end(), p + i * ndim, p + (i + 1) * ndim);
          }
      }
    }
    if (who.empty()) break;
    ys.assign(who.size(), 0.0);
    int rc = cost((int)who.size(), who.data(), xs.data(), ys.data(), ctx);
    if (rc) return rc;
    // ---- consume results (requests of one simplex are contiguous, in order)
    size_t q = 0;
    while (q < who.size()) {
      const int k = who[q];
      Simplex& s = S[k];
      double* p = P + (size_t)k * mp * ndim;
      double* y = Y + (size_t)k * mp;
      if (s.phase == 1) {
        const double ypr = ys[q], ype = ys[q + 1], yco = ys[q + 2], yci = ys[q + 3];
        q += 4;
        const int ilo = s.ilo, ihi = s.ihi, inhi = s.inhi;
        s.phase = 0;
        if (ypr <= y[ilo]) {
          if (ype < y[ilo]) {
            for (int j = 0; j < ndim; ++j) p[ihi * ndim + j] = s.pe[j];
            y[ihi] = ype;
          } else {
            for (int j = 0; j < ndim; ++j) p[ihi * ndim + j] = s.pr[j];
            y[ihi] = ypr;
          }
        } else if (ypr >= y[inhi]) {
          const std::vector<double>* pc = &s.pci;
          double yc = yci;
          if (ypr < y[ihi]) {
            for (int j = 0; j < ndim; ++j) p[ihi * ndim + j] = s.pr[j];
            y[ihi] = ypr;
            pc = &s.pco;  // the contraction is then taken from the reflected point
            yc = yco;
          }
          if (yc < y[ihi]) {
            for (int j = 0; j < ndim; ++j) p[ihi * ndim + j] = (*pc)[j];
            y[ihi] = yc;
          } else {
            for (int i = 0; i < mp; ++i)
              if (i != ilo)
                for (int j = 0; j < ndim; ++j) p[i * ndim + j] = 0.5 * (p[i * ndim + j] + p[ilo * ndim + j]);
            s.phase = 2;  // their values come with the next batch
          }
        } else {
          for (int j = 0; j < ndim; ++j) p[ihi * ndim + j] = s.pr[j];
          y[ihi] = ypr;
        }
      } else {  // shrink values
        for (int i = 0; i < mp; ++i)
          if (i != s.ilo) y[i] = ys[q++];
        s.phase = 0;
      }
    }
  }
  if (iterations)
    for (int k = 0; k < ns; ++k) iterations[k] = S[k].iter;
  return ASC_OK;
}
