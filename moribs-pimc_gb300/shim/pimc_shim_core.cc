// pimc_shim_core.cc -- look-ahead queues over the reference's streams around
// the library's replay entry points (see pimc_shim_core.h).
#include "pimc_shim_core.h"

#include <deque>
#include <new>
#include <vector>

struct Lookahead {
  pimc_shim_draw draw = nullptr;
  void *ctx = nullptr;
  std::deque<double> q;
  // the first n values of the stream, drawing what is missing
  void fill(size_t n, std::vector<double> &out)
  {
    while (q.size() < n) q.push_back(draw(ctx));
    out.assign(q.begin(), q.begin() + (long)n);
  }
  void take(long n)
  {
    for (long i = 0; i < n && !q.empty(); i++) q.pop_front();
  }
};

struct pimc_shim {
  pimc_handle *h = nullptr;
  Lookahead rnd1, rnd2, rnd3, gauss;
};

extern "C" pimc_shim *pimc_shim_create(pimc_handle *h, pimc_shim_draw rnd1, pimc_shim_draw rnd2,
                                       pimc_shim_draw rnd3, pimc_shim_draw gauss_x1, void *ctx)
{
  if (!h || !rnd1 || !rnd2 || !rnd3 || !gauss_x1) return nullptr;
  pimc_shim *s = new (std::nothrow) pimc_shim();
  if (!s) return nullptr;
  s->h = h;
  s->rnd1.draw = rnd1; s->rnd2.draw = rnd2; s->rnd3.draw = rnd3; s->gauss.draw = gauss_x1;
  s->rnd1.ctx = s->rnd2.ctx = s->rnd3.ctx = s->gauss.ctx = ctx;
  return s;
}

extern "C" void pimc_shim_destroy(pimc_shim *s) { delete s; }

extern "C" pimc_status pimc_shim_bisection(pimc_shim *s, int type, int time, double *total, double *accep)
{
  if (!s || !total || !accep) return PIMC_ERR_BAD_ARG;
  double t0[6], a0[6], t1[6], a1[6];
  pimc_status e = pimc_counters(s->h, t0, a0);
  if (e) return e;
  // the most one call can use: 3 gauss() per midpoint of every level and one
  // rnd3() per level, for every atom of the type
  int numb = 0, levels = 0;
  if ((e = pimc_type_info(s->h, type, &numb, &levels))) return e;
  const size_t ng = 3 * (size_t)numb * ((1u << levels) - 1), nu = (size_t)numb * levels;
  std::vector<double> g, u;
  s->gauss.fill(ng, g);
  s->rnd3.fill(nu, u);
  long used[2] = {0, 0};
  e = pimc_bisection_move(s->h, type, time, 0, g.data(), (long)g.size(), u.data(), (long)u.size(), used, nullptr,
                          nullptr);
  if (e) return e;
  s->gauss.take(used[0]);
  s->rnd3.take(used[1]);
  if ((e = pimc_counters(s->h, t1, a1))) return e;
  *total = t1[type * 3 + 1] - t0[type * 3 + 1];
  *accep = a1[type * 3 + 1] - a0[type * 3 + 1];
  return PIMC_OK;
}

extern "C" pimc_status pimc_shim_molecular(pimc_shim *s, int type, double *total, double *accep)
{
  if (!s || !total || !accep) return PIMC_ERR_BAD_ARG;
  double t0[6], a0[6], t1[6], a1[6];
  pimc_status e = pimc_counters(s->h, t0, a0);
  if (e) return e;
  int numb = 0, levels = 0;
  if ((e = pimc_type_info(s->h, type, &numb, &levels))) return e;
  std::vector<double> u1, u2;
  s->rnd1.fill(3 * (size_t)numb, u1);        // rnd1() x3 per atom, always drawn (mc_piqmc.cc:67-68)
  s->rnd2.fill((size_t)numb, u2);            // rnd2() per atom whose dV >= 0 (mc_piqmc.cc:84-86)
  long used[2] = {0, 0};
  e = pimc_molecular_move(s->h, type, u1.data(), (long)u1.size(), u2.data(), (long)u2.size(), used, nullptr,
                          nullptr);
  if (e) return e;
  s->rnd1.take(used[0]);
  s->rnd2.take(used[1]);
  if ((e = pimc_counters(s->h, t1, a1))) return e;
  *total = t1[type * 3 + 0] - t0[type * 3 + 0];
  *accep = a1[type * 3 + 0] - a0[type * 3 + 0];
  return PIMC_OK;
}

extern "C" pimc_status pimc_shim_rotations(pimc_shim *s, const double *urot, long n, double *total, double *accep)
{
  if (!s || !urot || n < 0 || !total || !accep) return PIMC_ERR_BAD_ARG;
  double t0[6], a0[6], t1[6], a1[6];
  pimc_status e = pimc_counters(s->h, t0, a0);
  if (e) return e;
  if ((e = pimc_rotations_move(s->h, urot, n, nullptr, nullptr))) return e;
  if ((e = pimc_counters(s->h, t1, a1))) return e;
  *total = 0.0;
  *accep = 0.0;
  for (int t = 0; t < 2; t++) {
    *total += t1[t * 3 + 2] - t0[t * 3 + 2];
    *accep += a1[t * 3 + 2] - a0[t * 3 + 2];
  }
  return PIMC_OK;
}

extern "C" void pimc_shim_pending(const pimc_shim *s, long *pending)
{
  if (!s || !pending) return;
  pending[0] = (long)s->rnd1.q.size();
  pending[1] = (long)s->rnd2.q.size();
  pending[2] = (long)s->rnd3.q.size();
  pending[3] = (long)s->gauss.q.size();
}
