// pimc_io.cu -- the estimators' block files (host code).
//
// The reference writes its accumulated estimators as text files at the end
// of each block (mc_main.cc:715-760) and of the run (mc_main.cc:445-465).
// These functions write the same files, with the same names, columns,
// normalisations and number format (io_setout: scientific, 6 digits, width
// 14, columns separated by three blanks; mc_input.cc:853-858,
// mc_input.h:45-91, mc_confg.h:29), from the arrays the estimator entry
// points of the C ABI return: the pair-density histograms of
// pimc_densities_read, the cycle counts of pimc_exchange_lengths and the
// summed increments of pimc_area_estimators / pimc_area_estim3d.  Units are
// the reference's (Angstrom, amu, Kelvin: all 1, mc_setup.cc:196-199).
#include <cmath>
#include <cstdio>
#include <string>

#include "../../include/pimc_gb300.h"

namespace {

constexpr int kWidth = 14;            // IO_WIDTH
constexpr int kWidthBlock = 4;        // IO_WIDTH_BLOCK
const char *const kBlank = "   ";     // BLANK
constexpr int kGsLoopMax = 7;         // GSLOOP_MAX (mc_confg.h:67)

// densities_init (mc_estim.cc:236-255)
struct Bins {
  double dr, dth, dch, rmin;
  Bins()
  {
    dr = (PIMC_DENS_MAX_RADIUS - PIMC_DENS_MIN_RADIUS) / (double)PIMC_BINSR;
    dth = M_PI / (double)(PIMC_BINST - 1);
    dch = 2.0 * M_PI / (double)(PIMC_BINSC - 1);
    rmin = PIMC_DENS_MIN_RADIUS;
  }
  double r(int ir) const
  {
    double v = (double)ir * dr;
    v += (0.5 * dr);
    v += rmin;
    return v;
  }
  double theta(int it) const
  {
    double v = (double)it * dth;
    v += (0.5 * dth);
    return v;
  }
  double chi(int ic) const
  {
    double v = (double)ic * dch;
    v += (0.5 * dch);
    return v;
  }
};

struct Out {
  FILE *f = nullptr;
  Out(const std::string &path, bool append) { f = fopen(path.c_str(), append ? "a" : "w"); }
  ~Out()
  {
    if (f) fclose(f);
  }
  void num(double v) { fprintf(f, "%*.*e%s", kWidth, 6, v, kBlank); }
  void integer(long v, int w) { fprintf(f, "%*ld%s", w, v, kBlank); }
  void end() { fputc('\n', f); }
};

int atom_types(const pimc_system *s)
{
  int n = 0;
  for (int t = 0; t < s->ntypes; t++)
    if (s->type[t].molecule == PIMC_ATOM) n++;
  return n;
}

// the molecule type (IMTYPE) and its kind, or -1 without an impurity
int impurity(const pimc_system *s, int *kind)
{
  for (int t = 0; t < s->ntypes; t++)
    if (s->type[t].molecule != PIMC_ATOM) {
      *kind = s->type[t].molecule;
      return t;
    }
  *kind = 0;
  return -1;
}

bool valid(const pimc_system *s, const char *fname)
{
  return s && fname && s->ntypes >= 1 && s->ntypes <= PIMC_MAX_TYPES && s->nslices > 0;
}

}  // namespace

// SaveDensities1D (mc_estim.cc:1327-1443): .gra, and with a linear impurity
// its radial (.gri) and angular (.grt) densities from the 2D histogram.
extern "C" pimc_status pimc_save_densities_1d(const pimc_system *s, const char *fname, double acount,
                                              const double *gr1d, const double *gr2d)
{
  if (!valid(s, fname) || !gr1d) return PIMC_ERR_BAD_ARG;
  const Bins b;
  const int nd1 = atom_types(s), P = s->nslices;
  int kind = 0;
  impurity(s, &kind);
  {
    Out o(std::string(fname) + ".gra", false);
    if (!o.f) return PIMC_ERR_BAD_ARG;
    double volume = 1.0;
    for (int d = 0; d < 3; d++) volume *= s->box[d];
    const double norm0 = 2.0 * M_PI * b.dr * acount * (double)P / volume;
    for (int ir = 0; ir < PIMC_BINSR; ir++) {
      const double r = b.r(ir), r2 = r * r;
      o.num(r);
      for (int id = 0; id < nd1; id++) {
        const double nfact = norm0 * (double)(s->type[id].numb * (s->type[id].numb - 1));
        o.num(gr1d[(size_t)id * PIMC_BINSR + ir] / (r2 * nfact));
      }
      o.end();
    }
  }
  if (kind != PIMC_LINEAR) return PIMC_OK;
  if (!gr2d) return PIMC_ERR_BAD_ARG;
  auto g2 = [&](int id, int ir, int it) { return gr2d[((size_t)id * PIMC_BINSR + ir) * PIMC_BINST + it]; };
  {
    Out o(std::string(fname) + ".gri", false);
    if (!o.f) return PIMC_ERR_BAD_ARG;
    double norm1 = b.dr * (double)P * acount;
    norm1 *= (4.0 * M_PI * pow(1.0, 3.0));
    for (int ir = 0; ir < PIMC_BINSR; ir++) {
      const double r = b.r(ir), r2 = r * r;
      o.num(r);
      for (int id = 0; id < nd1; id++) {
        double densr = 0.0;
        for (int it = 0; it < PIMC_BINST; it++) densr += g2(id, ir, it);
        o.num(densr / (norm1 * r2));
      }
      o.end();
    }
  }
  {
    Out o(std::string(fname) + ".grt", false);
    if (!o.f) return PIMC_ERR_BAD_ARG;
    const double norm2 = (double)P * acount * b.dth;
    for (int it = 0; it < PIMC_BINST; it++) {
      o.num(b.theta(it) * 180.0 / M_PI);
      for (int id = 0; id < nd1; id++) {
        double denst = 0.0;
        for (int ir = 0; ir < PIMC_BINSR; ir++) denst += g2(id, ir, it);
        o.num(denst / (norm2 * (double)s->type[id].numb));
      }
      o.end();
    }
  }
  return PIMC_OK;
}

// SaveGraSum (mc_estim.cc:1288-1325): _sum.gra, the accumulated pair
// distributions normalised to one over r (no Jacobian)
extern "C" pimc_status pimc_save_gra_sum(const pimc_system *s, const char *fname, double acount, const double *gr1d)
{
  if (!valid(s, fname) || !gr1d) return PIMC_ERR_BAD_ARG;
  const Bins b;
  const int nd1 = atom_types(s);
  Out o(std::string(fname) + "_sum.gra", false);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  const double norma = b.dr * acount * (double)(s->nslices);
  for (int ir = 0; ir < PIMC_BINSR; ir++) {
    o.num(b.r(ir));
    for (int id = 0; id < nd1; id++)
      o.num(gr1d[(size_t)id * PIMC_BINSR + ir] / (norma * (s->type[id].numb * (s->type[id].numb - 1)) / 2.0));
    o.end();
  }
  return PIMC_OK;
}

// SaveDensities2D (mc_estim.cc:1666-1726): .g2d (mode 1: _sum.g2d) with a
// linear impurity
extern "C" pimc_status pimc_save_densities_2d(const pimc_system *s, const char *fname, double acount, int mode,
                                              const double *gr2d)
{
  if (!valid(s, fname) || !gr2d || (mode != 0 && mode != 1)) return PIMC_ERR_BAD_ARG;
  int kind = 0;
  impurity(s, &kind);
  if (kind != PIMC_LINEAR) return PIMC_OK;
  const Bins b;
  const int nd2 = atom_types(s);
  Out o(std::string(fname) + (mode ? "_sum" : "") + ".g2d", false);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  const double norm3 = b.dr * b.dth * (double)s->nslices * acount;
  for (int it = 0; it < PIMC_BINST; it++) {
    const double theta = b.theta(it);
    for (int ir = 0; ir < PIMC_BINSR; ir++) {
      const double r = b.r(ir);
      for (int id = 0; id < nd2; id++) {
        o.num(theta * 180.0 / M_PI);
        o.num(r);
        o.num(gr2d[((size_t)id * PIMC_BINSR + ir) * PIMC_BINST + it] / (norm3));
      }
      o.end();
    }
  }
  return PIMC_OK;
}

// SaveDensities3D (mc_estim.cc:1728-1800): .g3d (mode 1: _sum.g3d) with a
// nonlinear impurity; the density types are the atom types and the molecule
extern "C" pimc_status pimc_save_densities_3d(const pimc_system *s, const char *fname, double acount, int mode,
                                              const double *gr3d)
{
  if (!valid(s, fname) || !gr3d || (mode != 0 && mode != 1)) return PIMC_ERR_BAD_ARG;
  int kind = 0;
  impurity(s, &kind);
  if (kind != PIMC_NONLINEAR) return PIMC_OK;
  const Bins b;
  const int nd3 = atom_types(s) + 1;
  const size_t nb = (size_t)PIMC_BINSR * PIMC_BINST * PIMC_BINSC;
  Out o(std::string(fname) + (mode ? "_sum" : "") + ".g3d", false);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  const double norm5 = b.dr * b.dth * b.dch * (double)s->nslices * acount;
  for (int ir = 0; ir < PIMC_BINSR; ir++) {
    const double r = b.r(ir);
    for (int it = 0; it < PIMC_BINST; it++) {
      const double theta = b.theta(it);
      for (int ic = 0; ic < PIMC_BINSC; ic++) {
        const double chi = b.chi(ic);
        for (int id = 0; id < nd3; id++) {
          o.num(r);
          o.num(theta * 180.0 / M_PI);
          o.num(chi * 180.0 / M_PI);
          const size_t ijk = ((size_t)ir * PIMC_BINST + it) * PIMC_BINSC + ic;
          o.num(gr3d[id * nb + ijk] / (norm5 * r * r * sin(theta)));
        }
        o.end();
      }
    }
  }
  return PIMC_OK;
}

// SaveRho1D (mc_estim.cc:1445-1590): the radial (.gri), theta (.grt) and chi
// (.grc) densities around a nonlinear impurity from the 3D histogram (mode 1:
// _sum before the extension).  The relative-Euler-angle files it adds in
// mode 1 come from histograms of the rotational slices that the estimator
// path does not keep and are not written.
extern "C" pimc_status pimc_save_rho_1d(const pimc_system *s, const char *fname, double acount, int mode,
                                        const double *gr3d)
{
  if (!valid(s, fname) || !gr3d || (mode != 0 && mode != 1)) return PIMC_ERR_BAD_ARG;
  int kind = 0;
  impurity(s, &kind);
  if (kind != PIMC_NONLINEAR) return PIMC_OK;
  const Bins b;
  const int nd3 = atom_types(s) + 1, P = s->nslices;
  const size_t nb = (size_t)PIMC_BINSR * PIMC_BINST * PIMC_BINSC;
  const std::string stem = std::string(fname) + (mode ? "_sum" : "");
  auto g3 = [&](int id, int ir, int it, int ic) {
    return gr3d[id * nb + ((size_t)ir * PIMC_BINST + it) * PIMC_BINSC + ic];
  };
  {
    Out o(stem + ".gri", false);
    if (!o.f) return PIMC_ERR_BAD_ARG;
    const double norm1 = b.dr * (double)P * acount;
    for (int ir = 0; ir < PIMC_BINSR; ir++) {
      o.num(b.r(ir));
      for (int id = 0; id < nd3; id++) {
        double densr = 0.0;
        for (int it = 0; it < PIMC_BINST; it++)
          for (int ic = 0; ic < PIMC_BINSC; ic++) densr += g3(id, ir, it, ic);
        o.num(densr / (norm1));
      }
      o.end();
    }
  }
  {
    Out o(stem + ".grt", false);
    if (!o.f) return PIMC_ERR_BAD_ARG;
    const double norm2 = (double)P * acount * b.dth * (180.0 / M_PI);
    for (int it = 0; it < PIMC_BINST; it++) {
      o.num(b.theta(it) * 180.0 / M_PI);
      for (int id = 0; id < nd3; id++) {
        double denst = 0.0;
        for (int ir = 0; ir < PIMC_BINSR; ir++)
          for (int ic = 0; ic < PIMC_BINSC; ic++) denst += g3(id, ir, it, ic);
        o.num(denst / (norm2 * (double)s->type[id].numb));
      }
      o.end();
    }
  }
  {
    Out o(stem + ".grc", false);
    if (!o.f) return PIMC_ERR_BAD_ARG;
    const double norm4 = (double)P * acount * b.dch * (180. / M_PI);
    for (int ic = 0; ic < PIMC_BINSC; ic++) {
      o.num(b.chi(ic) * 180.0 / M_PI);
      for (int id = 0; id < nd3; id++) {
        double densc = 0.0;
        for (int ir = 0; ir < PIMC_BINSR; ir++)
          for (int it = 0; it < PIMC_BINST; it++) densc += g3(id, ir, it, ic);
        o.num(densc / (norm4 * (double)s->type[id].numb));
      }
      o.end();
    }
  }
  return PIMC_OK;
}

// SaveRhoThetaChi (mc_estim.cc:1930-1996): the (theta, chi) density around a
// nonlinear impurity (.gtc, mode 1: _sum.gtc) from the 3D histogram summed
// over r; a blank line after each theta row.
extern "C" pimc_status pimc_save_rho_theta_chi(const pimc_system *s, const char *fname, double acount, int mode,
                                               const double *gr3d)
{
  if (!valid(s, fname) || !gr3d || (mode != 0 && mode != 1)) return PIMC_ERR_BAD_ARG;
  int kind = 0;
  impurity(s, &kind);
  if (kind != PIMC_NONLINEAR) return PIMC_OK;
  const Bins b;
  const int nd3 = atom_types(s) + 1;
  const size_t nb = (size_t)PIMC_BINSR * PIMC_BINST * PIMC_BINSC;
  Out o(std::string(fname) + (mode ? "_sum" : "") + ".gtc", false);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  const double norm6 = b.dth * b.dch * (double)s->nslices * acount * (180.0 * 180.0 / (M_PI * M_PI));
  for (int it = 0; it < PIMC_BINST; it++) {
    const double theta = b.theta(it);
    for (int ic = 0; ic < PIMC_BINSC; ic++) {
      const double chi = b.chi(ic);
      o.num(theta * 180.0 / M_PI);
      o.num(chi * 180.0 / M_PI);
      for (int id = 0; id < nd3; id++) {
        double denstc = 0.0;
        for (int ir = 0; ir < PIMC_BINSR; ir++)
          denstc = denstc + gr3d[id * nb + ((size_t)ir * PIMC_BINST + it) * PIMC_BINSC + ic];
        o.num(denstc / (norm6 * (double)s->type[id].numb));
      }
      o.end();
    }
    o.end();
  }
  return PIMC_OK;
}

// The relative-Euler-angle files SaveRho1D adds at the end of the run
// (mc_estim.cc:1590-1660): _sum.eulphi and _sum.eulchi (chi-width bins),
// _sum.eulthe (theta bins), each line the bin centre in degrees and the count
// over Q acount times the bin width in degrees.
extern "C" pimc_status pimc_save_rel_euler(const pimc_system *s, const char *fname, double acount, const double *the,
                                           const double *phi, const double *chi)
{
  if (!valid(s, fname) || !the || !phi || !chi || s->nrotslices <= 0) return PIMC_ERR_BAD_ARG;
  const Bins b;
  const double norm5 = (double)s->nrotslices * acount * b.dch * (180. / M_PI);
  const double norm6 = (double)s->nrotslices * acount * b.dth * (180.0 / M_PI);
  const char *ext[2] = {".eulphi", ".eulchi"};
  const double *h[2] = {phi, chi};
  for (int k = 0; k < 2; k++) {
    Out o(std::string(fname) + "_sum" + ext[k], false);
    if (!o.f) return PIMC_ERR_BAD_ARG;
    for (int i = 0; i < PIMC_BINSC; i++) {
      o.num(b.chi(i) * 180.0 / M_PI);
      fprintf(o.f, "%*.*e\n", kWidth, 6, h[k][i] / norm5);
    }
  }
  Out o(std::string(fname) + "_sum.eulthe", false);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  for (int i = 0; i < PIMC_BINST; i++) {
    o.num(b.theta(i) * 180.0 / M_PI);
    fprintf(o.f, "%*.*e\n", kWidth, 6, the[i] / norm6);
  }
  return PIMC_OK;
}

// SaveExchangeLength (mc_estim.cc:2021-2085): one appended .prl line per
// block -- the block number, the ground-state-loop and excited-loop weights
// and their sum, the normalised count of every cycle length, PIndex and the
// PrintXYZprl flag.  bstype is the boson type (BSTYPE).
extern "C" pimc_status pimc_save_exchange_length(const pimc_system *s, const char *fname, double acount,
                                                 long blocknumb, int bstype, const double *ploops, const int *pindex,
                                                 int print_xyz_prl)
{
  if (!valid(s, fname) || !ploops || !pindex || bstype < 0 || bstype >= s->ntypes) return PIMC_ERR_BAD_ARG;
  const int numb = s->type[bstype].numb;
  Out o(std::string(fname) + ".prl", true);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  o.integer(blocknumb, kWidthBlock);
  double excited = 0.0, ground = 0.0;
  for (int cl = 0; cl < numb; cl++) {
    const double norm = (double)(cl + 1) / (acount * (double)numb);
    if (cl <= kGsLoopMax) excited += (ploops[cl] * norm);
    else ground += (ploops[cl] * norm);
  }
  o.num(ground);
  o.num(excited);
  o.num(ground + excited);
  for (int cl = 0; cl < numb; cl++) {
    const double norm = (double)(cl + 1) / (acount * (double)numb);
    o.num(ploops[cl] * norm);
  }
  o.end();
  for (int a = 0; a < numb; a++) o.integer(pindex[a], kWidth);
  fprintf(o.f, "%d", print_xyz_prl);
  o.end();
  return PIMC_OK;
}

// SaveAreaEstimators (mc_estim.cc:2596-2641): one appended .sup line per
// block from the summed pimc_area_estimators increments sums[6] =
// _areas[PERP,PARL], _area2[PERP,PARL], _inert[PERP,PARL]; mass of the boson
// type in amu.
extern "C" pimc_status pimc_save_area_estimators(const pimc_system *s, const char *fname, double acount,
                                                 long blocknumb, int bstype, const double *sums, double mass)
{
  if (!valid(s, fname) || !sums || bstype < 0 || bstype >= s->ntypes || !(s->temperature > 0.0))
    return PIMC_ERR_BAD_ARG;
  const double lambda = s->type[bstype].lambda, beta = 1.0 / s->temperature;
  const double norm = 2.0 / (beta * lambda);
  const double *areas = sums, *area2 = sums + 2, *inert = sums + 4;
  Out o(std::string(fname) + ".sup", true);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  o.integer(blocknumb, kWidthBlock);
  o.num(area2[0] * norm / inert[0]);
  o.num(area2[1] * norm / inert[1]);
  const double units = 1.0 * 1.0 * 1.0;
  o.num(inert[0] * units * mass / acount);
  o.num(inert[1] * units * mass / acount);
  o.num(areas[0] * sqrt(norm / inert[0]) / acount);
  o.num(areas[1] * sqrt(norm / inert[1]) / acount);
  o.end();
  return PIMC_OK;
}

// SaveAreaEstim3D (mc_estim.cc:2670-2720): one appended .sffs3d (iframe 0)
// or .mffs3d (iframe 1) line per block from the summed pimc_area_estim3d
// increments: areas[6] of _areas3D and inert[9] of _inert3D.
extern "C" pimc_status pimc_save_area_estim3d(const pimc_system *s, const char *fname, double acount,
                                              long blocknumb, int iframe, int bstype, const double *areas,
                                              const double *inert, double mass)
{
  if (!valid(s, fname) || !areas || !inert || (iframe != 0 && iframe != 1) || bstype < 0 || bstype >= s->ntypes ||
      !(s->temperature > 0.0))
    return PIMC_ERR_BAD_ARG;
  const double lambda = s->type[bstype].lambda, beta = 1.0 / s->temperature;
  const double norm = 2.0 * mass / (beta * lambda);
  Out o(std::string(fname) + (iframe ? ".mffs3d" : ".sffs3d"), true);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  o.integer(blocknumb, kWidthBlock);
  for (int i = 0; i < 9; i++) o.num(inert[i] / (double)acount);
  for (int i = 0; i < 6; i++) o.num(areas[i] * norm / (double)acount);
  o.end();
  return PIMC_OK;
}

// SaveRCF (mc_estim.cc:1141-1189): the .rcf file (mode 1: _sum.rcf) of the
// rotational correlation functions.  rcf[10][Q] are the ten rows of GetRCF's
// accumulator summed over the samples (mc_estim.cc:1099-1139): row 0 the sum
// of n(0).n(tau) (pimc_rcf's output), rows 1..9 the Legendre rows, which the
// reference accumulates as 1 per (origin, lag) -- in its block accumulator
// only where n(0).n(tau) < 0.9999999 (PLONE, mc_confg.h:64).  Q + 1 lines of
// the imaginary time it*tau_rot (tau_rot = beta/Q, mc_setup.cc:377) and row 0
// over acount Q, two blank lines, a "#" line, then Q + 1 lines of the time
// and rows 1..9 over acount Q.
extern "C" pimc_status pimc_save_rcf(const pimc_system *s, const char *fname, double acount, int mode,
                                     const double *rcf)
{
  if (!valid(s, fname) || !rcf || (mode != 0 && mode != 1) || s->nrotslices <= 0 || !(s->temperature > 0.0))
    return PIMC_ERR_BAD_ARG;
  const int Q = s->nrotslices, nrcf = 10;      // NUMB_RCF (mc_confg.h:58)
  const double beta = 1.0 / s->temperature, rtau = beta / (double)Q;
  Out o(std::string(fname) + (mode ? "_sum" : "") + ".rcf", false);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  const double norm = acount * (double)Q;
  for (int it = 0; it <= Q; it++) {
    o.num((double)it * rtau);
    o.num(rcf[it % Q] / norm);
    o.end();
  }
  fputs("\n\n#\n", o.f);
  for (int it = 0; it <= Q; it++) {
    o.num((double)it * rtau);
    for (int ip = 1; ip < nrcf; ip++) o.num(rcf[(size_t)ip * Q + it % Q] / norm);
    o.end();
  }
  return PIMC_OK;
}

// MCGetAverage's per-sample energy terms (mc_main.cc:551-616) from
// pimc_estimators' out[5] = {E_kin, E_pot, E_rot, ErotSQ, Erot_termSQ},
// added to the block sums[7] = {_bkin, _bpot, _brot, _brotsq, _bCv,
// _bCv_trans, _bCv_rot}; E_rot and ErotSQ count only with ROTATION.
// beta = 1/T, tau = beta/P (mc_setup.cc:373-377), N = all atoms, NDIM = 3.
extern "C" pimc_status pimc_energy_accumulate(const pimc_system *s, const double *est, double *sums)
{
  if (!valid(s, "") || !est || !sums || !(s->temperature > 0.0)) return PIMC_ERR_BAD_ARG;
  int natoms = 0;
  for (int t = 0; t < s->ntypes; t++) natoms += s->type[t].numb;
  const double beta = 1.0 / s->temperature, tau = beta / (double)s->nslices;
  const double skin = est[0], spot = est[1];
  double srot = 0.0;
  sums[0] += skin;
  sums[1] += spot;
  if (s->rotation) {
    srot = est[2];
    sums[2] += srot;
    sums[3] += est[3];
  }
  const double d = (double)(3 * natoms);
  const double sCv = -0.5 * d / (beta * tau) - (d * 0.5 / tau - skin - spot - srot) * (d * 0.5 / tau - skin - spot - srot) +
                     (2.0 / beta) * (0.5 * d / tau - skin) + est[4] - est[3];
  const double sCv_trans = -0.5 * d / (beta * tau) - (d * 0.5 / tau - skin) * (d * 0.5 / tau - skin) +
                           (2.0 / beta) * (0.5 * d / tau - skin);
  const double sCv_rot = -srot * srot + est[4] - est[3];
  sums[4] += sCv;
  sums[5] += sCv_trans;
  sums[6] += sCv_rot;
  return PIMC_OK;
}

// SaveEnergy (mc_main.cc:764-795): one appended .eng line per block from the
// block sums of pimc_energy_accumulate over acount samples -- the block
// number, E_kin, E_pot, E_kin + E_pot, E_rot, ErotSQ, the total, Cv, Cv_trans
// and Cv_rot, each over acount.
extern "C" pimc_status pimc_save_energy(const pimc_system *s, const char *fname, double acount, long blocknumb,
                                        const double *sums)
{
  if (!valid(s, fname) || !sums) return PIMC_ERR_BAD_ARG;
  Out o(std::string(fname) + ".eng", true);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  const double e = 1.0;                         // Units.energy
  o.integer(blocknumb, kWidthBlock);
  o.num(sums[0] * e / acount);
  o.num(sums[1] * e / acount);
  o.num((sums[0] + sums[1]) * e / acount);
  o.num(sums[2] * e / acount);
  o.num(sums[3] * (e * e) / acount);
  o.num((sums[0] + sums[1] + sums[2]) * e / acount);
  o.num(sums[4] / acount);
  o.num(sums[5] / acount);
  o.num(sums[6] / acount);
  o.end();
  return PIMC_OK;
}

// SaveSumEnergy (mc_main.cc:797-836): one line of the run's _sum.eng (opened
// for writing at the start of the run, mc_main.cc:838-872: append = 0 for the
// first line, 1 after) from the run sums of pimc_energy_accumulate over
// acount samples: numb (the block count, printed as the reference prints a
// double), E_kin, E_pot, their sum, E_rot, ErotSQ, the total, then the heat
// capacities -beta/T [(3 N P T / 2 - <E>)^2 + <Cv terms>] for the total, the
// translational part and (with -<E_rot> in place of the first term) the rotor.
extern "C" pimc_status pimc_save_sum_energy(const pimc_system *s, const char *fname, double acount, double numb,
                                            const double *sums, int append)
{
  if (!valid(s, fname) || !sums || !(s->temperature > 0.0)) return PIMC_ERR_BAD_ARG;
  int natoms = 0;
  for (int t = 0; t < s->ntypes; t++) natoms += s->type[t].numb;
  const double T = s->temperature, beta = 1.0 / T, e = 1.0;   // Units.energy
  Out o(std::string(fname) + "_sum.eng", append != 0);
  if (!o.f) return PIMC_ERR_BAD_ARG;
  fprintf(o.f, "%*.*e%s", kWidthBlock, 6, numb, kBlank);
  o.num(sums[0] * e / acount);
  o.num(sums[1] * e / acount);
  o.num((sums[0] + sums[1]) * e / acount);
  o.num(sums[2] * e / acount);
  o.num(sums[3] * (e * e) / acount);
  o.num((sums[0] + sums[1] + sums[2]) * e / acount);
  const double npt = (double)(3 * natoms * s->nslices * T);
  double cv = 0.5 * npt - (sums[0] + sums[1] + sums[2]) * e / acount;
  cv = cv * cv + sums[4] * e * e / acount;
  cv = -cv * beta / T;
  o.num(cv);
  double cvt = 0.5 * npt - sums[0] * e / acount;
  cvt = cvt * cvt + sums[5] * e * e / acount;
  cvt = -cvt * beta / T;
  o.num(cvt);
  double cvr = -sums[2] * e / acount;
  cvr = cvr * cvr + sums[6] * e * e / acount;
  cvr = -cvr * beta / T;
  o.num(cvr);
  o.end();
  return PIMC_OK;
}

