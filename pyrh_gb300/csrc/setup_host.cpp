// setup_host.cpp -- host-side set-up of the radiative-transfer path: the
// RH model-atom reader, the wavelength grids of the active transitions, the
// global wavelength grid with each transition's range, the output index that
// drops the reference wavelength, and the hydrogenic bound-free
// cross-sections on that grid.
//
// Reference routines restated here (file:line in the reference tree):
//   readAtom          rh/readatom.c:62-470   (levels, lines, continua; the
//                                             collision block is kept as
//                                             tabulated records)
//   getLambda         rh/getlambda.c:44-162  (line grids, qcore/qwing spacing)
//   getLambdaCont     rh/getlambda.c:166-180
//   determinate, Lande, effectiveLande       rh/zeeman.c:37-140
//   SortLambda        rh/sortlambda.c:42-420 (union, sort, strict dedupe,
//                                             Hunt of each transition's ends,
//                                             hydrogenic alpha)
//   Gaunt_bf          rh/hydrogen.c:269-281
//   output grid       rh/rhf1d/pyrh_solveray.c:115-156 (lambda_ref dropped)
// Every expression keeps the reference's operation order and its constants
// (rh/constant.h), so the grids and integer ranges come out bit-identical.
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/pyrh_gb300.h"

namespace pyrh {
void set_error(const char* fmt, ...);
}

namespace {

// rh/constant.h values (old CODATA, as the reference uses them)
constexpr double kC = 2.99792458E+08;
constexpr double kH = 6.6260755E-34;
constexpr double kQe = 1.60217733E-19;
constexpr double kEps0 = 8.854187817E-12;
constexpr double kMe = 9.1093897E-31;
constexpr double kERyd = 2.1798741E-18;
constexpr double kPi = 3.14159265358979;
constexpr double kNm = 1.0E-09;
constexpr double kCm = 1.0E-02;

pyrh_status fail(pyrh_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  pyrh::set_error("%s", buf);
  return s;
}

// getLine of the reference: the next line that is neither empty nor a
// comment ('#' in the first column).
struct Lines {
  const char* p;
  bool next(std::string& out) {
    while (*p) {
      const char* e = strchr(p, '\n');
      const size_t n = e ? (size_t)(e - p) : strlen(p);
      std::string s(p, n);
      p = e ? e + 1 : p + n;
      if (s.empty() || s[0] == '#') continue;
      bool blank = true;
      for (char c : s)
        if (!isspace((unsigned char)c)) { blank = false; break; }
      if (blank) continue;
      out = s;
      return true;
    }
    return false;
  }
};

// getOrbital (rh/zeeman.c): spectroscopic letter to L
int orbital(char c) {
  static const char kLetters[] = "SPDFGHIKLMNOQRTUV";
  const char* q = strchr(kLetters, c);
  return q ? (int)(q - kLetters) : -1;
}

std::vector<std::string> words(const char* s) {
  std::vector<std::string> w;
  std::string cur;
  for (; *s; ++s) {
    if (*s == ' ') {
      if (!cur.empty()) w.push_back(cur), cur.clear();
    } else {
      cur += *s;
    }
  }
  if (!cur.empty()) w.push_back(cur);
  return w;
}

// determinate (rh/zeeman.c:37-82): S, L, J of a level from its label
bool determinate(const char* label, double g, double* S, int* L, double* J) {
  char multiplet[64];
  snprintf(multiplet, sizeof multiplet, "%s", label);
  char* ptr = multiplet + (strlen(multiplet) - 1);
  while ((*ptr != 'E') && (*ptr != 'O') && (ptr > multiplet)) ptr--;
  if (ptr > multiplet) *(ptr + 1) = '\0';
  else return false;
  std::vector<std::string> w = words(multiplet);
  if (w.size() < 2) return false;
  const std::string& last = w.back();
  if (last.size() < 3) return false;
  int multiplicity = 0;
  char orbit[8] = {0};
  if (sscanf(last.c_str() + last.size() - 3, "%d%7s", &multiplicity, orbit) != 2) return false;
  *S = (multiplicity - 1) / 2.0;
  *L = orbital(orbit[0]);
  *J = (g - 1.0) / 2.0;
  if (*L < 0) return false;
  if (*J > *L + *S) return false;
  return true;
}

// Lande (rh/zeeman.c:128-135)
double lande(double S, int L, double J) {
  if (J == 0.0) return 0.0;
  return 1.5 + (S * (S + 1.0) - L * (L + 1)) / (2.0 * J * (J + 1.0));
}

// Locate (bisection for the interval containing x in an ascending table)
int locate(int n, const double* xt, double x) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (hi + lo) >> 1;
    if (x >= xt[mid]) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Hunt with an exact member of an ascending array: the index of the value
// (the largest index whose element is <= value).
int hunt_exact(int n, const double* a, double v) { return locate(n, a, v); }

}  // namespace

extern "C" {

pyrh_status pyrh_atom_read(const char* text, pyrh_atom* a) {
  if (!text || !a) return fail(PYRH_ERR_ARG, "atom text or output is NULL");
  memset(a, 0, sizeof(*a));
  Lines in{text};
  std::string s;
  if (!in.next(s)) return fail(PYRH_ERR_ARG, "atom: missing ID");
  char id[8] = {0};
  if (sscanf(s.c_str(), "%2s", id) != 1) return fail(PYRH_ERR_ARG, "atom: bad ID line");
  for (int n = 0; id[n]; ++n) id[n] = (char)toupper((unsigned char)id[n]);
  if (strlen(id) == 1) strcat(id, " ");
  memcpy(a->id, id, 3);
  if (!in.next(s) ||
      sscanf(s.c_str(), "%d %d %d %d", &a->nlevel, &a->nline, &a->ncont, &a->nfixed) != 4)
    return fail(PYRH_ERR_ARG, "atom: bad count line");
  if (a->nlevel < 2 || a->nlevel > PYRH_ATOM_MAX_LEVELS || a->nline < 0 ||
      a->nline > PYRH_ATOM_MAX_LINES || a->ncont < 0 || a->ncont > PYRH_ATOM_MAX_CONT ||
      a->nfixed < 0)
    return fail(PYRH_ERR_UNSUPPORTED, "atom: %d levels / %d lines / %d continua beyond limits",
                a->nlevel, a->nline, a->ncont);
  for (int i = 0; i < a->nlevel; ++i) {
    pyrh_atom_level& L = a->level[i];
    if (!in.next(s)) return fail(PYRH_ERR_ARG, "atom: missing level %d", i);
    char label[PYRH_ATOM_LABEL + 1];
    memset(label, 0, sizeof label);
    int dummy = 0, abo = -1;
    const int nr = sscanf(s.c_str(), "%lf %lf '%20c' %d %d %d", &L.E, &L.g, label, &L.stage,
                          &dummy, &abo);
    if (nr < 4) return fail(PYRH_ERR_ARG, "atom: bad level line %d", i);
    memcpy(L.label, label, PYRH_ATOM_LABEL);
    L.abo_level = abo;
    L.E_cm = L.E;
    L.E *= (kH * kC) / kCm;
  }
  if (a->level[a->nlevel - 1].stage != a->level[a->nlevel - 2].stage + 1)
    return fail(PYRH_ERR_ARG, "atom %s has no overlying continuum", a->id);
  const double Cfac = 2 * kPi * (kQe / kEps0) * (kQe / kMe) / kC;
  for (int kr = 0; kr < a->nline; ++kr) {
    pyrh_atom_line& l = a->line[kr];
    if (!in.next(s)) return fail(PYRH_ERR_ARG, "atom: missing line %d", kr);
    int i = 0, j = 0;
    char shape[32] = {0}, symm[32] = {0}, vdw[32] = {0};
    const int nr = sscanf(s.c_str(), "%d %d %lf %31s %d %31s %lf %lf %31s %lf %lf %lf %lf %lf %lf %lf",
                          &j, &i, &l.f, shape, &l.nlambda, symm, &l.qcore, &l.qwing, vdw,
                          &l.cvdw[0], &l.cvdw[1], &l.cvdw[2], &l.cvdw[3], &l.Grad, &l.cStark,
                          &l.g_lande_eff);
    if (nr < 15) return fail(PYRH_ERR_ARG, "atom: bad line record %d", kr);
    if (nr == 15) l.g_lande_eff = 0.0;
    l.j = std::max(i, j);
    l.i = std::min(i, j);
    if (l.i < 0 || l.j >= a->nlevel || l.i == l.j)
      return fail(PYRH_ERR_ARG, "atom: line %d between levels %d and %d", kr, i, j);
    const pyrh_atom_level &li = a->level[l.i], &lj = a->level[l.j];
    const double lambda0 = (kH * kC) / (lj.E - li.E);
    l.Aji = Cfac / ((lambda0) * (lambda0)) * (li.g / lj.g) * l.f;
    l.Bji = ((lambda0) * (lambda0) * (lambda0)) / (2.0 * kH * kC) * l.Aji;
    l.Bij = (lj.g / li.g) * l.Bji;
    l.lambda0 = lambda0 / kNm;
    if (!strstr(shape, "PRD") && !strstr(shape, "VOIGT") && !strstr(shape, "GAUSS") &&
        !strstr(shape, "COMPOSIT"))
      return fail(PYRH_ERR_ARG, "atom: line shape %s", shape);
    l.prd = strstr(shape, "PRD") != nullptr;
    l.voigt = strstr(shape, "GAUSS") == nullptr;
    l.ncomponent = 1;
    l.c_shift[0] = 0.0;
    l.c_fraction[0] = 1.0;
    if (strstr(shape, "COMPOSIT")) {
      if (!in.next(s) || sscanf(s.c_str(), "%d", &l.ncomponent) != 1 || l.ncomponent < 1 ||
          l.ncomponent > PYRH_ATOM_MAX_COMPONENTS)
        return fail(PYRH_ERR_UNSUPPORTED, "atom: composite line %d component count", kr);
      for (int n = 0; n < l.ncomponent; ++n)
        if (!in.next(s) || sscanf(s.c_str(), "%lf %lf", &l.c_shift[n], &l.c_fraction[n]) != 2)
          return fail(PYRH_ERR_ARG, "atom: composite line %d component %d", kr, n);
    }
    if (strstr(vdw, "PARAMTR")) l.vdwaals = PYRH_ATOM_VDW_RIDDER_RENSBERGEN;
    else if (strstr(vdw, "UNSOLD")) {
      l.vdwaals = PYRH_ATOM_VDW_UNSOLD;
      l.cvdw[3] = l.cvdw[1] = 0.0;
    } else if (strstr(vdw, "BARKLEM")) l.vdwaals = PYRH_ATOM_VDW_BARKLEM;
    else return fail(PYRH_ERR_ARG, "atom: van der Waals type %s", vdw);
    l.symmetric = strstr(symm, "ASYMM") ? 0 : 1;
  }
  int ntab = 0;
  for (int kr = 0; kr < a->ncont; ++kr) {
    pyrh_atom_cont& c = a->cont[kr];
    if (!in.next(s)) return fail(PYRH_ERR_ARG, "atom: missing continuum %d", kr);
    int i = 0, j = 0;
    char dep[32] = {0};
    if (sscanf(s.c_str(), "%d %d %lf %d %31s %lf", &j, &i, &c.alpha0, &c.nlambda, dep,
               &c.lambda_min) != 6)
      return fail(PYRH_ERR_ARG, "atom: bad continuum record %d", kr);
    c.j = std::max(i, j);
    c.i = std::min(i, j);
    if (c.i < 0 || c.j >= a->nlevel || c.nlambda < 2)
      return fail(PYRH_ERR_ARG, "atom: continuum %d", kr);
    const double lambda0 = (kH * kC) / (a->level[c.j].E - a->level[c.i].E);
    c.lambda0 = lambda0 / kNm;
    if (strstr(dep, "EXPLICIT")) {
      c.hydrogenic = 0;
      if (ntab + c.nlambda > PYRH_ATOM_MAX_TABLE)
        return fail(PYRH_ERR_UNSUPPORTED, "atom: explicit cross-section tables too long");
      c.table_off = ntab;
      for (int la = c.nlambda - 1; la >= 0; --la)
        if (!in.next(s) || sscanf(s.c_str(), "%lf %lf", &a->table_lambda[ntab + la],
                                  &a->table_alpha[ntab + la]) != 2)
          return fail(PYRH_ERR_ARG, "atom: continuum %d table row %d", kr, la);
      ntab += c.nlambda;
    } else if (strstr(dep, "HYDROGENIC")) {
      c.hydrogenic = 1;
      if (c.lambda_min >= c.lambda0)
        return fail(PYRH_ERR_ARG, "atom: continuum %d minimum wavelength above its edge", kr);
    } else {
      return fail(PYRH_ERR_ARG, "atom: wavelength dependence %s", dep);
    }
  }
  a->ntable = ntab;
  for (int kf = 0; kf < a->nfixed; ++kf)
    if (!in.next(s)) return fail(PYRH_ERR_ARG, "atom: missing fixed transition %d", kf);
  // collision block: tabulated records on the latest TEMP grid
  int ntemp = 0, tempoff = -1, nvals = 0;
  while (in.next(s)) {
    char key[32] = {0};
    if (sscanf(s.c_str(), "%31s", key) != 1) continue;
    if (!strcmp(key, "END")) break;
    const char* rest = s.c_str() + s.find(key) + strlen(key);
    if (!strcmp(key, "TEMP")) {
      int n = 0, used = 0;
      if (sscanf(rest, "%d%n", &n, &used) != 1 || n < 1 || nvals + n > PYRH_ATOM_MAX_COLLVALS)
        return fail(PYRH_ERR_UNSUPPORTED, "atom: TEMP grid");
      rest += used;
      tempoff = nvals;
      for (int t = 0; t < n; ++t) {
        if (sscanf(rest, "%lf%n", &a->coll_values[nvals + t], &used) != 1)
          return fail(PYRH_ERR_ARG, "atom: TEMP value %d", t);
        rest += used;
      }
      ntemp = n;
      nvals += n;
      continue;
    }
    int type = -1;
    if (!strcmp(key, "OMEGA")) type = PYRH_COLL_OMEGA;
    else if (!strcmp(key, "CE")) type = PYRH_COLL_CE;
    else if (!strcmp(key, "CI")) type = PYRH_COLL_CI;
    else if (!strcmp(key, "CP")) type = PYRH_COLL_CP;
    else if (!strcmp(key, "CH")) type = PYRH_COLL_CH;
    else if (!strcmp(key, "CH0")) type = PYRH_COLL_CH0;
    else if (!strcmp(key, "CH+")) type = PYRH_COLL_CHP;
    else if (!strcmp(key, "CR")) type = PYRH_COLL_CR;
    else return fail(PYRH_ERR_UNSUPPORTED, "atom: collision type %s", key);
    if (a->ncoll >= PYRH_ATOM_MAX_COLL || tempoff < 0 || nvals + ntemp > PYRH_ATOM_MAX_COLLVALS)
      return fail(PYRH_ERR_UNSUPPORTED, "atom: collision records beyond limits");
    pyrh_atom_coll& c = a->coll[a->ncoll];
    int i = 0, j = 0, used = 0;
    if (sscanf(rest, "%d %d%n", &i, &j, &used) != 2)
      return fail(PYRH_ERR_ARG, "atom: collision record %s", key);
    rest += used;
    c.type = type;
    c.i = std::min(i, j);
    c.j = std::max(i, j);
    c.ntemp = ntemp;
    c.temp_off = tempoff;
    c.value_off = nvals;
    for (int t = 0; t < ntemp; ++t) {
      if (sscanf(rest, "%lf%n", &a->coll_values[nvals + t], &used) != 1)
        return fail(PYRH_ERR_ARG, "atom: collision record %s value %d", key, t);
      rest += used;
    }
    nvals += ntemp;
    a->ncoll++;
  }
  a->ncoll_values = nvals;
  return PYRH_OK;
}

double pyrh_atom_lande_eff(const pyrh_atom* a, int32_t kr) {
  // effectiveLande (rh/zeeman.c:106-125)
  const pyrh_atom_line& l = a->line[kr];
  if (l.g_lande_eff != 0.0) return l.g_lande_eff;
  double Sl, Su, Jl, Ju;
  int Ll, Lu;
  bool ok = determinate(a->level[l.i].label, a->level[l.i].g, &Sl, &Ll, &Jl);
  ok = determinate(a->level[l.j].label, a->level[l.j].g, &Su, &Lu, &Ju) && ok;
  if (!ok) return 0.0;
  const double gl = lande(Sl, Ll, Jl), gu = lande(Su, Lu, Ju);
  return 0.5 * (gu + gl) + 0.25 * (gu - gl) * (Ju * (Ju + 1.0) - Jl * (Jl + 1.0));
}

int32_t pyrh_atom_line_polarizable(const pyrh_atom* a, int32_t kr, int32_t stokes) {
  // readatom.c:347-366 (for an active atom, with atmos.Stokes)
  if (!stokes) return 0;
  const pyrh_atom_line& l = a->line[kr];
  double S, Jl, Ju;
  int L;
  if (l.g_lande_eff != 0.0 ||
      (determinate(a->level[l.i].label, a->level[l.i].g, &S, &L, &Jl) &&
       determinate(a->level[l.j].label, a->level[l.j].g, &S, &L, &Ju) && fabs(Ju - Jl) <= 1.0))
    return l.ncomponent > 1 ? -1 : 1;
  return 0;
}

int32_t pyrh_line_grid(const pyrh_atom* a, int32_t kr, const pyrh_grid_config* g, double* lam,
                       int32_t cap) {
  if (!a || !g || kr < 0 || kr >= a->nline) {
    fail(PYRH_ERR_ARG, "line grid: atom, config or line index");
    return -1;
  }
  const pyrh_atom_line& line = a->line[kr];
  if (line.qcore <= 0.0 || line.qwing <= 0.0) {
    fail(PYRH_ERR_ARG, "line %d: qcore or qwing not positive", kr);
    return -1;
  }
  const int pol = pyrh_atom_line_polarizable(a, kr, g->stokes);
  if (pol < 0) {
    fail(PYRH_ERR_UNSUPPORTED, "line %d: composite line with polarization", kr);
    return -1;
  }
  bool symmetric = line.symmetric != 0;
  if ((g->stokes && pol) || g->moving || line.ncomponent > 1) symmetric = false;
  int Nlambda;
  if (symmetric) Nlambda = (line.nlambda % 2) ? line.nlambda : line.nlambda + 1;
  else Nlambda = (line.nlambda % 2) ? (line.nlambda / 2) : (line.nlambda + 1) / 2;
  const double beta = (line.qwing <= 2.0 * line.qcore) ? 1.0 : line.qwing / (2.0 * line.qcore);
  const double y = beta + sqrt(((beta) * (beta)) + (beta - 1.0) * Nlambda + 2.0 - 3.0 * beta);
  const double b = 2.0 * log(y) / (Nlambda - 1);
  const double av = line.qwing / (Nlambda - 2.0 + ((y) * (y)));
  std::vector<double> q(Nlambda);
  for (int la = 0; la < Nlambda; la++) q[la] = av * (la + (exp(b * la) - 1.0));
  if (pol) {
    const double geff = pyrh_atom_lande_eff(a, kr);
    const double qB_char = geff * (kQe / (4.0 * kPi * kMe)) * (line.lambda0 * kNm) * g->B_char /
                           g->vmicro_char;
    const int NB = locate(Nlambda, q.data(), qB_char / 2.0);
    const double qB_shift = 2 * q[NB];
    q.resize(Nlambda + 2 * NB);
    for (int la = NB + 1; la <= 2 * NB; la++)
      q[la] = qB_shift - av * (2 * NB - la + (exp(b * (2 * NB - la)) - 1.0));
    for (int la = 2 * NB + 1; la < Nlambda + 2 * NB; la++)
      q[la] = qB_shift + av * (la - 2 * NB + (exp(b * (la - 2 * NB)) - 1.0));
    Nlambda += 2 * NB;
  }
  const double q_to_lambda = line.lambda0 * (g->vmicro_char / kC);
  const int n = symmetric ? Nlambda : (2 * Nlambda - 1) * line.ncomponent;
  if (!lam) return n;
  if (n > cap) {
    fail(PYRH_ERR_ARG, "line %d: grid of %d points exceeds capacity %d", kr, n, cap);
    return -1;
  }
  if (symmetric) {
    for (int la = 0; la < n; la++) lam[la] = line.lambda0 + q_to_lambda * q[la];
  } else {
    for (int c = 0; c < line.ncomponent; c++) {
      const int Nmid = c * (2 * Nlambda - 1) + Nlambda - 1;
      const double lambda0 = line.lambda0 + line.c_shift[c];
      lam[Nmid] = lambda0;
      for (int la = 1; la < Nlambda; la++) {
        const double dlambda = q_to_lambda * q[la];
        lam[Nmid - la] = lambda0 - dlambda;
        lam[Nmid + la] = lambda0 + dlambda;
      }
    }
    if (line.ncomponent > 1) std::sort(lam, lam + n);
  }
  return n;
}

int32_t pyrh_cont_grid(const pyrh_atom* a, int32_t kr, double* lam, int32_t cap) {
  if (!a || kr < 0 || kr >= a->ncont) {
    fail(PYRH_ERR_ARG, "continuum grid: atom or continuum index");
    return -1;
  }
  const pyrh_atom_cont& c = a->cont[kr];
  if (!lam) return c.nlambda;
  if (c.nlambda > cap) {
    fail(PYRH_ERR_ARG, "continuum %d: %d points exceed capacity %d", kr, c.nlambda, cap);
    return -1;
  }
  if (c.hydrogenic) {
    // getLambdaCont: equidistant from lambda_min to the edge, cumulative
    const double dlamb = (c.lambda0 - c.lambda_min) / (c.nlambda - 1);
    lam[0] = c.lambda_min;
    for (int la = 1; la < c.nlambda; la++) lam[la] = lam[la - 1] + dlamb;
  } else {
    for (int la = 0; la < c.nlambda; la++) lam[la] = a->table_lambda[c.table_off + la];
  }
  return c.nlambda;
}

pyrh_status pyrh_sort_lambda(const double* wave, int32_t nwave, double lambda_ref,
                             const double* grids, const int32_t* grid_n, int32_t ngrid,
                             double* lam, int32_t cap, int32_t* nspect, int32_t* wave_inds,
                             int32_t* nblue, int32_t* nlambda) {
  if ((nwave > 0 && !wave) || nwave < 0 || ngrid < 0 || (ngrid > 0 && (!grids || !grid_n)) ||
      !lam || !nspect)
    return fail(PYRH_ERR_ARG, "sort_lambda: NULL or negative argument");
  std::vector<double> all;
  if (lambda_ref > 0.0) all.push_back(lambda_ref);
  for (int i = 0; i < nwave; ++i) all.push_back(wave[i]);
  int64_t off = 0;
  std::vector<int64_t> goff(ngrid);
  for (int g = 0; g < ngrid; ++g) {
    if (grid_n[g] < 1) return fail(PYRH_ERR_ARG, "sort_lambda: grid %d is empty", g);
    goff[g] = off;
    for (int la = 0; la < grid_n[g]; ++la) all.push_back(grids[off + la]);
    off += grid_n[g];
  }
  if (all.empty()) return fail(PYRH_ERR_ARG, "sort_lambda: no wavelengths");
  std::sort(all.begin(), all.end());
  int n = 1;
  for (size_t k = 1; k < all.size(); ++k)
    if (all[k] > all[n - 1]) all[n++] = all[k];
  if (n > cap) return fail(PYRH_ERR_ARG, "sort_lambda: %d wavelengths exceed capacity %d", n, cap);
  for (int k = 0; k < n; ++k) lam[k] = all[k];
  *nspect = n;
  if (wave_inds) {
    int last = 0;
    for (int i = 0; i < nwave; ++i) {
      wave_inds[i] = -1;
      for (int k = last; k < n; ++k)
        if (lam[k] == wave[i]) {
          wave_inds[i] = k;
          last = k;
          break;
        }
    }
  }
  for (int g = 0; g < ngrid; ++g) {
    const double* gr = grids + goff[g];
    const int lo = hunt_exact(n, lam, gr[0]), hi = hunt_exact(n, lam, gr[grid_n[g] - 1]);
    if (nblue) nblue[g] = lo;
    if (nlambda) nlambda[g] = hi - lo + 1;
  }
  return PYRH_OK;
}

pyrh_status pyrh_output_index(const double* lam, int32_t nspect, double lambda_ref, int32_t* idx,
                              int32_t* nout) {
  if (!lam || !idx || !nout || nspect < 1) return fail(PYRH_ERR_ARG, "output_index: arguments");
  int n = 0;
  bool found = false;
  for (int k = 0; k < nspect; ++k) {
    if (lam[k] == lambda_ref) { found = true; continue; }
    idx[n++] = k;
  }
  // the reference always returns Nspect - 1 points and assumes lambda_ref
  // is on the grid (pyrh_solveray.c:115-124)
  if (!found) return fail(PYRH_ERR_ARG, "output_index: lambda_ref %g is not on the grid", lambda_ref);
  *nout = n;
  return PYRH_OK;
}

double pyrh_gaunt_bf(double lambda, double n_eff, int32_t charge) {
  // Gaunt_bf (rh/hydrogen.c:269-281): Seaton (1960)
  const double x = ((kH * kC) / (lambda * kNm)) / (kERyd * ((charge) * (charge)));
  const double x3 = pow(x, 0.33333333);
  const double nsqx = 1.0 / (((n_eff) * (n_eff)) * x);
  return 1.0 + 0.1728 * x3 * (1.0 - 2.0 * nsqx) -
         0.0496 * ((x3) * (x3)) * (1.0 - (1.0 - nsqx) * 0.66666667 * nsqx);
}

pyrh_status pyrh_cont_alpha(const pyrh_atom* a, int32_t kr, const double* lam, int32_t n,
                            double* alpha) {
  if (!a || kr < 0 || kr >= a->ncont || !lam || !alpha || n < 1)
    return fail(PYRH_ERR_ARG, "cont_alpha: arguments");
  const pyrh_atom_cont& c = a->cont[kr];
  if (!c.hydrogenic)
    return fail(PYRH_ERR_UNSUPPORTED, "cont_alpha: continuum %d has an explicit table", kr);
  // sortlambda.c:331-344
  const int Z = a->level[c.j].stage;
  const double n_eff = Z * sqrt(kERyd / (a->level[c.j].E - a->level[c.i].E));
  const double gbf_0 = pyrh_gaunt_bf(c.lambda0, n_eff, Z);
  for (int la = 0; la < n; ++la)
    alpha[la] = c.alpha0 * pyrh_gaunt_bf(lam[la], n_eff, Z) / gbf_0 *
                ((lam[la] / c.lambda0) * (lam[la] / c.lambda0) * (lam[la] / c.lambda0));
  return PYRH_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------
// Kurucz line list (readKuruczLines, rh/kurucz.c:121-430), with the van der
// Waals cross-sections of Barklem's tables (getBarklemcross, getABOcross,
// rh/barklem.c:139-225, interpolated by cubic convolution as
// rh/cubeconvol.c:31-151 does) or Unsold's formula (getUnsoldcross,
// rh/kurucz.c:985-1020), and the Zeeman pattern of polarizable lines
// (RLKZeeman, rh/kurucz.c:832-920; ZeemanStrength and Lande,
// rh/zeeman.c:128-200).
// ------------------------------------------------------------------------

namespace {

constexpr double kAMU_ = 1.6605402E-27;
constexpr double kKB_ = 1.380658E-23;
constexpr double kRBOHR_ = 5.29177349E-11;
constexpr double kABARH_ = 7.42E-41;
constexpr double kMILLI = 1.0E-03;
constexpr double kAIR_TO_VACUUM_LIMIT = 199.9352;
constexpr double kDELTA_NEFF = 0.1;
constexpr double kLG10 = 2.30258509299404568402;

// 10^x as the reference evaluates it (exp of x ln 10)
double pow10_ref(double x) { return exp(kLG10 * (x)); }

// air_to_vacuum (rh/vacuumtoair.c), nm
double air_to_vacuum(double la) {
  if (la < kAIR_TO_VACUUM_LIMIT) return la;
  const double sqwave = ((1.0E+07 / la) * (1.0E+07 / la));
  const double increase = 1.0000834213E+00 + 2.406030E+06 / (1.30E+10 - sqwave) +
                          1.5997E+04 / (3.89E+09 - sqwave);
  return la * increase;
}

// Keys' cubic-convolution kernel
void cc_kernel(double s, double* k) {
  k[0] = -s * (1.0 - s * (2.0 - s)) / 2.0;
  k[1] = 1.0 + s * s * (3.0 * s - 5.0) / 2.0;
  k[2] = s * (1.0 + s * (4.0 - 3.0 * s)) / 2.0;
  k[3] = s * s * (s - 1.0) / 2.0;
}

// Cubic convolution on the table f[Ny][Nx] at fractional indices (x, y),
// the outermost rows and columns extrapolated linearly at the table's edges
double cubeconvol(int Nx, int Ny, const double* f, double x, double y) {
  int i, j;
  double ux[4], uy[4], ip, jp;
  if (x <= 0.0) { i = 0; cc_kernel(0.0, ux); }
  else if (x >= (double)(Nx - 1)) { i = Nx - 2; cc_kernel(1.0, ux); }
  else { cc_kernel(modf(x, &ip), ux); i = (int)ip; }
  if (y <= 0.0) { j = 0; cc_kernel(0.0, uy); }
  else if (y >= (double)(Ny - 1)) { j = Ny - 2; cc_kernel(1.0, uy); }
  else { cc_kernel(modf(y, &jp), uy); j = (int)jp; }
  // the 4x4 neighbourhood, rows j-1..j+2 and columns i-1..i+2
  double c[4][4];
  const bool lo_x = i == 0, hi_x = i == Nx - 2, lo_y = j == 0, hi_y = j == Ny - 2;
  for (int m = 0; m < 4; ++m) {
    const int row = j - 1 + m;
    if ((lo_y && m == 0) || (hi_y && m == 3)) continue;
    for (int n = 0; n < 4; ++n) {
      const int col = i - 1 + n;
      if ((lo_x && n == 0) || (hi_x && n == 3)) continue;
      c[m][n] = f[(long)Nx * row + col];
    }
    if (lo_x) c[m][0] = 3.0 * (c[m][1] - c[m][2]) + c[m][3];
    if (hi_x) c[m][3] = 3.0 * (c[m][2] - c[m][1]) + c[m][0];
  }
  if (lo_y)
    for (int n = 0; n < 4; ++n) c[0][n] = 3.0 * (c[1][n] - c[2][n]) + c[3][n];
  if (hi_y)
    for (int n = 0; n < 4; ++n) c[3][n] = 3.0 * (c[2][n] - c[1][n]) + c[0][n];
  double g = 0.0;
  for (int m = 0; m < 4; ++m)
    for (int n = 0; n < 4; ++n) g += c[m][n] * ux[n] * uy[m];
  return g;
}

// RLKdeterminate (rh/kurucz.c:925-980): spin and orbital momentum from the
// last word of a level label ("... z5P")
bool rlk_term(const char* label, double* S, int* L) {
  std::vector<std::string> w = words(label);
  if (w.empty()) return false;
  const std::string& last = w.back();
  if (last.size() < 2) return false;
  int multiplicity = 0;
  char orbit[4] = {0};
  if (sscanf(last.c_str() + last.size() - 2, "%d%1s", &multiplicity, orbit) != 2 ||
      !isupper((unsigned char)orbit[0]))
    return false;
  *L = orbital(orbit[0]);
  if (*L < 0) return false;
  *S = (multiplicity - 1) / 2.0;
  return true;
}

// ZeemanStrength (rh/zeeman.c:149-200)
double zeeman_strength(double Ju, double Mu, double Jl, double Ml) {
  const int q = (int)(Ml - Mu), dJ = (int)(Ju - Jl);
  switch (dJ) {
    case 0:
      if (q == 0) return 2.0 * (Mu * Mu);
      if (q == -1) return (Ju + Mu) * (Ju - Mu + 1.0);
      return (Ju - Mu) * (Ju + Mu + 1.0);
    case 1:
      if (q == 0) return 2.0 * ((Ju * Ju) - (Mu * Mu));
      if (q == -1) return (Ju + Mu) * (Ju + Mu - 1.0);
      return (Ju - Mu) * (Ju - Mu - 1.0);
    case -1:
      if (q == 0) return 2.0 * (((Ju + 1.0) * (Ju + 1.0)) - (Mu * Mu));
      if (q == -1) return (Ju - Mu + 1.0) * (Ju - Mu + 2.0);
      return (Ju + Mu + 1.0) * (Ju + Mu + 2.0);
  }
  return -1.0;
}

}  // namespace

extern "C" {

pyrh_status pyrh_barklem_parse(const char* text, int32_t type, double* cross, double* alpha,
                               pyrh_barklem_table* table) {
  // readBarklemTable (rh/barklem.c:61-135): three header lines, the cross
  // table, the rest of that line and one more, the alpha table
  static const int N1s[3] = {21, 18, 18}, N2s[3] = {18, 18, 18};
  static const double neff1s[3] = {1.0, 1.3, 2.3}, neff2s[3] = {1.3, 2.3, 3.3};
  if (!text || !cross || !alpha || !table || type < 0 || type > 2)
    return fail(PYRH_ERR_ARG, "barklem_parse: arguments");
  const int N1 = N1s[type], N2 = N2s[type];
  const char* p = text;
  auto skip_line = [&]() {
    while (*p && *p != '\n') ++p;
    if (*p) ++p;
  };
  for (int n = 0; n < 3; ++n) skip_line();
  auto read_block = [&](double* dst) {
    for (int e = 0; e < N1 * N2; ++e) {
      char* end = nullptr;
      dst[e] = strtod(p, &end);
      if (end == p) return false;
      p = end;
    }
    return true;
  };
  if (!read_block(cross)) return fail(PYRH_ERR_ARG, "barklem_parse: cross table short");
  skip_line();
  skip_line();
  if (!read_block(alpha)) return fail(PYRH_ERR_ARG, "barklem_parse: alpha table short");
  table->n1 = N1;
  table->n2 = N2;
  table->neff1_0 = neff1s[type];
  table->neff2_0 = neff2s[type];
  table->cross = cross;
  table->alpha = alpha;
  return PYRH_OK;
}

pyrh_status pyrh_kurucz_read(const char* text, const pyrh_kurucz_config* cfg, pyrh_line* lines,
                             pyrh_kurucz_extra* extra, int32_t cap, int32_t* nline) {
  if (!text || !cfg || !lines || !nline || cap < 0 || !cfg->elements || cfg->nelem < 2)
    return fail(PYRH_ERR_ARG, "kurucz_read: arguments (hydrogen and helium needed)");
  const double Cfac = 2.0 * kPi * (kQe / kEps0) * (kQe / kMe) / kC;
  const pyrh_element& H = cfg->elements[0];
  const pyrh_element& He = cfg->elements[1];
  int n = 0;
  const char* p = text;
  int line_index = 0;
  while (*p) {
    const char* e = strchr(p, '\n');
    const size_t len = e ? (size_t)(e - p) : strlen(p);
    // fgets of RLK_RECORD_LENGTH + 1 bytes: at most 171 characters a record
    std::string rec(p, len < 171 ? len : 171);
    p = e ? e + 1 : p + len;
    if (rec.empty() || rec[0] == '#') continue;
    bool blank = true;
    for (char c : rec)
      if (!isspace((unsigned char)c)) { blank = false; break; }
    if (blank) continue;
    if (n >= cap) return fail(PYRH_ERR_ARG, "kurucz_read: more than %d lines", cap);
    rec.resize(171, ' ');
    const char* r = rec.c_str();
    double lambda_air = 0, gf = 0, Ei = 0, Ej = 0, Ji = 0, Jj = 0;
    char code[16] = {0};
    if (sscanf(r, "%lf %lf %15s %lf", &lambda_air, &gf, code, &Ei) != 4 ||
        sscanf(r + 53, "%lf", &Ej) != 1 || sscanf(r + 35, "%lf", &Ji) != 1 ||
        sscanf(r + 63, "%lf", &Jj) != 1)
      return fail(PYRH_ERR_ARG, "kurucz_read: record %d unreadable", line_index);
    int pt_index = 0, stage = 0;
    if (sscanf(code, "%d.%d", &pt_index, &stage) != 2 || pt_index < 1 || pt_index > cfg->nelem)
      return fail(PYRH_ERR_ARG, "kurucz_read: element code %s of record %d", code, line_index);
    const pyrh_element& el = cfg->elements[pt_index - 1];
    Ei = fabs(Ei) * (kH * kC) / kCm;
    Ej = fabs(Ej) * (kH * kC) / kCm;
    const bool swap = Ej < Ei;
    char labeli[11] = {0}, labelj[11] = {0};
    double rEi, rEj;
    if (swap) {
      rEi = Ej; rEj = Ei;
      memcpy(labeli, r + 69, 10);
      memcpy(labelj, r + 41, 10);
      std::swap(Ji, Jj);
    } else {
      rEi = Ei; rEj = Ej;
      memcpy(labeli, r + 41, 10);
      memcpy(labelj, r + 69, 10);
    }
    const double gi = 2 * Ji + 1, gj = 2 * Jj + 1;
    // tabulated (air) wavelength; the upper energy follows from it
    const double lambda0 = air_to_vacuum(lambda_air) * kNm;
    rEj = rEi + (kH * kC) / lambda0;
    double loggf = gf;
    for (int k = 0; k < cfg->nloggf; ++k)
      if (cfg->loggf_ids[k] == line_index) loggf = cfg->loggf_values[k];
    const double Aji = Cfac / ((lambda0) * (lambda0)) * pow10_ref(loggf) / gj;
    const double Bji = ((lambda0) * (lambda0) * (lambda0)) / (2.0 * kH * kC) * Aji;
    const double Bij = (gj / gi) * Bji;
    // orbital numbers of the levels, or ABO coefficients (kurucz.c:263-291)
    int li = -1, lj = -1;
    bool abo = false;
    double a_abo = 0, s_abo = 0;
    {
      const int nr = sscanf(r + 160, "%lf %lf", &a_abo, &s_abo);
      if (nr == 2) {
        auto small = [](double x) { return x == 0.0 || x == 1.0 || x == 2.0 || x == 3.0; };
        if (small(a_abo) || small(s_abo)) {
          li = (int)a_abo;
          lj = (int)s_abo;
          if (swap) std::swap(li, lj);
        } else {
          abo = true;
        }
      }
    }
    double Si = 0, Sj = 0;
    int Li = -1, Lj = -1;
    const bool determined = rlk_term(labeli, &Si, &Li) && rlk_term(labelj, &Sj, &Lj);
    bool polarizable = cfg->stokes && determined;
    double Grad = 0, GStark = 0, GvdW = 0;
    {
      char g[19] = {0};
      memcpy(g, r + 79, 18);
      if (sscanf(g, "%lf %lf %lf", &Grad, &GStark, &GvdW) != 3)
        return fail(PYRH_ERR_ARG, "kurucz_read: damping of record %d", line_index);
    }
    GStark = (GStark != 0.0) ? pow10_ref(GStark) * (kCm * kCm * kCm) : 0.0;
    GvdW = (GvdW != 0.0) ? pow10_ref(GvdW) * (kCm * kCm * kCm) : 0.0;
    // van der Waals cross-section
    double cross = 0.0, alpha = 0.0;
    int vdw = PYRH_VDW_KURUCZ;
    const double reducedmass = kAMU_ / (1.0 / H.weight + 1.0 / el.weight);
    const double meanvelocity = sqrt(8.0 * kKB_ / (kPi * reducedmass));
    auto abo_scale = [&](double sigma, double a) {
      const double crossmean = (kRBOHR_ * kRBOHR_) * pow(meanvelocity / 1.0E4, -a);
      return sigma * 2.0 * pow(4.0 / kPi, a / 2.0) * exp(lgamma((4.0 - a) / 2.0)) *
             meanvelocity * crossmean;
    };
    bool barklem = false;
    if (abo) {
      alpha = a_abo;
      cross = abo_scale(s_abo, a_abo);
      vdw = PYRH_VDW_BARKLEM;
      barklem = true;
    } else {
      int t = -1;
      if ((li == 0 && lj == 1) || (li == 1 && lj == 0)) t = 0;
      if ((li == 1 && lj == 2) || (li == 2 && lj == 1)) t = 1;
      if ((li == 2 && lj == 3) || (li == 3 && lj == 2)) t = 2;
      const pyrh_barklem_table* bt = t >= 0 ? cfg->barklem[t] : nullptr;
      if (bt && stage == 0 && stage < el.nstage) {
        const double dEi = el.ionpot[stage] - rEi, dEj = el.ionpot[stage] - rEj;
        if (dEi > 0.0 && dEj > 0.0) {
          const double Z = (double)(stage + 1);
          const double ERyd = kERyd / (1.0 + kMe / (el.weight * kAMU_));
          double neff1 = Z * sqrt(ERyd / dEi), neff2 = Z * sqrt(ERyd / dEj);
          if (li > lj) std::swap(neff1, neff2);
          const double top1 = bt->neff1_0 + (bt->n1 - 1) * kDELTA_NEFF;
          const double top2 = bt->neff2_0 + (bt->n2 - 1) * kDELTA_NEFF;
          if (neff1 >= bt->neff1_0 && neff1 <= top1 && neff2 >= bt->neff2_0 && neff2 <= top2) {
            std::vector<double> g1(bt->n1), g2(bt->n2);
            for (int k = 0; k < bt->n1; ++k) g1[k] = bt->neff1_0 + k * kDELTA_NEFF;
            for (int k = 0; k < bt->n2; ++k) g2[k] = bt->neff2_0 + k * kDELTA_NEFF;
            int i1 = locate(bt->n1, g1.data(), neff1);
            const double f1 = (double)i1 + (neff1 - g1[i1]) / kDELTA_NEFF;
            int i2 = locate(bt->n2, g2.data(), neff2);
            const double f2 = (double)i2 + (neff2 - g2[i2]) / kDELTA_NEFF;
            const double c = cubeconvol(bt->n2, bt->n1, bt->cross, f2, f1);
            alpha = cubeconvol(bt->n2, bt->n1, bt->alpha, f2, f1);
            cross = abo_scale(c, alpha);
            vdw = PYRH_VDW_BARKLEM;
            barklem = true;
          }
        }
      }
    }
    if (!barklem) {
      // Unsold (kurucz.c:985-1020)
      vdw = PYRH_VDW_KURUCZ;
      if (stage <= el.nstage - 1 && stage < PYRH_ELEM_MAX_STAGES) {
        const double Z = stage + 1;
        const double deltaR = ((kERyd / (el.ionpot[stage] - rEj)) * (kERyd / (el.ionpot[stage] - rEj))) -
                              ((kERyd / (el.ionpot[stage] - rEi)) * (kERyd / (el.ionpot[stage] - rEi)));
        if (deltaR > 0.0) {
          const double fourpieps0 = 4.0 * kPi * kEps0;
          const double vrel35_H = pow(8.0 * kKB_ / (kPi * kAMU_ * el.weight) *
                                          (1.0 + el.weight / H.weight), 0.3);
          const double vrel35_He = pow(8.0 * kKB_ / (kPi * kAMU_ * el.weight) *
                                           (1.0 + el.weight / He.weight), 0.3);
          const double C625 = pow(2.5 * ((kQe * kQe) / fourpieps0) * (kABARH_ / fourpieps0) * 2 *
                                      kPi * ((Z * kRBOHR_) * (Z * kRBOHR_)) / kH * deltaR,
                                  0.4);
          cross = 8.08 * (vrel35_H + He.abund * vrel35_He) * C625;
          vdw = PYRH_VDW_UNSOLD;
        }
      }
    }
    Grad = (Grad != 0.0) ? pow10_ref(Grad) : Aji;
    double iso_frac = 0.0, hfs_frac = 0.0;
    int gLi = 0, gLj = 0;
    if (sscanf(r + 108, "%lf", &iso_frac) != 1 || sscanf(r + 117, "%lf", &hfs_frac) != 1 ||
        sscanf(r + 143, "%5d%5d", &gLi, &gLj) != 2)
      return fail(PYRH_ERR_ARG, "kurucz_read: isotope or Lande fields of record %d", line_index);
    iso_frac = pow10_ref(iso_frac);
    hfs_frac = pow10_ref(hfs_frac);
    double gL_i = gLi * kMILLI, gL_j = gLj * kMILLI;
    if (swap) std::swap(gL_i, gL_j);
    if (!cfg->ls_lande && cfg->stokes && gL_i != -99 * kMILLI && gL_j != -99 * kMILLI)
      polarizable = true;
    pyrh_line& L = lines[n];
    memset(&L, 0, sizeof(L));
    L.lambda0 = lambda0 / kNm;
    L.Ei = rEi;
    L.gi = gi;
    L.Aji = Aji;
    L.Bji = Bji;
    L.Bij = Bij;
    L.Grad = Grad;
    L.GStark = GStark;
    L.GvdWaals = GvdW;
    L.cross = cross;
    L.alpha = alpha;
    L.vdwaals = vdw;
    L.isotope_frac = iso_frac;
    L.hyperfine_frac = hfs_frac;
    L.weight = el.weight;
    L.contributes = (stage < el.nstage - 1) && el.abundance_set;
    L.polarizable = polarizable;
    L.ncomp = 0;
    if (polarizable) {
      // RLKZeeman (kurucz.c:832-920)
      const double Jl = (gi - 1.0) / 2.0, Ju = (gj - 1.0) / 2.0;
      double gLl, gLu;
      if (cfg->ls_lande) {
        gLl = lande(Si, Li, Jl);
        gLu = lande(Sj, Lj, Ju);
      } else {
        gLl = (gL_i == -99 * kMILLI) ? lande(Si, Li, Jl) : gL_i;
        gLu = (gL_j == -99 * kMILLI) ? lande(Sj, Lj, Ju) : gL_j;
      }
      double norm[3] = {0, 0, 0};
      int nc = 0;
      for (double Ml = -Jl; Ml <= Jl; Ml++)
        for (double Mu = -Ju; Mu <= Ju; Mu++)
          if (fabs(Mu - Ml) <= 1.0) {
            if (nc >= PYRH_MAX_COMPONENTS)
              return fail(PYRH_ERR_UNSUPPORTED, "kurucz_read: record %d has more than %d "
                          "Zeeman components", line_index, PYRH_MAX_COMPONENTS);
            L.comp_q[nc] = (int)(Ml - Mu);
            L.comp_shift[nc] = gLl * Ml - gLu * Mu;
            L.comp_strength[nc] = zeeman_strength(Ju, Mu, Jl, Ml);
            norm[L.comp_q[nc] + 1] += L.comp_strength[nc];
            ++nc;
          }
      for (int c = 0; c < nc; ++c) L.comp_strength[c] /= norm[L.comp_q[c] + 1];
      L.ncomp = nc;
    }
    if (extra) {
      pyrh_kurucz_extra& X = extra[n];
      X.pt_index = pt_index;
      X.stage = stage;
      X.gj = gj;
      X.Ej = rEj;
      X.gL_i = gL_i;
      X.gL_j = gL_j;
    }
    ++n;
    ++line_index;
  }
  *nline = n;
  return PYRH_OK;
}

}  // extern "C"
