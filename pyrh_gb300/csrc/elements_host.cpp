// elements_host.cpp -- host readers of the element and molecule data: the
// abundance file, the Kurucz partition-function file and molecule files.
//
// Reference routines restated here (file:line in the reference tree):
//   readAbundance   rh/abundance.c:72-220  (record matching, the pyrh
//                                           overrides by record number, the
//                                           DEX and metallicity conversions,
//                                           the XDR partition-function file
//                                           and its conversion to ln U and J)
//   getLine         rh/getline.c:30-55     (comment and blank lines)
//   readMolecule    rh/readmolecule.c:66-240 (the molecule file up to its
//                                           equilibrium-constant fit)
// The file formats are the reference's, so they are parsed field for field;
// every conversion keeps the reference's expression (POW10(x) is
// exp(LG10 x), rh/rh.h:50) so the tables come out bit-identical.
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "../../include/pyrh_gb300.h"

namespace pyrh {
void set_error(const char* fmt, ...);
}

namespace {

constexpr double kLG10 = 2.30258509299404568402;   // ln 10
constexpr double kH = 6.6260755E-34;
constexpr double kC = 2.99792458E+08;
constexpr double kCM_TO_M = 1.0E-02;

// Symbols of the 99 elements in atomic-number order, two characters wide
// (the IDs the abundance records are matched against).
const char* const kElementID[PYRH_NELEM] = {
    "H ", "HE", "LI", "BE", "B ", "C ", "N ", "O ", "F ", "NE", "NA", "MG", "AL", "SI", "P ",
    "S ", "CL", "AR", "K ", "CA", "SC", "TI", "V ", "CR", "MN", "FE", "CO", "NI", "CU", "ZN",
    "GA", "GE", "AS", "SE", "BR", "KR", "RB", "SR", "Y ", "ZR", "NB", "MO", "TC", "RU", "RH",
    "PD", "AG", "CD", "IN", "SN", "SB", "TE", "I ", "XE", "CS", "BA", "LA", "CE", "PR", "ND",
    "PM", "SM", "EU", "GD", "TB", "DY", "HO", "ER", "TM", "YB", "LU", "HF", "TA", "W ", "RE",
    "OS", "IR", "PT", "AU", "HG", "TL", "PB", "BI", "PO", "AT", "RN", "FR", "RA", "AC", "TH",
    "PA", "U ", "NP", "PU", "AM", "CM", "BK", "CF", "ES"};

// Atomic weights [amu] of the same 99 elements as the reference tabulates
// them (rh/atomweights.h); the mean weight per hydrogen atom sums them.
const double kElementWeight[PYRH_NELEM] = {
    1.008,   4.003,   6.939,   9.013,   10.810,  12.010,  14.010,  16.000,  19.000,  20.180,
    22.990,  24.310,  26.980,  28.090,  30.980,  32.070,  35.450,  39.950,  39.100,  40.080,
    44.960,  47.900,  50.940,  52.000,  54.940,  55.850,  58.940,  58.710,  63.550,  65.370,
    69.720,  72.600,  74.920,  78.960,  79.910,  83.800,  85.480,  87.630,  88.910,  91.220,
    92.910,  95.950,  99.000,  101.100, 102.900, 106.400, 107.900, 112.400, 114.800, 118.700,
    121.800, 127.600, 126.900, 131.300, 132.900, 137.400, 138.900, 140.100, 140.900, 144.300,
    147.000, 150.400, 152.000, 157.300, 158.900, 162.500, 164.900, 167.300, 168.900, 173.000,
    175.000, 178.500, 181.000, 183.900, 186.300, 190.200, 192.200, 195.100, 197.000, 200.600,
    204.400, 207.200, 209.000, 210.000, 211.000, 222.000, 223.000, 226.100, 227.100, 232.000,
    231.000, 238.000, 237.000, 244.000, 243.000, 247.000, 247.000, 251.000, 254.000};

pyrh_status fail(pyrh_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  pyrh::set_error("%s", buf);
  return s;
}

// Big-endian XDR words.
struct Xdr {
  const unsigned char* p;
  size_t n, off = 0;
  bool ok = true;
  bool i32(int32_t* v) {
    if (off + 4 > n) return ok = false;
    const uint32_t u = (uint32_t)p[off] << 24 | (uint32_t)p[off + 1] << 16 |
                       (uint32_t)p[off + 2] << 8 | (uint32_t)p[off + 3];
    memcpy(v, &u, 4);
    off += 4;
    return true;
  }
  bool f64(double* v) {
    if (off + 8 > n) return ok = false;
    uint64_t u = 0;
    for (int i = 0; i < 8; ++i) u = (u << 8) | p[off + i];
    memcpy(v, &u, 8);
    off += 8;
    return true;
  }
};

}  // namespace

extern "C" pyrh_status pyrh_abundance_parse(const char* text, int32_t nabun,
                                            const int32_t* ab_id, const double* ab_val,
                                            double metallicity, double* abund,
                                            int32_t* abundance_set) {
  if (!text || !abund || !abundance_set) return fail(PYRH_ERR_ARG, "abundance: NULL argument");
  if (nabun < 0 || (nabun > 0 && (!ab_id || !ab_val)))
    return fail(PYRH_ERR_ARG, "abundance: override arrays missing");
  for (int n = 0; n < PYRH_NELEM; ++n) {
    abund[n] = 0.0;
    abundance_set[n] = 0;
  }
  bool dex = false;
  int record = 1;
  const char* s = text;
  while (*s) {
    const char* e = strchr(s, '\n');
    std::string line = e ? std::string(s, e - s) : std::string(s);
    s = e ? e + 1 : s + line.size();
    // getLine: skip lines whose first character is the comment mark and
    // lines without a token
    char tok[2];
    if (line.empty() || line[0] == '#' || sscanf(line.c_str(), "%1s", tok) < 1) continue;
    char id[64];
    double value;
    if (sscanf(line.c_str(), "%63s %lf", id, &value) != 2)
      return fail(PYRH_ERR_ARG, "abundance: unreadable record '%s'", line.c_str());
    for (char* c = id; *c; ++c) *c = (char)toupper((unsigned char)*c);
    if (strlen(id) == 1) strcat(id, " ");
    for (int i = 0; i < nabun; ++i)
      if (ab_id[i] == record) {
        value = ab_val[i];
        break;
      }
    ++record;
    for (int n = 0; n < PYRH_NELEM; ++n)
      if (strstr(kElementID[n], id)) {
        abund[n] = value;
        if (strstr(id, "H ") && value == 12.0) dex = true;
        abundance_set[n] = 1;
        break;
      }
  }
  const double metal = exp(kLG10 * metallicity);
  for (int n = 0; n < PYRH_NELEM; ++n) {
    if (!abundance_set[n]) continue;
    if (dex) abund[n] = exp(kLG10 * (abund[n] - 12.0));
    if (metal != 1.0 && n != 0) abund[n] *= metal;
  }
  return PYRH_OK;
}

extern "C" pyrh_status pyrh_abundance_totals(const double* abund, const int32_t* abundance_set,
                                             double* total_abund, double* wght_per_H) {
  if (!abund || !abundance_set || !total_abund || !wght_per_H)
    return fail(PYRH_ERR_ARG, "abundance totals: NULL argument");
  // rh/abundance.c:168-221: sums in element order over the elements with an
  // abundance
  double total = 0.0, weight = 0.0;
  for (int n = 0; n < PYRH_NELEM; ++n) {
    if (!abundance_set[n]) continue;
    total += abund[n];
    weight += abund[n] * kElementWeight[n];
  }
  *total_abund = total;
  *wght_per_H = weight;
  return PYRH_OK;
}

extern "C" int32_t pyrh_element_index(const char* id) {
  // readAtom (rh/readatom.c:109-126): the first two characters, upper case,
  // one-letter symbols padded with a blank, matched as a substring of the
  // table's symbols
  if (!id || !id[0]) return -1;
  char a[3] = {(char)toupper((unsigned char)id[0]),
               id[1] ? (char)toupper((unsigned char)id[1]) : ' ', 0};
  if (a[1] == 0) a[1] = ' ';
  for (int n = 0; n < PYRH_NELEM; ++n)
    if (strstr(kElementID[n], a)) return n;
  return -1;
}

extern "C" pyrh_status pyrh_pf_parse(const unsigned char* bytes, size_t nbytes,
                                     const int32_t* abundance_set, int32_t* npf,
                                     int32_t* nrows, double* Tpf, int32_t* nstage,
                                     int32_t* stage_off, double* lnpf, double* ionpot) {
  if (!bytes || !npf || !nrows) return fail(PYRH_ERR_ARG, "pf: NULL argument");
  Xdr x{bytes, nbytes};
  int32_t np = 0;
  if (!x.i32(&np) || np < 2 || np > 100000) return fail(PYRH_ERR_ARG, "pf: bad Npf");
  const bool fill = lnpf != nullptr;
  if (fill && (!abundance_set || !Tpf || !nstage || !stage_off || !ionpot))
    return fail(PYRH_ERR_ARG, "pf: NULL output array");
  for (int k = 0; k < np; ++k) {
    double t;
    if (!x.f64(&t)) return fail(PYRH_ERR_ARG, "pf: file ends in the temperature grid");
    if (fill) Tpf[k] = t;
  }
  int32_t rows = 0;
  for (int n = 0; n < PYRH_NELEM; ++n) {
    int32_t pti, ns;
    if (!x.i32(&pti) || !x.i32(&ns))
      return fail(PYRH_ERR_ARG, "pf: file ends before element %d", n + 1);
    if (ns < 1 || ns > PYRH_PF_MAX_STAGES)
      return fail(PYRH_ERR_UNSUPPORTED, "pf: element %d has %d stages (limit %d)", n + 1, ns,
                  PYRH_PF_MAX_STAGES);
    if (fill) {
      nstage[n] = ns;
      stage_off[n] = rows;
    }
    for (int i = 0; i < ns * np; ++i) {
      double u;
      if (!x.f64(&u)) return fail(PYRH_ERR_ARG, "pf: file ends in element %d", n + 1);
      if (fill) lnpf[(int64_t)rows * np + i] = abundance_set[n] ? log(u) : u;
    }
    for (int i = 0; i < ns; ++i) {
      double v;
      if (!x.f64(&v)) return fail(PYRH_ERR_ARG, "pf: file ends in element %d", n + 1);
      if (fill) ionpot[rows + i] = abundance_set[n] ? v * ((kH * kC) / kCM_TO_M) : v;
    }
    rows += ns;
  }
  *npf = np;
  *nrows = rows;
  return PYRH_OK;
}

// ---------------------------------------------------------------- molecules --
// readMolecule (rh/readmolecule.c:66-240): the records up to the
// equilibrium-constant fit, each on the next line that is neither blank nor
// a comment (getLine).
namespace {

struct Lines {
  const char* s;
  bool next(std::string& out) {
    while (*s) {
      const char* e = strchr(s, '\n');
      std::string line = e ? std::string(s, e - s) : std::string(s);
      s = e ? e + 1 : s + line.size();
      char tok[2];
      if (line.empty() || line[0] == '#' || sscanf(line.c_str(), "%1s", tok) < 1) continue;
      out = line;
      return true;
    }
    return false;
  }
};

// "N c_1 ... c_N" stored backwards, as the reference reads them
bool read_fit(const std::string& line, int32_t* n, double* coef) {
  std::string buf = line;
  char* save = nullptr;
  char* tok = strtok_r(&buf[0], " ", &save);
  if (!tok || sscanf(tok, "%d", n) != 1 || *n < 0 || *n > PYRH_MOL_MAX_COEF) return false;
  for (int i = *n - 1; i >= 0; --i) {
    tok = strtok_r(nullptr, " ", &save);
    if (!tok || sscanf(tok, "%lf", coef + i) != 1) return false;
  }
  return true;
}

}  // namespace

extern "C" pyrh_status pyrh_molecule_read(const char* text, const int32_t* abundance_set,
                                          pyrh_molecule* m) {
  if (!text || !abundance_set || !m) return fail(PYRH_ERR_ARG, "molecule: NULL argument");
  memset(m, 0, sizeof(*m));
  Lines in{text};
  std::string line;
  if (!in.next(line) || sscanf(line.c_str(), "%15s", m->id) != 1)
    return fail(PYRH_ERR_ARG, "molecule: no ID");
  if (!in.next(line) || sscanf(line.c_str(), "%d", &m->charge) != 1)
    return fail(PYRH_ERR_ARG, "molecule %s: no charge", m->id);
  if (m->charge < 0 || m->charge > 1)
    return fail(PYRH_ERR_ARG, "molecule %s: only neutral or singly charged molecules", m->id);
  if (!in.next(line)) return fail(PYRH_ERR_ARG, "molecule %s: no constituents", m->id);
  {
    std::string buf = line;
    char* save = nullptr;
    for (char* tok = strtok_r(&buf[0], " ,", &save); tok; tok = strtok_r(nullptr, " ,", &save)) {
      if (m->nelement == PYRH_MOL_MAX_ELEMENTS)
        return fail(PYRH_ERR_UNSUPPORTED, "molecule %s: more than %d elements", m->id,
                    PYRH_MOL_MAX_ELEMENTS);
      int count = 1;
      char el[32];
      if (sscanf(tok, "%d%31s", &count, el) == 0) {
        count = 1;
        if (sscanf(tok, "%31s", el) != 1) continue;
      }
      for (char* c = el; *c; ++c) *c = (char)toupper((unsigned char)*c);
      if (strlen(el) == 1) strcat(el, " ");
      int found = -1;
      for (int n = 0; n < PYRH_NELEM; ++n)
        if (strstr(el, kElementID[n])) {
          if (abundance_set[n]) found = n;
          break;
        }
      if (found < 0)
        return fail(PYRH_ERR_ARG, "molecule %s: element %s unknown or without abundance", m->id,
                    el);
      m->pt_index[m->nelement] = found;
      m->pt_count[m->nelement] = count;
      m->nnuclei += count;
      ++m->nelement;
    }
    if (m->nelement == 0) return fail(PYRH_ERR_ARG, "molecule %s: no constituents", m->id);
  }
  if (!in.next(line) || sscanf(line.c_str(), "%lf", &m->ediss) != 1)
    return fail(PYRH_ERR_ARG, "molecule %s: no dissociation energy", m->id);
  m->ediss *= 1.60217733E-19;   // EV
  char fit[64] = "";
  if (!in.next(line) || sscanf(line.c_str(), "%63s", fit) != 1)
    return fail(PYRH_ERR_ARG, "molecule %s: no fit type", m->id);
  if (strstr(fit, "KURUCZ_70")) m->fit = PYRH_FIT_KURUCZ_70;
  else if (strstr(fit, "KURUCZ_85")) m->fit = PYRH_FIT_KURUCZ_85;
  else if (strstr(fit, "SAUVAL_TATUM_84")) m->fit = PYRH_FIT_SAUVAL_TATUM_84;
  else if (strstr(fit, "IRWIN_81")) m->fit = PYRH_FIT_IRWIN_81;
  else if (strstr(fit, "TSUJI_73")) m->fit = PYRH_FIT_TSUJI_73;
  else return fail(PYRH_ERR_ARG, "molecule %s: unknown fit %s", m->id, fit);
  if (m->charge > 0 && m->fit != PYRH_FIT_KURUCZ_70 && m->fit != PYRH_FIT_KURUCZ_85)
    return fail(PYRH_ERR_ARG, "molecule %s: a charged molecule needs a KURUCZ fit", m->id);
  if (!in.next(line) || sscanf(line.c_str(), "%lf %lf", &m->tmin, &m->tmax) != 2)
    return fail(PYRH_ERR_ARG, "molecule %s: no formation temperatures", m->id);
  if (!in.next(line) || !read_fit(line, &m->npf, m->pf_coef))
    return fail(PYRH_ERR_ARG, "molecule %s: partition-function fit", m->id);
  if (!in.next(line) || !read_fit(line, &m->neqc, m->eqc_coef))
    return fail(PYRH_ERR_ARG, "molecule %s: equilibrium-constant fit", m->id);
  return PYRH_OK;
}
