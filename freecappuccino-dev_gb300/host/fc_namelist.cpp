// The case namelist &input_parameters (read_input.f90:28-227) as the path
// uses it: fc_namelist_read parses the file into fc_case_settings, starting
// from the reference's module defaults (velocity.f90:24-33, pressure.f90:
// 28-33, temperature.f90:14-25, nablap.f90:8); fc_apply_settings passes them
// to the context.
//
// Namelist syntax handled: `name = value[, value ...]` (commas or blanks),
// `!` comments outside quotes, 'strings' and "strings", logicals T / F /
// .true. / .false. (any case), numbers with e or d exponents, names in any
// case, `name(i) = value` for one element.  As in Fortran, an array given
// fewer values keeps its remaining elements.  Keys of other modules
// (turbulence, MHD, energy, ...) are skipped.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "fc_gpu.h"

namespace {

struct Tok {
  enum Kind { NAME, EQ, VAL } kind;
  std::string s;     // NAME: lower-case name (with "(i)" kept apart); VAL: the text
  bool quoted = false;
  int index = 0;     // NAME(i)
};

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

bool tokenize(const std::string& body, std::vector<Tok>& out, std::string& err) {
  size_t i = 0;
  const size_t n = body.size();
  while (i < n) {
    const char c = body[i];
    if (std::isspace((unsigned char)c) || c == ',') { ++i; continue; }
    if (c == '!') { while (i < n && body[i] != '\n') ++i; continue; }
    if (c == '=') { out.push_back({Tok::EQ, "="}); ++i; continue; }
    if (c == '\'' || c == '"') {
      const size_t e = body.find(c, i + 1);
      if (e == std::string::npos) { err = "unterminated string"; return false; }
      Tok t{Tok::VAL, body.substr(i + 1, e - i - 1)};
      t.quoted = true;
      out.push_back(t);
      i = e + 1;
      continue;
    }
    size_t j = i;
    while (j < n && !std::isspace((unsigned char)body[j]) && body[j] != ',' && body[j] != '=' && body[j] != '!' &&
           body[j] != '\'' && body[j] != '"')
      ++j;
    std::string w = body.substr(i, j - i);
    i = j;
    // a name is followed (after blanks) by '='
    size_t k = i;
    while (k < n && std::isspace((unsigned char)body[k])) ++k;
    if (k < n && body[k] == '=') {
      Tok t{Tok::NAME, lower(w)};
      const size_t p = t.s.find('(');
      if (p != std::string::npos) {
        t.index = std::atoi(t.s.c_str() + p + 1);
        t.s.resize(p);
      }
      out.push_back(t);
    } else {
      out.push_back({Tok::VAL, w});
    }
  }
  return true;
}

bool as_logical(const Tok& t, int* v) {
  std::string s = lower(t.s);
  if (!s.empty() && s[0] == '.') s = s.substr(1);
  if (s.empty()) return false;
  if (s[0] == 't') { *v = 1; return true; }
  if (s[0] == 'f') { *v = 0; return true; }
  return false;
}

bool as_double(const Tok& t, double* v) {
  if (t.quoted) return false;
  std::string s = t.s;
  for (char& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  char* end = nullptr;
  *v = std::strtod(s.c_str(), &end);
  return end && *end == '\0' && !s.empty();
}

bool as_int(const Tok& t, int* v) {
  double d;
  if (!as_double(t, &d)) return false;
  *v = (int)d;
  return (double)*v == d;
}

void copy_name(char* dst, size_t cap, const std::string& s) {
  std::snprintf(dst, cap, "%s", s.c_str());
}

int scheme_id(const std::string& s) {
  static const char* names[] = {"cds", "central", "linearUpwind", "kappa"};
  for (int k = 0; k < 4; ++k)
    if (s == names[k]) return k;
  static const char* fl[] = {"muscl", "umist", "koren", "smart", "avl-smart", "charm", "vanleer", "ospre", "minmod",
                             "boundedLinearUpwind", "boundedLinearUpwind02", "boundedCentral", "fromm", "cui",
                             "quick", "spl13"};
  for (int k = 0; k < 16; ++k)
    if (s == fl[k]) return 10 + k;
  return -1;
}

int limiter_id(const std::string& s) {
  if (s == "Barth-Jespersen") return FC_LIMITER_BJ;
  if (s == "Venkatakrishnan") return FC_LIMITER_VENKAT;
  if (s == "R3") return FC_LIMITER_R;
  if (s == "multidimensional") return FC_LIMITER_MD;
  return FC_LIMITER_NONE;  // 'none', 'no-limit' and anything else: the select's default
}

void defaults(fc_case_settings* c) {
  std::memset(c, 0, sizeof(*c));
  fc_simple_params& s = c->simple;
  for (double& u : s.urfU) u = (double)0.7f;  // (/ 0.7, 0.7, 0.7 /), default-real literals
  s.gdsU = 1.0;
  s.cSchemeU = FC_SCHEME_LINEAR_UPWIND;
  s.gradScheme = FC_GRAD_GAUSS;
  s.maxiterU = 5;
  s.tolAbsU = (double)1e-13f;
  s.tolRelU = (double)0.025f;
  s.urfP = 0.2;
  s.maxiterP = 30;
  s.tolAbsP = (double)1e-13f;
  s.tolRelP = 0.025;
  s.npcor = 1;
  s.pRefCell = 1;
  copy_name(s.lSolverU, sizeof s.lSolverU, "bicgstab");
  copy_name(s.lSolverP, sizeof s.lSolverP, "iccg");
  fc_temperature_params& t = c->temperature;
  t.urfT = 0.9;
  t.gdsT = 1.0;
  t.sigt = 1.0;
  t.cSchemeT = FC_SCHEME_LINEAR_UPWIND;
  t.maxiterT = 10;
  t.tolAbsT = (double)1e-13f;
  t.tolRelT = 0.02;
  copy_name(t.lSolverT, sizeof t.lSolverT, "bicgstab");
  c->transient.timestep = 1.0;
  c->transient.ncorr = 1;
  c->run.numstep = 1;
  c->run.maxit = 1;
  c->calcU = c->calcP = 1;
}

}  // namespace

extern "C" int fc_namelist_read(const char* path, fc_case_settings* out, char* errmsg, int errlen) {
  auto fail = [&](const std::string& m) {
    if (errmsg && errlen > 0) std::snprintf(errmsg, (size_t)errlen, "%s", m.c_str());
    return FC_ERR_BAD_INPUT;
  };
  if (!path || !out) return fail("fc_namelist_read: bad arguments");
  std::ifstream f(path);
  if (!f) return fail(std::string("cannot open ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string text = ss.str();
  // the group: from &input_parameters to the '/' that ends it (outside quotes)
  const std::string lt = lower(text);
  const size_t g = lt.find("&input_parameters");
  if (g == std::string::npos) return fail("no &input_parameters group");
  size_t i = g + std::strlen("&input_parameters");
  size_t end = std::string::npos;
  char q = 0;
  for (size_t k = i; k < text.size(); ++k) {
    const char c = text[k];
    if (q) { if (c == q) q = 0; continue; }
    if (c == '\'' || c == '"') { q = c; continue; }
    if (c == '!') { while (k < text.size() && text[k] != '\n') ++k; continue; }
    if (c == '/') { end = k; break; }
  }
  if (end == std::string::npos) return fail("&input_parameters is not closed by '/'");
  std::vector<Tok> toks;
  std::string err;
  if (!tokenize(text.substr(i, end - i), toks, err)) return fail(err);
  fc_case_settings c;
  defaults(&c);
  int lstsq = 0, lstsq_qr = 0, lstsq_dm = 0, node_gauss = 0, ltransient = 0, bdf = 0, bdf2 = 0, bdf3 = 0, cn = 0;
  int simple = -1, piso = 0, compressible = 0, const_mflux = 0;
  for (size_t k = 0; k < toks.size();) {
    if (toks[k].kind != Tok::NAME || k + 1 >= toks.size() || toks[k + 1].kind != Tok::EQ)
      return fail("unexpected '" + toks[k].s + "'");
    const std::string key = toks[k].s;
    const int idx = toks[k].index;
    k += 2;
    std::vector<Tok> v;
    while (k < toks.size() && toks[k].kind == Tok::VAL) v.push_back(toks[k++]);
    if (v.empty()) return fail("no value for " + key);
    int iv = 0;
    double dv = 0;
    auto need_d = [&](double* dst) { return as_double(v[0], dst) ? 0 : -1; };
    auto need_i = [&](int* dst) { return as_int(v[0], dst) ? 0 : -1; };
    auto need_l = [&](int* dst) { return as_logical(v[0], dst) ? 0 : -1; };
    int bad = 0;
    fc_simple_params& s = c.simple;
    fc_temperature_params& t = c.temperature;
    if (key == "title") copy_name(c.title, sizeof c.title, v[0].s);
    else if (key == "mesh_format") c.mesh_foam = v[0].s == "foamMesh";
    else if (key == "calcu") bad = need_l(&c.calcU);
    else if (key == "calcp") bad = need_l(&c.calcP);
    else if (key == "calct") bad = need_l(&c.calcT);
    else if (key == "urfu") {
      // urfU(i) = x sets one element; a list fills from the first (or i-th) on
      const int start = idx > 0 ? idx - 1 : 0;
      for (size_t e = 0; e < v.size() && start + e < 3; ++e)
        if (!as_double(v[e], &s.urfU[start + e])) bad = -1;
    } else if (key == "gdsu") bad = need_d(&s.gdsU);
    else if (key == "cschemeu") { s.cSchemeU = scheme_id(v[0].s); if (s.cSchemeU < 0) return fail("unknown cSchemeU '" + v[0].s + "'"); }
    else if (key == "lsolveru") copy_name(s.lSolverU, sizeof s.lSolverU, v[0].s);
    else if (key == "maxiteru") bad = need_i(&s.maxiterU);
    else if (key == "tolabsu") bad = need_d(&s.tolAbsU);
    else if (key == "tolrelu") bad = need_d(&s.tolRelU);
    else if (key == "pscheme") {
      if (v[0].s == "linear") s.pscheme = 0;
      else if (v[0].s == "central") s.pscheme = 1;
      else if (v[0].s == "weighted") s.pscheme = 2;
      else return fail("unknown pscheme '" + v[0].s + "'");
    } else if (key == "urfp") bad = need_d(&s.urfP);
    else if (key == "lsolverp") copy_name(s.lSolverP, sizeof s.lSolverP, v[0].s);
    else if (key == "maxiterp") bad = need_i(&s.maxiterP);
    else if (key == "tolabsp") bad = need_d(&s.tolAbsP);
    else if (key == "tolrelp") bad = need_d(&s.tolRelP);
    else if (key == "urft") bad = need_d(&t.urfT);
    else if (key == "gdst") bad = need_d(&t.gdsT);
    else if (key == "cschemet") { t.cSchemeT = scheme_id(v[0].s); if (t.cSchemeT < 0) return fail("unknown cSchemeT '" + v[0].s + "'"); }
    else if (key == "lsolvert") copy_name(t.lSolverT, sizeof t.lSolverT, v[0].s);
    else if (key == "maxitert") bad = need_i(&t.maxiterT);
    else if (key == "tolabst") bad = need_d(&t.tolAbsT);
    else if (key == "tolrelt") bad = need_d(&t.tolRelT);
    else if (key == "sigt") bad = need_d(&t.sigt);
    else if (key == "densit") bad = need_d(&s.densit);
    else if (key == "viscos") bad = need_d(&s.viscos);
    else if (key == "pranl") bad = need_d(&t.pranl);
    else if (key == "ltransient") bad = need_l(&ltransient);
    else if (key == "bdf") bad = need_l(&bdf);
    else if (key == "bdf2") bad = need_l(&bdf2);
    else if (key == "bdf3") bad = need_l(&bdf3);
    else if (key == "cn") bad = need_l(&cn);
    else if (key == "lstsq") bad = need_l(&lstsq);
    else if (key == "lstsq_qr") bad = need_l(&lstsq_qr);
    else if (key == "lstsq_dm") bad = need_l(&lstsq_dm);
    else if (key == "node_gauss") bad = need_l(&node_gauss);
    else if (key == "gauss") bad = need_l(&iv);
    else if (key == "limiter") c.limiter = limiter_id(v[0].s);
    else if (key == "simple") bad = need_l(&simple);
    else if (key == "piso") bad = need_l(&piso);
    else if (key == "compressible") bad = need_l(&compressible);
    else if (key == "const_mflux") bad = need_l(&const_mflux);
    else if (key == "ncorr") bad = need_i(&c.transient.ncorr);
    else if (key == "npcor") bad = need_i(&s.npcor);
    else if (key == "prefcell") bad = need_i(&s.pRefCell);
    else if (key == "tolerance") bad = need_d(&c.run.tolerance);
    else if (key == "numstep") bad = need_i(&c.run.numstep);
    else if (key == "timestep") bad = need_d(&c.transient.timestep);
    else if (key == "maxit") bad = need_i(&c.run.maxit);
    (void)dv;
    if (bad) return fail("bad value for " + key);
  }
  // gradient selection as grad_scalar_field (gradients.f90:117-138)
  if (lstsq) c.simple.gradScheme = FC_GRAD_LSQ;
  else if (lstsq_qr) return fail("lstsq_qr (LAPACK QR least squares) is not supported");
  else if (lstsq_dm) c.simple.gradScheme = FC_GRAD_LSQ_DM;
  else if (node_gauss) c.simple.gradScheme = FC_GRAD_NODE_GAUSS;
  else c.simple.gradScheme = FC_GRAD_GAUSS;
  c.temperature.gradScheme = c.simple.gradScheme;
  c.temperature.viscos = c.simple.viscos;
  if (compressible) return fail("compressible flow is not supported");
  if (const_mflux) return fail("const_mflux is not supported");
  if (cn) return fail("Crank-Nicolson time stepping is not supported");
  c.transient.scheme = !ltransient ? FC_TIME_STEADY : bdf ? FC_TIME_BDF : bdf2 ? FC_TIME_BDF2 : bdf3 ? FC_TIME_BDF3
                                                                                                  : FC_TIME_STEADY;
  if (ltransient && c.transient.scheme == FC_TIME_STEADY) return fail("ltransient without bdf, bdf2 or bdf3");
  c.transient.piso = piso;
  if (piso && simple == 1) return fail("both SIMPLE and PISO are set");
  c.run.temperature = c.calcT;
  *out = c;
  return FC_OK;
}

extern "C" int fc_apply_settings(fc_ctx* ctx, const fc_case_settings* s) {
  if (!ctx || !s) return FC_ERR_BAD_INPUT;
  int st;
  if ((st = fc_simple_set_params(ctx, &s->simple))) return st;
  if ((st = fc_transient_set_params(ctx, &s->transient))) return st;
  if ((st = fc_set_gradient_limiter(ctx, s->limiter))) return st;
  if (s->calcT && (st = fc_temperature_set_params(ctx, &s->temperature, nullptr))) return st;
  return FC_OK;
}
