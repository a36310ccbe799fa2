// OpenFOAM-format polyMesh files (read_mesh_openfoam, geometry.f90:846-1400):
// ASCII `points` ((x y z) per point), `faces` (n(v0 v1 ...) per face),
// `owner` and `neighbour` (one cell per face), each behind a FoamFile header
// and as an OpenFOAM list: its size, then "(", the entries and ")".  The
// sizes come from the owner file's note line (nPoints, nCells, nFaces,
// nInternalFaces), and every list's own size must confirm them, as the
// reference checks.  Indices are 0-based in the files and 1-based in
// fc_mesh.  `boundary` is the reference's one-line-per-patch file (a header
// line, then `name type nFaces startFace [startFaceTwin]`) or OpenFOAM's own
// dictionary form.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "fc_gpu.h"
#include "fc_mesh.hpp"

namespace {

bool slurp(const std::string& path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

// the text with // and /* */ comments blanked (quoted strings kept)
std::string strip_comments(const std::string& s) {
  std::string o(s);
  bool quoted = false;
  for (size_t i = 0; i < o.size(); ++i) {
    if (o[i] == '"') { quoted = !quoted; continue; }
    if (quoted) continue;
    if (o[i] == '/' && i + 1 < o.size() && o[i + 1] == '/') {
      while (i < o.size() && o[i] != '\n') o[i++] = ' ';
    } else if (o[i] == '/' && i + 1 < o.size() && o[i + 1] == '*') {
      size_t e = o.find("*/", i + 2);
      e = e == std::string::npos ? o.size() : e + 2;
      for (; i < e; ++i)
        if (o[i] != '\n') o[i] = ' ';
      --i;
    }
  }
  return o;
}

// the body after the FoamFile { ... } header: the list as a stream of
// numbers with its parentheses turned into blanks; *count receives the
// list's own size
bool list_body(const std::string& text, long long* count, std::istringstream& body) {
  std::string s = strip_comments(text);
  size_t pos = 0;
  const size_t ff = s.find("FoamFile");
  if (ff != std::string::npos) {
    const size_t open = s.find('{', ff);
    if (open == std::string::npos) return false;
    int depth = 0;
    size_t i = open;
    for (; i < s.size(); ++i) {
      if (s[i] == '{') ++depth;
      else if (s[i] == '}' && --depth == 0) break;
    }
    if (i >= s.size()) return false;
    pos = i + 1;
  }
  // the size, then the opening parenthesis
  size_t i = pos;
  while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
  size_t j = i;
  while (j < s.size() && std::isdigit((unsigned char)s[j])) ++j;
  if (j == i) return false;
  *count = std::atoll(s.substr(i, j - i).c_str());
  const size_t open = s.find('(', j);
  if (open == std::string::npos) return false;
  std::string rest = s.substr(open + 1);
  const size_t close = rest.rfind(')');
  if (close == std::string::npos) return false;
  rest.resize(close);
  for (char& c : rest)
    if (c == '(' || c == ')') c = ' ';
  body.str(rest);
  return true;
}

// "nPoints:8 nCells:1 nFaces:6 nInternalFaces:0" in the owner file's note
bool note_value(const std::string& s, const char* key, long long* v) {
  const size_t note = s.find("note");
  if (note == std::string::npos) return false;
  const size_t k = s.find(key, note);
  if (k == std::string::npos) return false;
  size_t i = k + std::strlen(key);
  while (i < s.size() && (s[i] == ':' || std::isspace((unsigned char)s[i]))) ++i;
  size_t j = i;
  while (j < s.size() && std::isdigit((unsigned char)s[j])) ++j;
  if (j == i) return false;
  *v = std::atoll(s.substr(i, j - i).c_str());
  return true;
}

// OpenFOAM's dictionary-form boundary file: N ( name { type T; nFaces n;
// startFace s; ... } ... ).  A patch's role: its type where the type names
// one (wall, symmetryPlane / symmetry, empty, cyclic with its
// neighbourPatch), else its name when that is one of the reference's types
// (inlet, outlet, pressure, ...).
bool boundary_dict(const std::string& text, fc_mesh* m) {
  std::string s = strip_comments(text);
  std::vector<std::string> nbr;  // neighbourPatch per patch
  const size_t ff = s.find("FoamFile");
  size_t pos = 0;
  if (ff != std::string::npos) {
    int depth = 0;
    size_t i = s.find('{', ff);
    for (; i < s.size(); ++i) {
      if (s[i] == '{') ++depth;
      else if (s[i] == '}' && --depth == 0) break;
    }
    pos = i + 1;
  }
  size_t open = s.find('(', pos);
  if (open == std::string::npos) return false;
  size_t i = open + 1;
  auto skip_ws = [&]() { while (i < s.size() && std::isspace((unsigned char)s[i])) ++i; };
  auto word = [&]() {
    skip_ws();
    size_t j = i;
    while (j < s.size() && !std::isspace((unsigned char)s[j]) && s[j] != '{' && s[j] != '}' && s[j] != ';' &&
           s[j] != '(' && s[j] != ')')
      ++j;
    std::string w = s.substr(i, j - i);
    i = j;
    return w;
  };
  for (;;) {
    skip_ws();
    if (i >= s.size()) return false;
    if (s[i] == ')') break;
    const std::string name = word();
    skip_ws();
    if (name.empty() || i >= s.size() || s[i] != '{') return false;
    const size_t close = s.find('}', i);
    if (close == std::string::npos) return false;
    std::string type, nbp;
    long long nf = -1, sf = -1;
    std::istringstream body(s.substr(i + 1, close - i - 1));
    std::string entry;
    while (std::getline(body, entry, ';')) {
      std::istringstream es(entry);
      std::string key, val;
      es >> key >> val;
      if (key == "type") type = val;
      else if (key == "nFaces") nf = std::atoll(val.c_str());
      else if (key == "startFace") sf = std::atoll(val.c_str());
      else if (key == "neighbourPatch") nbp = val;
    }
    i = close + 1;
    if (nf < 0 || sf < 0) return false;
    int t = 0;
    if (type == "wall") t = FC_BC_WALL;
    else if (type == "symmetryPlane" || type == "symmetry") t = FC_BC_SYMMETRY;
    else if (type == "empty") t = FC_BC_EMPTY;
    else if (type == "cyclic") t = FC_BC_PERIODIC;
    else t = bc_type_of(name);
    if (!t) return false;
    m->bcname.push_back(name);
    m->bctype.push_back(t);
    m->nfaces.push_back((int)nf);
    m->startFace.push_back((int)sf);
    m->startFaceTwin.push_back(-1);
    nbr.push_back(nbp);
  }
  // a cyclic pair in the reference's form: the patch listed first becomes
  // the 'empty' twin, the second the 'periodic' patch naming it
  for (size_t b = 0; b < m->bctype.size(); ++b) {
    if (m->bctype[b] != FC_BC_PERIODIC) continue;
    size_t t = 0;
    while (t < m->bcname.size() && m->bcname[t] != nbr[b]) ++t;
    if (t == m->bcname.size() || t == b || m->bctype[t] != FC_BC_PERIODIC || nbr[t] != m->bcname[b]) return false;
    if (t < b) {
      m->bctype[t] = FC_BC_EMPTY;
      m->startFaceTwin[b] = m->startFace[t];
    }
  }
  return true;
}

void header(FILE* f, const char* cls, const char* object, const std::string& note) {
  std::fprintf(f, "FoamFile\n{\n    version     2.0;\n    format      ascii;\n    class       %s;\n", cls);
  if (!note.empty()) std::fprintf(f, "    note        \"%s\";\n", note.c_str());
  std::fprintf(f, "    location    \"constant/polyMesh\";\n    object      %s;\n}\n\n", object);
}

}  // namespace

extern "C" int fc_mesh_read_openfoam(const char* dir, fc_mesh** out) {
  if (!dir || !out) return FC_ERR_BAD_INPUT;
  const std::string d(dir);
  std::string own_t, nb_t, pts_t, fcs_t;
  if (!slurp(d + "/owner", own_t) || !slurp(d + "/neighbour", nb_t) || !slurp(d + "/points", pts_t) ||
      !slurp(d + "/faces", fcs_t))
    return FC_ERR_BAD_INPUT;
  long long nP, nC, nF, nI;
  if (!note_value(own_t, "nPoints", &nP) || !note_value(own_t, "nCells", &nC) || !note_value(own_t, "nFaces", &nF) ||
      !note_value(own_t, "nInternalFaces", &nI))
    return FC_ERR_BAD_INPUT;
  if (nP <= 0 || nC <= 0 || nF <= 0 || nI < 0 || nI > nF || nF >= (1LL << 31)) return FC_ERR_BAD_INPUT;
  fc_mesh* m = new fc_mesh();
  m->numNodes = (int)nP;
  m->numCells = (int)nC;
  m->numFaces = (int)nF;
  m->numInnerFaces = (int)nI;
  m->numBoundaryFaces = (int)(nF - nI);
  auto fail = [&]() { delete m; return FC_ERR_BAD_INPUT; };
  long long cnt;
  std::istringstream body;
  // points: each list's own size confirms the note's
  if (!list_body(pts_t, &cnt, body) || cnt != nP) return fail();
  m->x.resize(nP); m->y.resize(nP); m->z.resize(nP);
  for (long long i = 0; i < nP; ++i)
    if (!(body >> m->x[i] >> m->y[i] >> m->z[i])) return fail();
  std::istringstream fb;
  if (!list_body(fcs_t, &cnt, fb) || cnt != nF) return fail();
  m->nnodes.assign(nF, 0);
  m->nodes.assign((size_t)nF * FC_NOMAX, 0);
  for (long long f = 0; f < nF; ++f) {
    int n;
    if (!(fb >> n) || n < 3 || n > FC_NOMAX) return fail();
    m->nnodes[f] = n;
    for (int k = 0; k < n; ++k) {
      int v;
      if (!(fb >> v)) return fail();
      m->nodes[(size_t)f * FC_NOMAX + k] = v + 1;
    }
  }
  std::istringstream fo;
  if (!list_body(own_t, &cnt, fo) || cnt != nF) return fail();
  m->owner.resize(nF);
  for (long long f = 0; f < nF; ++f) {
    if (!(fo >> m->owner[f])) return fail();
    m->owner[f] += 1;
  }
  std::istringstream fn;
  if (!list_body(nb_t, &cnt, fn) || cnt != nI) return fail();
  m->neighbour.resize(nI);
  for (long long f = 0; f < nI; ++f) {
    if (!(fn >> m->neighbour[f])) return fail();
    m->neighbour[f] += 1;
  }
  // boundary: OpenFOAM's dictionary form, or the reference's: a header
  // line, then name type nFaces startFace [startFaceTwin]
  std::string bnd_t;
  if (!slurp(d + "/boundary", bnd_t)) return fail();
  if (bnd_t.find("FoamFile") != std::string::npos) {
    if (!boundary_dict(bnd_t, m)) return fail();
    std::string why;
    if (m->validate(&why) != FC_OK) return fail();
    *out = m;
    return FC_OK;
  }
  std::istringstream bf(bnd_t);
  std::string line;
  std::getline(bf, line);
  while (std::getline(bf, line))
    if (!parse_boundary_line(line, m)) return fail();
  std::string why;
  if (m->validate(&why) != FC_OK) return fail();
  *out = m;
  return FC_OK;
}

extern "C" int fc_mesh_write_openfoam(const fc_mesh* m, const char* dir) {
  if (!m || !dir) return FC_ERR_BAD_INPUT;
  const std::string d(dir);
  const std::string note = "nPoints:" + std::to_string(m->numNodes) + "  nCells:" + std::to_string(m->numCells) +
                           "  nFaces:" + std::to_string(m->numFaces) +
                           "  nInternalFaces:" + std::to_string(m->numInnerFaces);
  FILE* f = std::fopen((d + "/points").c_str(), "w");
  if (!f) return FC_ERR_BAD_INPUT;
  header(f, "vectorField", "points", "");
  std::fprintf(f, "%d\n(\n", m->numNodes);
  for (int i = 0; i < m->numNodes; ++i) std::fprintf(f, "(%.17g %.17g %.17g)\n", m->x[i], m->y[i], m->z[i]);
  std::fprintf(f, ")\n");
  std::fclose(f);
  f = std::fopen((d + "/faces").c_str(), "w");
  if (!f) return FC_ERR_BAD_INPUT;
  header(f, "faceList", "faces", "");
  std::fprintf(f, "%d\n(\n", m->numFaces);
  for (int i = 0; i < m->numFaces; ++i) {
    std::fprintf(f, "%d(", m->nnodes[i]);
    for (int k = 0; k < m->nnodes[i]; ++k)
      std::fprintf(f, k ? " %d" : "%d", m->nodes[(size_t)i * FC_NOMAX + k] - 1);
    std::fprintf(f, ")\n");
  }
  std::fprintf(f, ")\n");
  std::fclose(f);
  f = std::fopen((d + "/owner").c_str(), "w");
  if (!f) return FC_ERR_BAD_INPUT;
  header(f, "labelList", "owner", note);
  std::fprintf(f, "%d\n(\n", m->numFaces);
  for (int i = 0; i < m->numFaces; ++i) std::fprintf(f, "%d\n", m->owner[i] - 1);
  std::fprintf(f, ")\n");
  std::fclose(f);
  f = std::fopen((d + "/neighbour").c_str(), "w");
  if (!f) return FC_ERR_BAD_INPUT;
  header(f, "labelList", "neighbour", note);
  std::fprintf(f, "%d\n(\n", m->numInnerFaces);
  for (int i = 0; i < m->numInnerFaces; ++i) std::fprintf(f, "%d\n", m->neighbour[i] - 1);
  std::fprintf(f, ")\n");
  std::fclose(f);
  f = std::fopen((d + "/boundary").c_str(), "w");
  if (!f) return FC_ERR_BAD_INPUT;
  write_boundary_lines(f, *m);
  std::fclose(f);
  return FC_OK;
}
