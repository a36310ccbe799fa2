// Host-side mesh producer for the GB300 path: a seeded synthetic box generator
// (structured hexes, optionally split into 6 tetrahedra) and the reader/writer
// of the reference's native polyMesh files (read_mesh_native,
// src/mesh/geometry.f90:118-410).  Index arrays are 1-based as in the
// reference; inner faces are ordered by (owner, neighbour) with owner <
// neighbour and the area vector pointing owner -> neighbour, the convention of
// the reference's mesh converters (utilities/su2ToCappuccino.f90:362-382).
#include "fc_mesh.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

// splitmix64: a fixed, platform-independent generator for the vertex
// perturbation (the same bits on x86_64 and aarch64).
struct SplitMix64 {
  unsigned long long s;
  explicit SplitMix64(unsigned long long seed) : s(seed) {}
  unsigned long long next() {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  // uniform in [0,1) with 53 random bits
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

const char* kSideName[6] = {"xmin", "xmax", "ymin", "ymax", "zmin", "zmax"};

struct V3 { double x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

}  // namespace

// boundary type names of the reference (bctype) <-> FC_BC_*
const char* bc_name_of(int t) {
  switch (t) {
    case FC_BC_WALL: return "wall";
    case FC_BC_INLET: return "inlet";
    case FC_BC_OUTLET: return "outlet";
    case FC_BC_SYMMETRY: return "symmetry";
    case FC_BC_PRESSURE: return "pressure";
    case FC_BC_EMPTY: return "empty";
    case FC_BC_PERIODIC: return "periodic";
    default: return "unknown";
  }
}

int bc_type_of(const std::string& s) {
  if (s == "wall") return FC_BC_WALL;
  if (s == "inlet") return FC_BC_INLET;
  if (s == "outlet") return FC_BC_OUTLET;
  if (s == "symmetry") return FC_BC_SYMMETRY;
  if (s == "pressure") return FC_BC_PRESSURE;
  if (s == "empty") return FC_BC_EMPTY;
  if (s == "periodic") return FC_BC_PERIODIC;
  return 0;
}


// one line of the reference's boundary file: name type nFaces startFace, and
// for a periodic patch the startFace of its twin (geometry.f90:234-258);
// false on an unknown type, true (nothing added) on a line that is not a patch
bool parse_boundary_line(const std::string& line, fc_mesh* m) {
  std::istringstream ls(line);
  std::string name, type;
  int nf, sf;
  if (!(ls >> name >> type >> nf >> sf)) return true;
  const int t = bc_type_of(type);
  if (!t) return false;
  int tw = -1;
  if (t == FC_BC_PERIODIC && !(ls >> tw)) return false;
  m->bcname.push_back(name); m->bctype.push_back(t); m->nfaces.push_back(nf); m->startFace.push_back(sf);
  m->startFaceTwin.push_back(tw);
  return true;
}

void write_boundary_lines(FILE* f, const fc_mesh& m) {
  std::fprintf(f, "#bcname bctype nFaces startFace\n");
  for (size_t b = 0; b < m.bctype.size(); ++b) {
    std::fprintf(f, "%s %s %d %d", m.bcname[b].c_str(), bc_name_of(m.bctype[b]), m.nfaces[b], m.startFace[b]);
    if (m.bctype[b] == FC_BC_PERIODIC) std::fprintf(f, " %d", m.twin_of(b));
    std::fprintf(f, "\n");
  }
}

int fc_mesh::validate(std::string* why, bool complete) const {
  auto fail = [&](const char* m) { if (why) *why = m; return FC_ERR_BAD_INPUT; };
  if (numNodes <= 0 || numCells <= 0 || numInnerFaces < 0 || numBoundaryFaces < 0) return fail("non-positive mesh sizes");
  if (numFaces != numInnerFaces + numBoundaryFaces) return fail("numFaces != numInnerFaces + numBoundaryFaces");
  if ((int)owner.size() != numFaces || (int)neighbour.size() != numInnerFaces) return fail("owner/neighbour sizes");
  for (int f = 0; f < numFaces; ++f) {
    int n = nnodes[f];
    if (n < 3 || n > FC_NOMAX) return fail("face with <3 or >nomax nodes");
    for (int k = 0; k < n; ++k) {
      int v = nodes[(size_t)f * FC_NOMAX + k];
      if (v < 1 || v > numNodes) return fail("face node index out of range");
    }
    if (owner[f] < 1 || owner[f] > numCells) return fail("owner index out of range");
    if (f < numInnerFaces) {
      int nb = neighbour[f];
      if (nb < 1 || nb > numCells || nb == owner[f]) return fail("neighbour index out of range");
    }
  }
  int expect = numInnerFaces;
  for (size_t b = 0; b < bctype.size(); ++b) {
    if (startFace[b] != expect) return fail("boundary patches must be contiguous and follow the inner faces");
    if (nfaces[b] < 0) return fail("negative patch size");
    if (bctype[b] < FC_BC_WALL || bctype[b] > FC_BC_PERIODIC) return fail("unknown boundary type");
    expect += nfaces[b];
  }
  if (expect != numFaces) return fail("boundary patches do not cover all boundary faces");
  // periodic pairs: the twin is another patch of the same size typed 'empty',
  // twin of one periodic patch only; at most three pairs (startFaceTwin(3),
  // geometry.f90:82); the pair loops index Df and facint by the face's
  // position within its patch, so a patch has at most numInnerFaces faces
  int nper = 0;
  std::vector<int> used(bctype.size(), 0);
  for (size_t b = 0; b < bctype.size(); ++b) {
    if (bctype[b] != FC_BC_PERIODIC) continue;
    ++nper;
    const int tw = twin_of(b);
    if (tw < 0) {
      if (complete) return fail("a periodic patch names no twin (startFaceTwin)");
      continue;
    }
    size_t t = 0;
    while (t < bctype.size() && !(startFace[t] == tw && t != b)) ++t;
    if (t == bctype.size()) return fail("the startFaceTwin of a periodic patch is the start of no other patch");
    if (nfaces[t] != nfaces[b]) return fail("a periodic patch and its twin differ in size");
    if (bctype[t] != FC_BC_EMPTY) return fail("the twin of a periodic patch must be typed 'empty'");
    if (used[t]++) return fail("a patch is the twin of two periodic patches");
    if (nfaces[b] > numInnerFaces) return fail("a periodic patch has more faces than the mesh has inner faces");
  }
  if (nper > 3) return fail("more than three periodic pairs");
  return FC_OK;
}

static void box_hex(fc_mesh& m, int nx, int ny, int nz) {
  auto nid = [&](int i, int j, int k) { return i + (nx + 1) * (j + (ny + 1) * k) + 1; };
  auto cid = [&](int i, int j, int k) { return i + nx * (j + ny * k) + 1; };
  m.numInnerFaces = (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1);
  m.numBoundaryFaces = 2 * (ny * nz + nx * nz + nx * ny);
  m.numFaces = m.numInnerFaces + m.numBoundaryFaces;
  m.nnodes.assign(m.numFaces, 4);
  m.nodes.assign((size_t)m.numFaces * FC_NOMAX, 0);
  m.owner.assign(m.numFaces, 0);
  m.neighbour.assign(m.numInnerFaces, 0);
  int f = 0;
  auto put = [&](int a, int b, int c, int d, int own, int nb) {
    int* q = &m.nodes[(size_t)f * FC_NOMAX];
    q[0] = a; q[1] = b; q[2] = c; q[3] = d;
    m.owner[f] = own;
    if (nb > 0) m.neighbour[f] = nb;
    ++f;
  };
  // inner faces: for each cell in order its +x, +y, +z faces, so the list is
  // sorted by (owner, neighbour)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int c = cid(i, j, k);
        if (i + 1 < nx) put(nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i + 1, j + 1, k + 1), nid(i + 1, j, k + 1), c, cid(i + 1, j, k));
        if (j + 1 < ny) put(nid(i, j + 1, k), nid(i, j + 1, k + 1), nid(i + 1, j + 1, k + 1), nid(i + 1, j + 1, k), c, cid(i, j + 1, k));
        if (k + 1 < nz) put(nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1), c, cid(i, j, k + 1));
      }
  // boundary patches xmin, xmax, ymin, ymax, zmin, zmax; outward normals
  int start = f;
  m.nfaces.clear(); m.startFace.clear();
  auto begin_patch = [&]() { start = f; };
  auto end_patch = [&]() { m.startFace.push_back(start); m.nfaces.push_back(f - start); };
  begin_patch();
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j)
    put(nid(0, j, k), nid(0, j, k + 1), nid(0, j + 1, k + 1), nid(0, j + 1, k), cid(0, j, k), 0);
  end_patch(); begin_patch();
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j)
    put(nid(nx, j, k), nid(nx, j + 1, k), nid(nx, j + 1, k + 1), nid(nx, j, k + 1), cid(nx - 1, j, k), 0);
  end_patch(); begin_patch();
  for (int k = 0; k < nz; ++k) for (int i = 0; i < nx; ++i)
    put(nid(i, 0, k), nid(i + 1, 0, k), nid(i + 1, 0, k + 1), nid(i, 0, k + 1), cid(i, 0, k), 0);
  end_patch(); begin_patch();
  for (int k = 0; k < nz; ++k) for (int i = 0; i < nx; ++i)
    put(nid(i, ny, k), nid(i, ny, k + 1), nid(i + 1, ny, k + 1), nid(i + 1, ny, k), cid(i, ny - 1, k), 0);
  end_patch(); begin_patch();
  for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i)
    put(nid(i, j, 0), nid(i, j + 1, 0), nid(i + 1, j + 1, 0), nid(i + 1, j, 0), cid(i, j, 0), 0);
  end_patch(); begin_patch();
  for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i)
    put(nid(i, j, nz), nid(i + 1, j, nz), nid(i + 1, j + 1, nz), nid(i, j + 1, nz), cid(i, j, nz - 1), 0);
  end_patch();
}

// Freudenthal split of every hex into 6 tetrahedra along the v000-v111
// diagonal: conforming across hexes because every quad face is cut along the
// diagonal joining its lowest and highest vertex.
static void box_tet(fc_mesh& m, int nx, int ny, int nz) {
  auto nid = [&](int i, int j, int k) { return i + (nx + 1) * (j + (ny + 1) * k) + 1; };
  const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  const long long ncell = 6LL * nx * ny * nz;
  std::vector<int> tetv((size_t)ncell * 4);
  long long c = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        for (int p = 0; p < 6; ++p) {
          int ijk[3] = {i, j, k};
          int* t = &tetv[(size_t)c * 4];
          t[0] = nid(ijk[0], ijk[1], ijk[2]);
          ijk[perm[p][0]]++;
          t[1] = nid(ijk[0], ijk[1], ijk[2]);
          ijk[perm[p][1]]++;
          t[2] = nid(ijk[0], ijk[1], ijk[2]);
          t[3] = nid(i + 1, j + 1, k + 1);
          ++c;
        }
  struct Rec { int a, b, c; int cell; int v[3]; };
  std::vector<Rec> rec((size_t)ncell * 4);
  for (long long t = 0; t < ncell; ++t) {
    const int* tv = &tetv[(size_t)t * 4];
    for (int o = 0; o < 4; ++o) {
      Rec r;
      int q = 0;
      for (int s = 0; s < 4; ++s) if (s != o) r.v[q++] = tv[s];
      int s3[3] = {r.v[0], r.v[1], r.v[2]};
      std::sort(s3, s3 + 3);
      r.a = s3[0]; r.b = s3[1]; r.c = s3[2];
      r.cell = (int)t + 1;
      rec[(size_t)t * 4 + o] = r;
    }
  }
  std::sort(rec.begin(), rec.end(), [](const Rec& x, const Rec& y) {
    if (x.a != y.a) return x.a < y.a;
    if (x.b != y.b) return x.b < y.b;
    if (x.c != y.c) return x.c < y.c;
    return x.cell < y.cell;
  });
  auto P = [&](int v) { return V3{m.x[v - 1], m.y[v - 1], m.z[v - 1]}; };
  auto centroid = [&](int cell) {
    const int* tv = &tetv[(size_t)(cell - 1) * 4];
    V3 s{0, 0, 0};
    for (int q = 0; q < 4; ++q) { V3 p = P(tv[q]); s.x += p.x; s.y += p.y; s.z += p.z; }
    return V3{s.x / 4, s.y / 4, s.z / 4};
  };
  struct Face { int own, nb; int v[3]; };
  std::vector<Face> inner;
  std::vector<Face> bnd[6];
  inner.reserve((size_t)ncell * 2);
  for (size_t r = 0; r < rec.size();) {
    if (r + 1 < rec.size() && rec[r + 1].a == rec[r].a && rec[r + 1].b == rec[r].b && rec[r + 1].c == rec[r].c) {
      Face F;
      F.own = std::min(rec[r].cell, rec[r + 1].cell);
      F.nb = std::max(rec[r].cell, rec[r + 1].cell);
      F.v[0] = rec[r].v[0]; F.v[1] = rec[r].v[1]; F.v[2] = rec[r].v[2];
      V3 n = cross(sub(P(F.v[1]), P(F.v[0])), sub(P(F.v[2]), P(F.v[0])));
      if (dot(n, sub(centroid(F.nb), centroid(F.own))) < 0) std::swap(F.v[1], F.v[2]);
      inner.push_back(F);
      r += 2;
    } else {
      Face F;
      F.own = rec[r].cell; F.nb = 0;
      F.v[0] = rec[r].v[0]; F.v[1] = rec[r].v[1]; F.v[2] = rec[r].v[2];
      // classify the side from the lattice indices of the three vertices
      int side = -1;
      int I[3], J[3], K[3];
      for (int q = 0; q < 3; ++q) {
        int v = F.v[q] - 1;
        I[q] = v % (nx + 1); J[q] = (v / (nx + 1)) % (ny + 1); K[q] = v / ((nx + 1) * (ny + 1));
      }
      if (I[0] == 0 && I[1] == 0 && I[2] == 0) side = 0;
      else if (I[0] == nx && I[1] == nx && I[2] == nx) side = 1;
      else if (J[0] == 0 && J[1] == 0 && J[2] == 0) side = 2;
      else if (J[0] == ny && J[1] == ny && J[2] == ny) side = 3;
      else if (K[0] == 0 && K[1] == 0 && K[2] == 0) side = 4;
      else side = 5;
      V3 n = cross(sub(P(F.v[1]), P(F.v[0])), sub(P(F.v[2]), P(F.v[0])));
      V3 fc{(P(F.v[0]).x + P(F.v[1]).x + P(F.v[2]).x) / 3, (P(F.v[0]).y + P(F.v[1]).y + P(F.v[2]).y) / 3,
            (P(F.v[0]).z + P(F.v[1]).z + P(F.v[2]).z) / 3};
      if (dot(n, sub(fc, centroid(F.own))) < 0) std::swap(F.v[1], F.v[2]);
      bnd[side].push_back(F);
      r += 1;
    }
  }
  std::sort(inner.begin(), inner.end(), [](const Face& p, const Face& q) {
    if (p.own != q.own) return p.own < q.own;
    return p.nb < q.nb;
  });
  m.numInnerFaces = (int)inner.size();
  m.numBoundaryFaces = 0;
  for (int s = 0; s < 6; ++s) {
    std::sort(bnd[s].begin(), bnd[s].end(), [](const Face& p, const Face& q) { return p.own < q.own; });
    m.numBoundaryFaces += (int)bnd[s].size();
  }
  m.numFaces = m.numInnerFaces + m.numBoundaryFaces;
  m.nnodes.assign(m.numFaces, 3);
  m.nodes.assign((size_t)m.numFaces * FC_NOMAX, 0);
  m.owner.assign(m.numFaces, 0);
  m.neighbour.assign(m.numInnerFaces, 0);
  int f = 0;
  for (const Face& F : inner) {
    for (int q = 0; q < 3; ++q) m.nodes[(size_t)f * FC_NOMAX + q] = F.v[q];
    m.owner[f] = F.own; m.neighbour[f] = F.nb; ++f;
  }
  m.nfaces.clear(); m.startFace.clear();
  for (int s = 0; s < 6; ++s) {
    m.startFace.push_back(f);
    m.nfaces.push_back((int)bnd[s].size());
    for (const Face& F : bnd[s]) {
      for (int q = 0; q < 3; ++q) m.nodes[(size_t)f * FC_NOMAX + q] = F.v[q];
      m.owner[f] = F.own; ++f;
    }
  }
}

extern "C" int fc_mesh_box(int nx, int ny, int nz, double lx, double ly, double lz, double perturb,
                           unsigned long long seed, int tets, const int* side_bctype, fc_mesh** out) {
  if (!out || nx < 1 || ny < 1 || nz < 1 || !(lx > 0) || !(ly > 0) || !(lz > 0) || perturb < 0 || perturb >= 0.5)
    return FC_ERR_BAD_INPUT;
  long long ncell = (long long)nx * ny * nz * (tets ? 6 : 1);
  if (ncell > 400000000LL) return FC_ERR_BAD_INPUT;
  fc_mesh* m = new fc_mesh();
  m->numNodes = (nx + 1) * (ny + 1) * (nz + 1);
  m->numCells = (int)ncell;
  m->x.resize(m->numNodes); m->y.resize(m->numNodes); m->z.resize(m->numNodes);
  const double hx = lx / nx, hy = ly / ny, hz = lz / nz;
  SplitMix64 rng(seed);
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        int v = i + (nx + 1) * (j + (ny + 1) * k);
        double X = i * hx, Y = j * hy, Z = k * hz;
        if (perturb > 0 && i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz) {
          X += (2.0 * rng.uniform() - 1.0) * perturb * hx;
          Y += (2.0 * rng.uniform() - 1.0) * perturb * hy;
          Z += (2.0 * rng.uniform() - 1.0) * perturb * hz;
        }
        m->x[v] = X; m->y[v] = Y; m->z[v] = Z;
      }
  if (tets) box_tet(*m, nx, ny, nz); else box_hex(*m, nx, ny, nz);
  m->bctype.resize(6); m->bcname.resize(6);
  m->startFaceTwin.assign(6, -1);
  for (int s = 0; s < 6; ++s) {
    m->bctype[s] = side_bctype ? side_bctype[s] : FC_BC_WALL;
    m->bcname[s] = kSideName[s];
  }
  // a periodic side pairs with the opposite side, which must be 'empty'
  for (int s = 0; s < 6; ++s)
    if (m->bctype[s] == FC_BC_PERIODIC) m->startFaceTwin[s] = m->startFace[s ^ 1];
  std::string why;
  if (m->validate(&why, true) != FC_OK) { delete m; return FC_ERR_BAD_INPUT; }
  *out = m;
  return FC_OK;
}

extern "C" int fc_mesh_from_arrays(int numNodes, int numCells, int numInnerFaces, int numBoundaryFaces,
                                   const double* x, const double* y, const double* z, const int* nnodes,
                                   const int* nodes, const int* owner, const int* neighbour, int numBoundaries,
                                   const int* bctype, const int* nfaces, const int* startFace, fc_mesh** out) {
  if (!out || !x || !y || !z || !nnodes || !nodes || !owner || (numInnerFaces > 0 && !neighbour) || numBoundaries < 0 ||
      (numBoundaries > 0 && (!bctype || !nfaces || !startFace)))
    return FC_ERR_BAD_INPUT;
  fc_mesh* m = new fc_mesh();
  m->numNodes = numNodes; m->numCells = numCells; m->numInnerFaces = numInnerFaces;
  m->numBoundaryFaces = numBoundaryFaces; m->numFaces = numInnerFaces + numBoundaryFaces;
  if (numNodes < 0 || m->numFaces < 0) { delete m; return FC_ERR_BAD_INPUT; }
  m->x.assign(x, x + numNodes); m->y.assign(y, y + numNodes); m->z.assign(z, z + numNodes);
  m->nnodes.assign(nnodes, nnodes + m->numFaces);
  m->nodes.assign(nodes, nodes + (size_t)m->numFaces * FC_NOMAX);
  m->owner.assign(owner, owner + m->numFaces);
  if (numInnerFaces > 0) m->neighbour.assign(neighbour, neighbour + numInnerFaces);
  for (int b = 0; b < numBoundaries; ++b) {
    m->bctype.push_back(bctype[b]); m->nfaces.push_back(nfaces[b]); m->startFace.push_back(startFace[b]);
    m->bcname.push_back(std::string("patch") + std::to_string(b + 1));
    m->startFaceTwin.push_back(-1);
  }
  std::string why;
  if (m->validate(&why) != FC_OK) { delete m; return FC_ERR_BAD_INPUT; }
  *out = m;
  return FC_OK;
}

extern "C" int fc_mesh_write_native(const fc_mesh* m, const char* dir) {
  if (!m || !dir) return FC_ERR_BAD_INPUT;
  std::string d(dir);
  auto open = [&](const char* name) { return std::fopen((d + "/" + name).c_str(), "w"); };
  FILE* f = open("points");
  if (!f) return FC_ERR_BAD_INPUT;
  for (int i = 0; i < m->numNodes; ++i) std::fprintf(f, "%.17g %.17g %.17g\n", m->x[i], m->y[i], m->z[i]);
  std::fclose(f);
  f = open("faces");
  if (!f) return FC_ERR_BAD_INPUT;
  for (int i = 0; i < m->numFaces; ++i) {
    std::fprintf(f, "%d", m->nnodes[i]);
    for (int k = 0; k < m->nnodes[i]; ++k) std::fprintf(f, " %d", m->nodes[(size_t)i * FC_NOMAX + k]);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
  f = open("owner");
  if (!f) return FC_ERR_BAD_INPUT;
  for (int i = 0; i < m->numFaces; ++i) std::fprintf(f, "%d\n", m->owner[i]);
  std::fclose(f);
  f = open("neighbour");
  if (!f) return FC_ERR_BAD_INPUT;
  for (int i = 0; i < m->numInnerFaces; ++i) std::fprintf(f, "%d\n", m->neighbour[i]);
  std::fclose(f);
  f = open("boundary");
  if (!f) return FC_ERR_BAD_INPUT;
  write_boundary_lines(f, *m);
  std::fclose(f);
  f = open("size");
  if (!f) return FC_ERR_BAD_INPUT;
  std::fprintf(f, "%d\n%d\n%d\n%d\n%d\n", m->numNodes, m->numCells, m->numInnerFaces, m->numBoundaryFaces, m->numFaces);
  std::fclose(f);
  return FC_OK;
}

extern "C" int fc_mesh_read_native(const char* dir, fc_mesh** out) {
  if (!dir || !out) return FC_ERR_BAD_INPUT;
  std::string d(dir);
  std::ifstream fs(d + "/size");
  if (!fs) return FC_ERR_BAD_INPUT;
  fc_mesh* m = new fc_mesh();
  fs >> m->numNodes >> m->numCells >> m->numInnerFaces >> m->numBoundaryFaces >> m->numFaces;
  if (!fs || m->numNodes <= 0 || m->numFaces != m->numInnerFaces + m->numBoundaryFaces) { delete m; return FC_ERR_BAD_INPUT; }
  std::ifstream fb(d + "/boundary");
  std::string line;
  while (fb && std::getline(fb, line)) {
    if (line.empty() || line[0] == '#') continue;
    if (!parse_boundary_line(line, m)) { delete m; return FC_ERR_BAD_INPUT; }
  }
  std::ifstream fp(d + "/points");
  m->x.resize(m->numNodes); m->y.resize(m->numNodes); m->z.resize(m->numNodes);
  for (int i = 0; i < m->numNodes; ++i) fp >> m->x[i] >> m->y[i] >> m->z[i];
  std::ifstream ff(d + "/faces");
  m->nnodes.assign(m->numFaces, 0);
  m->nodes.assign((size_t)m->numFaces * FC_NOMAX, 0);
  for (int i = 0; i < m->numFaces; ++i) {
    ff >> m->nnodes[i];
    if (m->nnodes[i] < 0 || m->nnodes[i] > FC_NOMAX) { delete m; return FC_ERR_BAD_INPUT; }
    for (int k = 0; k < m->nnodes[i]; ++k) ff >> m->nodes[(size_t)i * FC_NOMAX + k];
  }
  std::ifstream fo(d + "/owner");
  m->owner.resize(m->numFaces);
  for (int i = 0; i < m->numFaces; ++i) fo >> m->owner[i];
  std::ifstream fn(d + "/neighbour");
  m->neighbour.resize(m->numInnerFaces);
  for (int i = 0; i < m->numInnerFaces; ++i) fn >> m->neighbour[i];
  if (!fp || !ff || !fo || (m->numInnerFaces > 0 && !fn)) { delete m; return FC_ERR_BAD_INPUT; }
  std::string why;
  if (m->validate(&why) != FC_OK) { delete m; return FC_ERR_BAD_INPUT; }
  *out = m;
  return FC_OK;
}

extern "C" int fc_mesh_info(const fc_mesh* m, int* info) {
  if (!m || !info) return FC_ERR_BAD_INPUT;
  info[0] = m->numNodes; info[1] = m->numCells; info[2] = m->numInnerFaces;
  info[3] = m->numBoundaryFaces; info[4] = m->numFaces; info[5] = (int)m->bctype.size();
  return FC_OK;
}

extern "C" int fc_mesh_export(const fc_mesh* m, double* x, double* y, double* z, int* nnodes, int* nodes, int* owner,
                              int* neighbour, int* bctype, int* nfaces, int* startFace) {
  if (!m) return FC_ERR_BAD_INPUT;
  if (x) std::memcpy(x, m->x.data(), sizeof(double) * m->numNodes);
  if (y) std::memcpy(y, m->y.data(), sizeof(double) * m->numNodes);
  if (z) std::memcpy(z, m->z.data(), sizeof(double) * m->numNodes);
  if (nnodes) std::memcpy(nnodes, m->nnodes.data(), sizeof(int) * m->numFaces);
  if (nodes) std::memcpy(nodes, m->nodes.data(), sizeof(int) * (size_t)m->numFaces * FC_NOMAX);
  if (owner) std::memcpy(owner, m->owner.data(), sizeof(int) * m->numFaces);
  if (neighbour && m->numInnerFaces) std::memcpy(neighbour, m->neighbour.data(), sizeof(int) * m->numInnerFaces);
  size_t nb = m->bctype.size();
  if (bctype && nb) std::memcpy(bctype, m->bctype.data(), sizeof(int) * nb);
  if (nfaces && nb) std::memcpy(nfaces, m->nfaces.data(), sizeof(int) * nb);
  if (startFace && nb) std::memcpy(startFace, m->startFace.data(), sizeof(int) * nb);
  return FC_OK;
}

extern "C" int fc_mesh_set_twin(fc_mesh* m, int patch, int startFaceTwin) {
  if (!m || patch < 0 || patch >= (int)m->bctype.size() || m->bctype[patch] != FC_BC_PERIODIC) return FC_ERR_BAD_INPUT;
  m->startFaceTwin.resize(m->bctype.size(), -1);
  const int old = m->startFaceTwin[patch];
  m->startFaceTwin[patch] = startFaceTwin;
  std::string why;
  if (m->validate(&why) != FC_OK) {
    m->startFaceTwin[patch] = old;
    return FC_ERR_BAD_INPUT;
  }
  return FC_OK;
}

extern "C" int fc_mesh_twins(const fc_mesh* m, int* startFaceTwin) {
  if (!m || !startFaceTwin) return FC_ERR_BAD_INPUT;
  for (size_t b = 0; b < m->bctype.size(); ++b) startFaceTwin[b] = m->twin_of(b);
  return FC_OK;
}

extern "C" void fc_mesh_free(fc_mesh* m) { delete m; }
