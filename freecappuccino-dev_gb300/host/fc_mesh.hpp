// Host mesh record in the reference's native layout (1-based indices).
#pragma once
#include <cstdio>
#include <string>
#include <vector>

#include "fc_gpu.h"

// the reference's boundary type names ('wall', 'inlet', ...) and FC_BC_*
const char* bc_name_of(int t);
int bc_type_of(const std::string& s);

struct fc_mesh;
// the reference's boundary-file lines (shared by the native and the OpenFOAM
// readers and writers)
bool parse_boundary_line(const std::string& line, fc_mesh* m);
void write_boundary_lines(FILE* f, const fc_mesh& m);

struct fc_mesh {
  int numNodes = 0, numCells = 0, numInnerFaces = 0, numBoundaryFaces = 0, numFaces = 0;
  std::vector<double> x, y, z;      // numNodes
  std::vector<int> nnodes;          // numFaces
  std::vector<int> nodes;           // numFaces * FC_NOMAX, 1-based, zero padded
  std::vector<int> owner;           // numFaces, 1-based
  std::vector<int> neighbour;       // numInnerFaces, 1-based
  std::vector<std::string> bcname;  // per patch
  std::vector<int> bctype, nfaces, startFace;  // per patch; startFace is a 0-based face offset
  // per patch: the 0-based startFace of a 'periodic' patch's twin (the fifth
  // field of its boundary-file line, geometry.f90:250-258), -1 elsewhere
  std::vector<int> startFaceTwin;
  // complete: every periodic patch must name its twin (a mesh handed to a
  // context); otherwise a periodic patch may still lack it (fc_mesh_set_twin
  // follows)
  int validate(std::string* why, bool complete = false) const;
  int twin_of(size_t b) const { return b < startFaceTwin.size() ? startFaceTwin[b] : -1; }
};
