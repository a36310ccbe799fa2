// Host mesh record in the reference's native layout (1-based indices).
#pragma once
#include <string>
#include <vector>

#include "fc_gpu.h"

// the reference's boundary type names ('wall', 'inlet', ...) and FC_BC_*
const char* bc_name_of(int t);
int bc_type_of(const std::string& s);

struct fc_mesh {
  int numNodes = 0, numCells = 0, numInnerFaces = 0, numBoundaryFaces = 0, numFaces = 0;
  std::vector<double> x, y, z;      // numNodes
  std::vector<int> nnodes;          // numFaces
  std::vector<int> nodes;           // numFaces * FC_NOMAX, 1-based, zero padded
  std::vector<int> owner;           // numFaces, 1-based
  std::vector<int> neighbour;       // numInnerFaces, 1-based
  std::vector<std::string> bcname;  // per patch
  std::vector<int> bctype, nfaces, startFace;  // per patch; startFace is a 0-based face offset
  int validate(std::string* why) const;
};
