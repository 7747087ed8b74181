// Host-side geometry of one core (box, outline, neighbour masks, sweep
// order), built from the reference's sdata view by build_geometry (capi.cu)
// and used by the single-core handle and the batch.
#pragma once

#include <string>
#include <vector>

#include "../../include/adpres_gb300.h"

namespace adp {

struct HostGeom {
  int nxx = 0, nyy = 0, nzz = 0, nnod = 0, NB = 0, plane = 0;
  long long NBH = 0;
  int bcf[6] = {0, 0, 0, 0, 0, 0};               // faces X+ X- Y+ Y- Z+ Z-
  std::vector<int> node2box;                       // [nnod] box index in reference node order
  std::vector<int> ysmin, ysmax, xsmin, xsmax;     // plane-1 outline, 0-based
  std::vector<int> evbase;                         // [3][NB] sweep-order index of a node's minus face
  std::vector<unsigned char> nbm;                  // [NB] neighbour mask
  std::vector<double> xdel, ydel, zdel, vdel;
};

adp_status build_geometry(const adp_geom& g, HostGeom& H, std::string& err);

}  // namespace adp
