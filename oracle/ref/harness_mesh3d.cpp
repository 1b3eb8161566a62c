// Oracle harness around the reference's 3D mesh reader (test infrastructure
// only; built into oracle/_ref/mesh3d by oracle/ref/build_ref.sh with the
// reference's CONST.h overridden to DIM 3).
//
// MshBlock::readMsh -> splitInformationData3D / dataToMesh3D
// (mesh/MshBlock.cpp:436-789), then every geometric and connectivity array
// the product's 3D reader reproduces, as raw little-endian binaries.  The
// L-neighbour lists are private members of Cell; the harness opens them
// with a preprocessor switch around the include, as harness_io.cpp does.
//
// usage: ref_mesh3d MESH OUTDIR
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <iomanip>
#include <iostream>
#include <istream>
#include <limits>
#include <math.h>
#include <sstream>
#include <type_traits>
#include <Eigen/Dense>
#include <Eigen/Eigen>

#define private public
#include "mesh/MshBlock.h"
#undef private

static void dump(const std::string& dir, const char* name, const void* p, size_t bytes) {
  std::string path = dir + "/" + name;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  if (bytes) std::fwrite(p, 1, bytes, f);
  std::fclose(f);
}

static std::string lf_copy(const std::string& src, const std::string& dir) {
  std::ifstream in(src, std::ios::binary);
  if (!in) {
    std::fprintf(stderr, "cannot read %s\n", src.c_str());
    std::exit(2);
  }
  std::string s((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  std::string o;
  for (char c : s)
    if (c != '\r') o.push_back(c);
  std::string dst = dir + "/mesh3d.msh";
  std::ofstream out(dst, std::ios::binary);
  out << o;
  return dst;
}

template <class T>
static void put(const std::string& dir, const char* name, const std::vector<T>& v) {
  dump(dir, name, v.data(), v.size() * sizeof(T));
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: ref_mesh3d MESH OUTDIR\n");
    return 2;
  }
  const std::string dir = argv[2];
  MshBlock* mb = new MshBlock();
  mb->readMsh(lf_copy(argv[1], dir));
  const int nN = mb->getNumOfNodes(), nC = mb->getNumOfCells(), nF = mb->getNumOfFaces();
  Node* nodes = mb->getBeginItNodesList();
  Face* faces = mb->getBeginItFacesList();
  Cell* cells = mb->getBeginItCellsList();
  std::vector<double> xyz, fctr, fdir, farea, feta, fcmd, cctr, cvol, dof, e0c;
  std::vector<int> counts, fdac, fcells, fptr{0}, fnodes, cptr{0}, cfaces, cnb, nptr{0}, cnodes,
      nlow;
  std::vector<unsigned char> flag;
  for (int i = 0; i < nN; ++i)
    for (int d = 0; d < 3; ++d) xyz.push_back(nodes[i].getCenter()(d));
  for (int f = 0; f < nF; ++f) {
    Face& F = faces[f];
    for (int d = 0; d < 3; ++d) {
      fctr.push_back(F.getCenter()(d));
      fdir.push_back(F.getDirect()(d));
      flag.push_back(F.getFlagLeftRight()[d] ? 1 : 0);
    }
    farea.push_back(F.getArea());
    feta.push_back(F.getEta0());
    fdac.push_back(F.getDirectAndCells());
    auto cb = F.getBeginItPNbCells();
    fcells.push_back(cb[0]->getId());
    fcells.push_back(F.getNumOfpNbCells() == 2 ? cb[1]->getId() : -1);
    auto nb = F.getBeginItPNbNodes();
    for (int j = 0; j < F.getNumOfpNbNodes(); ++j) fnodes.push_back(nb[j]->getId());
    fptr.push_back((int)fnodes.size());
    for (int d = 0; d < 3; ++d)
      fcmd.push_back(f < mb->getNumOfIntFaces() ? F.getCenterMiddleDef()(d) : 0.0);
  }
  for (int c = 0; c < nC; ++c) {
    Cell& C = cells[c];
    for (int d = 0; d < 3; ++d) cctr.push_back(C.getCenter()(d));
    cvol.push_back(C.getVolume());
    auto fb = C.getBeginItPNbFaces();
    auto cb = C.getBeginItPNbCells();
    VCTDIM* dv = C.getBeginItDirectOfNbFaces();
    NUM* e0 = C.getBeginItEta0C();
    for (int k = 0; k < C.getNumOfNbFaces(); ++k) {
      cfaces.push_back(fb[k]->getId());
      cnb.push_back(cb[k]->getId());
      for (int d = 0; d < 3; ++d) dof.push_back(dv[k](d));
      e0c.push_back(e0[k]);
    }
    cptr.push_back((int)cfaces.size());
    auto nb = C.getBeginItPNbNodes();
    for (int k = 0; k < C.getNumOfNbNodes(); ++k) cnodes.push_back(nb[k]->getId());
    nptr.push_back((int)cnodes.size());
    nlow.push_back((int)C.pNbCellL.size());
  }
  counts = {nN, nC, nF, mb->getNumOfIntFaces(), mb->getNumOfInnerCells(),
            mb->getNumOfBond1Cells(), mb->getNumOfBond2Cells()};
  std::vector<int> inner(mb->getBeginItInnerIdList(),
                         mb->getBeginItInnerIdList() + mb->getNumOfInnerCells());
  std::vector<int> b1(mb->getBeginItBond1IdList(),
                      mb->getBeginItBond1IdList() + mb->getNumOfBond1Cells());
  std::vector<int> b2(mb->getBeginItBond2IdList(),
                      mb->getBeginItBond2IdList() + mb->getNumOfBond2Cells());
  put(dir, "counts.i32", counts);
  put(dir, "node_xyz.f64", xyz);
  put(dir, "face_ctr.f64", fctr);
  put(dir, "face_dir.f64", fdir);
  put(dir, "face_area.f64", farea);
  put(dir, "face_eta0.f64", feta);
  put(dir, "face_cmd.f64", fcmd);
  put(dir, "face_dac.i32", fdac);
  put(dir, "face_flag.u8", flag);
  put(dir, "face_cells.i32", fcells);
  put(dir, "face_ptr.i32", fptr);
  put(dir, "face_nodes.i32", fnodes);
  put(dir, "cell_ctr.f64", cctr);
  put(dir, "cell_vol.f64", cvol);
  put(dir, "cell_ptr.i32", cptr);
  put(dir, "cell_faces.i32", cfaces);
  put(dir, "cell_nb.i32", cnb);
  put(dir, "cell_dof.f64", dof);
  put(dir, "cell_eta0c.f64", e0c);
  put(dir, "cell_node_ptr.i32", nptr);
  put(dir, "cell_nodes.i32", cnodes);
  put(dir, "cell_nlow.i32", nlow);
  put(dir, "inner.i32", inner);
  put(dir, "bond1.i32", b1);
  put(dir, "bond2.i32", b2);
  std::fflush(stdout);
  std::_Exit(0);
}
