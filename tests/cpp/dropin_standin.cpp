// Drop-in check on machines without the reference sources: stand-in mesh and
// state classes exposing the getters of the reference's MshBlock, Node, Face,
// Cell, FacesInf and AllData (mesh/MshBlock.h, data/AllData.h), driven
// through GpuRhoSolverT exactly like Time::goNextTimeStep drives RhoSolver.
//
// input (binary): int32 nN, nC, nF, nZ, nsteps; f64 node_xy[nN*2];
//   int32 face_nodes[nF*2]; int32 face_cells[nF*2]; int32 zones[nZ*4];
//   f64 q0[nC*4].   output: f64 q[nC*4] after nsteps steps.
#include <cstdio>
#include <vector>

#include "Eigen/Dense"
#include "mstcfd_gpu_rhosolver.hpp"

typedef Eigen::Matrix<double, 2, 1> Vec2;
typedef Eigen::Matrix<double, 4, 1> Vec4;

struct Node {
  Vec2 c;
  int id;
  Vec2 getCenter() { return c; }
  int getId() { return id; }
};
struct Cell {
  int id;
  int getId() { return id; }
};
struct Face {
  std::vector<Node*> nodes;
  std::vector<Cell*> cells;
  std::vector<Node*>::iterator getBeginItPNbNodes() { return nodes.begin(); }
  std::vector<Cell*>::iterator getBeginItPNbCells() { return cells.begin(); }
  int getNumOfpNbCells() { return (int)cells.size(); }
};
struct FacesInf {
  int num, st, en, ty;
  int getNumber() { return num; }
  int getStart() { return st; }
  int getEnd() { return en; }
  int getType() { return ty; }
};
struct Block {
  std::vector<Node> nodes;
  std::vector<Cell> cells;
  std::vector<Face> faces;
  std::vector<FacesInf> zones;
  int getNumOfNodes() { return (int)nodes.size(); }
  int getNumOfCells() { return (int)cells.size(); }
  int getNumOfFaces() { return (int)faces.size(); }
  int getNumOfFacesInfs() { return (int)zones.size(); }
  Node* getBeginItNodesList() { return nodes.data(); }
  Face* getBeginItFacesList() { return faces.data(); }
  std::vector<FacesInf>::iterator getBeginItFacesInfList() { return zones.begin(); }
};
struct Data {
  std::vector<Vec4> oldq, newq, ntq;
  Vec4* getP1OldCellQs() { return oldq.data(); }
  Vec4* getP1NewCellQs() { return newq.data(); }
  Vec4* getPtP1OldNTimeCellQs() { return ntq.data(); }
};

template <class T>
static void rd(FILE* f, T* p, size_t n) {
  if (n && std::fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short input");
}

int main(int argc, char** argv) {
  if (argc != 3) return 1;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int h[5];
  rd(f, h, 5);
  const int nN = h[0], nC = h[1], nF = h[2], nZ = h[3], nsteps = h[4];
  std::vector<double> xy(2 * (size_t)nN), q0(4 * (size_t)nC);
  std::vector<int> fn(2 * (size_t)nF), fc(2 * (size_t)nF), z(4 * (size_t)nZ);
  rd(f, xy.data(), xy.size());
  rd(f, fn.data(), fn.size());
  rd(f, fc.data(), fc.size());
  rd(f, z.data(), z.size());
  rd(f, q0.data(), q0.size());
  std::fclose(f);
  Block b;
  b.nodes.resize(nN);
  for (int i = 0; i < nN; ++i) {
    b.nodes[i].c(0) = xy[2 * i];
    b.nodes[i].c(1) = xy[2 * i + 1];
    b.nodes[i].id = i;
  }
  b.cells.resize(nC);
  for (int i = 0; i < nC; ++i) b.cells[i].id = i;
  b.faces.resize(nF);
  for (int i = 0; i < nF; ++i) {
    b.faces[i].nodes = {&b.nodes[fn[2 * i]], &b.nodes[fn[2 * i + 1]]};
    b.faces[i].cells.push_back(&b.cells[fc[2 * i]]);
    if (fc[2 * i + 1] >= 0) b.faces[i].cells.push_back(&b.cells[fc[2 * i + 1]]);
  }
  for (int k = 0; k < nZ; ++k) b.zones.push_back({z[4 * k], z[4 * k + 1], z[4 * k + 2], z[4 * k + 3]});
  Data d;
  d.oldq.resize(nC);
  for (int c = 0; c < nC; ++c)
    for (int m = 0; m < 4; ++m) d.oldq[c](m) = q0[4 * c + m];
  d.newq = d.oldq;
  d.ntq = d.oldq;
  for (int s = 0; s < nsteps; ++s) {
    mstcfd::GpuRhoSolverT<Block, Data, Vec4> solver(&b, nullptr, &d);
    solver.setDT(1. / 4e+3);
    solver.solve();
    solver.updateNewToOld();
  }
  FILE* o = std::fopen(argv[2], "wb");
  for (int c = 0; c < nC; ++c)
    for (int m = 0; m < 4; ++m) {
      double v = d.oldq[c](m);
      std::fwrite(&v, 8, 1, o);
    }
  std::fclose(o);
  mstcfd::release_mesh(&b);
  return 0;
}
