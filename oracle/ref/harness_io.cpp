// Oracle harness around the reference's result writer and checkpoint files
// (test infrastructure only; built into oracle/_ref by oracle/ref/build_ref.sh).
//
// It reads a mesh with the reference's MshBlock, loads a cell state, and calls
// the reference's own Work members (work/Work.cpp):
//   writedataRhoBasedMshNodePlt (:204-319)  the Tecplot node-averaged .plt,
//   writedataCellContinue       (:483-514)  the text .cellPUVT checkpoint,
//   readPbasedCellPlt           (:432-482)  its reader (round trip dumped).
// Work keeps these members private; the harness opens them with a
// preprocessor switch around the include, the usual way a test reaches
// private members of code it may not change.
//
// usage: ref_io MESH OUTDIR QFILE ZONE_T TIME_NOW
//   QFILE: nC x 4 little-endian doubles (file cell order)
//   writes OUTDIR/result/mesh.msh_TIME4000_u0_t<TIME_NOW>.plt and .cellPUVT
//   and OUTDIR/readback.bin (the state readPbasedCellPlt reads back).
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

// Every library header the reference pulls in comes first, so the switch
// below reaches only the reference's own classes.
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
#include <omp.h>
#include <Eigen/Dense>
#include <Eigen/Eigen>

#define private public
#include "work/Work.h"
#undef private

static std::string lf_copy(const std::string& src, const std::string& dir) {
  std::ifstream in(src, std::ios::binary);
  if (!in) {
    std::fprintf(stderr, "cannot read %s\n", src.c_str());
    std::exit(2);
  }
  std::string s((std::istreambuf_iterator<char>(in)),
                std::istreambuf_iterator<char>());
  std::string o;
  for (char c : s)
    if (c != '\r') o.push_back(c);
  std::string dst = dir + "/mesh.msh";
  std::ofstream out(dst, std::ios::binary);
  out << o;
  return dst;
}

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: ref_io MESH OUTDIR QFILE ZONE_T TIME_NOW\n");
    return 2;
  }
  // DIMU is an unparenthesised DIM + 2 in the reference's CONST.h.
  const int NV = (DIMU);
  std::string dir = argv[2];
  std::string msh = lf_copy(argv[1], dir);
  std::string qpath = argv[3];
  if (qpath[0] != '/') qpath = std::string(getcwd(nullptr, 0)) + "/" + qpath;
  // The checkpoint members reset the output folder to "./" (Work.cpp:484,433).
  if (chdir(dir.c_str()) != 0 || (mkdir("result", 0755) != 0 && errno != EEXIST)) {
    std::fprintf(stderr, "cannot use %s\n", dir.c_str());
    return 2;
  }
  Work* wk = new Work();
  wk->mshAddress = "./";
  wk->mshName = "mesh.msh";
  wk->t = std::atoi(argv[4]);
  int time_now = std::atoi(argv[5]);
  wk->mesh.readMsh("mesh.msh");
  int nC = wk->mesh.getNumOfCells();
  wk->allData.createAllData(nC, wk->mesh.getNumOfFaces());
  std::vector<double> q((size_t)nC * NV);
  FILE* f = std::fopen(qpath.c_str(), "rb");
  if (!f || std::fread(q.data(), 8, q.size(), f) != q.size()) {
    std::fprintf(stderr, "cannot read %s\n", argv[3]);
    return 2;
  }
  std::fclose(f);
  VCTDIMU* cq = wk->allData.getP1OldCellQs();
  VCTDIMU* puvt = wk->allData.getPNewCellPUVT();
  for (int i = 0; i < nC; i++)
    for (int k = 0; k < NV; k++) {
      cq[i](k) = q[(size_t)i * NV + k];
      puvt[i](k) = q[(size_t)i * NV + k];
    }
  wk->writedataRhoBasedMshNodePlt(&wk->mesh, cq, time_now);
  wk->writedataCellContinue("mesh.msh", time_now);
  for (int i = 0; i < nC; i++)
    for (int k = 0; k < NV; k++) puvt[i](k) = 0;
  // readPbasedCellPlt reads the file of step READ_PLT; point it at ours by
  // renaming (READ_PLT is a compile-time constant of the reference).
  {
    char a[64], b[64];
    std::snprintf(a, sizeof a, "_t%d.cellPUVT", time_now);
    std::snprintf(b, sizeof b, "_t%d.cellPUVT", (int)READ_PLT);
    std::string base = "result/mesh.msh_TIME4000_u0";
    if (std::string(a) != std::string(b)) {
      std::ifstream in(base + a, std::ios::binary);
      std::ofstream out(base + b, std::ios::binary);
      out << in.rdbuf();
    }
  }
  wk->readPbasedCellPlt("mesh.msh");
  std::vector<double> back((size_t)nC * NV);
  for (int i = 0; i < nC; i++)
    for (int k = 0; k < NV; k++) back[(size_t)i * NV + k] = puvt[i](k);
  FILE* g = std::fopen("readback.bin", "wb");
  std::fwrite(back.data(), 8, back.size(), g);
  std::fclose(g);
  std::fflush(stdout);
  std::_Exit(0);  // skip ~Work: it frees mesh arrays the harness shares
}
