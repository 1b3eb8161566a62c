// Drop-in check (test infrastructure only): the reference's own time loop,
// written as Time::goNextTimeStep does it (time/Time.cpp:54-80), with the
// reference's RhoSolver replaced by GpuRhoSolver from
// include/mstcfd_gpu_rhosolver.hpp.  Compiled against the reference headers
// in oracle/_ref by tests/test_dropin.py (it needs a GPU to run).
//
// usage: dropin MESH OUTDIR NSTEPS
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "time/Time.h"
#include "mstcfd_gpu_rhosolver.hpp"

int main(int argc, char** argv) {
  if (argc != 4) return 1;
  MshBlock mesh;
  mesh.readMsh(argv[1]);
  AllData data;
  data.createAllData(mesh.getNumOfCells(), mesh.getNumOfFaces());
  std::fstream flog;
  Time timeLoop(&mesh, &flog, &data);
  VCTDIMU iniQ;
  iniQ << inirho, inirho * iniu, inirho * iniv, iniE;
  timeLoop.initialization(iniQ);
  for (int s = 0; s < std::atoi(argv[3]); ++s) {
    GpuRhoSolver thisSolver(&mesh, &flog, &data);
    thisSolver.setDT(1. / STEP_TIME);
    thisSolver.solve();
    thisSolver.updateNewToOld();
  }
  std::string out = std::string(argv[2]) + "/q_dropin.f64";
  FILE* f = std::fopen(out.c_str(), "wb");
  for (int c = 0; c < mesh.getNumOfCells(); ++c)
    for (int m = 0; m < 4; ++m) {
      double v = data.getP1OldCellQs()[c](m);
      std::fwrite(&v, 8, 1, f);
    }
  std::fclose(f);
  return 0;
}
