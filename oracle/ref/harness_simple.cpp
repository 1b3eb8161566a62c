// Oracle harness around the reference's pressure-based SIMPLE path (test
// infrastructure only; built into oracle/_ref by oracle/ref/build_ref.sh).
//
// It drives the reference's own classes the way Work::work and Time do with
// RHO_P 1 and FLAGPSUEDO 0 (time/Time.cpp:54-80, pSolver/PSolver.cpp:19-24):
// MshBlock::readMsh -> AllData::createAllData -> Time::initialization ->
// per time step a fresh SolverSIMPLE{setDT(1/STEP_TIME), solve} (which copies
// the old cell PUVT into the old-time-level array in its constructor,
// pSolver/SolverSIMPLE.cpp:34-36), the Time loop's residual row, then
// PSolver::updateNewToOld (pSolver/PSolver.cpp:38-44).
//
// Outputs (raw little-endian binaries and text):
//   puvt.f64     cell (p, u, v, T) after the last step   [n_cells][4]
//   face_sc.f64  face (p, u, v, T) the last solve used   [n_faces][4]
//   time.log     the SIMPLE iteration rows the solver writes to the log
//                (SolverSIMPLE.cpp:77; default stream precision)
//   time_rows.f64  per step the Time loop's residual row (Time.cpp:66-74),
//                full precision                          [steps][4]
//   gs.log       the solver's stdout: LU-residual-GS lines of every
//                Gauss-Seidel solve (lusolver/SparseSolverNUM.cpp:242)
//
// usage: ref_simple MESH OUTDIR [--puvt0 FILE] [--steps N] [--bench N]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "time/Time.h"
#include "pSolver/SolverSIMPLE.h"

static void dump(const std::string& dir, const char* name, const void* p,
                 size_t bytes) {
  std::string path = dir + "/" + name;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  if (bytes) std::fwrite(p, 1, bytes, f);
  std::fclose(f);
}

// The reference reads text with getline and keeps any '\r'; give it an
// LF-only copy in the output directory.
static std::string lf_copy(const std::string& src, const std::string& dir) {
  std::ifstream in(src, std::ios::binary);
  if (!in) {
    std::fprintf(stderr, "cannot read %s\n", src.c_str());
    std::exit(2);
  }
  std::string s((std::istreambuf_iterator<char>(in)),
                std::istreambuf_iterator<char>());
  std::string o;
  o.reserve(s.size());
  for (char c : s)
    if (c != '\r') o.push_back(c);
  std::string dst = dir + "/mesh.msh";
  std::ofstream out(dst, std::ios::binary);
  out << o;
  return dst;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s MESH OUTDIR [opts]\n", argv[0]);
    return 1;
  }
  std::string mesh_path = argv[1], out = argv[2];
  std::string p0file;
  int steps = 1, bench = 0;
  for (int i = 3; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "--puvt0" && i + 1 < argc) p0file = argv[++i];
    else if (a == "--steps" && i + 1 < argc) steps = std::atoi(argv[++i]);
    else if (a == "--bench" && i + 1 < argc) bench = std::atoi(argv[++i]);
    else {
      std::fprintf(stderr, "bad option %s\n", a.c_str());
      return 1;
    }
  }

  std::string lf = lf_copy(mesh_path, out);
  MshBlock mesh;
  mesh.readMsh(lf);
  const int nC = mesh.getNumOfCells(), nF = mesh.getNumOfFaces();

  AllData data;
  data.createAllData(nC, nF);
  std::fstream flog;
  flog.open(out + "/time.log", std::ios::out | std::ios::trunc);
  Time timeLoop(&mesh, &flog, &data);
  VCTDIMU iniQ;
  iniQ << inirho, inirho * iniu, inirho * iniv, iniE;
  timeLoop.initialization(iniQ);
  if (!p0file.empty()) {
    std::vector<double> p(4 * (size_t)nC);
    FILE* f = std::fopen(p0file.c_str(), "rb");
    if (!f || std::fread(p.data(), 8, p.size(), f) != p.size()) {
      std::fprintf(stderr, "bad puvt0 file %s\n", p0file.c_str());
      return 2;
    }
    std::fclose(f);
    for (int c = 0; c < nC; ++c)
      for (int m = 0; m < 4; ++m) {
        data.getPNewCellPUVT()[c](m) = p[4 * c + m];
        data.getPOldCellPUVT()[c](m) = p[4 * c + m];
      }
  }

  // The solver's stdout (Gauss-Seidel residual lines, SIMPLE rows) to gs.log
  std::ofstream gslog(out + "/gs.log");
  std::streambuf* saved = std::cout.rdbuf(gslog.rdbuf());

  const int total = bench > 0 ? bench : steps;
  std::vector<double> rows;
  auto t0 = std::chrono::steady_clock::now();
  for (int s = 0; s < total; ++s) {
    SolverSIMPLE solver(&mesh, &flog, &data);
    solver.setDT(1. / STEP_TIME);
    solver.solve();
    VCTDIMU* oldValue = data.getPOldNTimeCellPUVT();
    VCTDIMU* newValue = data.getPNewCellPUVT();
    VCTDIMU residual = VCTDIMU::Zero();
    for (int i = 0; i < nC; i++)
      for (int iR = 0; iR < DIMU; iR++)
        if (residual[iR] < std::abs(newValue[i][iR] - oldValue[i][iR]) / oldValue[i][iR])
          residual[iR] = std::abs(newValue[i][iR] - oldValue[i][iR]) / oldValue[i][iR];
    for (int m = 0; m < 4; ++m) rows.push_back(residual[m]);
    for (int i = 0; i < nC; i++) data.getPOldCellPUVT()[i] = data.getPNewCellPUVT()[i];
  }
  auto t1 = std::chrono::steady_clock::now();
  std::cout.rdbuf(saved);
  flog.close();

  if (bench > 0) {
    std::printf("%.9f\n", std::chrono::duration<double>(t1 - t0).count() / bench);
    return 0;
  }
  std::vector<double> pv(4 * (size_t)nC), fs(4 * (size_t)nF);
  for (int c = 0; c < nC; ++c)
    for (int m = 0; m < 4; ++m) pv[4 * c + m] = data.getPNewCellPUVT()[c](m);
  for (int f = 0; f < nF; ++f)
    for (int m = 0; m < 4; ++m) fs[4 * f + m] = data.getPFacePUVTSC()[f](m);
  dump(out, "puvt.f64", pv.data(), pv.size() * 8);
  dump(out, "face_sc.f64", fs.data(), fs.size() * 8);
  dump(out, "time_rows.f64", rows.data(), rows.size() * 8);
  return 0;
}
