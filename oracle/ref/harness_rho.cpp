// Oracle harness around the reference's density-based path (test
// infrastructure only; built into oracle/_ref by oracle/ref/build_ref.sh).
//
// It drives the reference's own classes exactly as Work::work / Time do
// (work/Work.cpp:7-92, time/Time.cpp:13-107): MshBlock::readMsh ->
// AllData::createAllData -> Time::initialization -> RhoSolver{setDT, solve},
// and dumps every quantity the GPU path must reproduce as raw little-endian
// binaries:
//   mesh geometry/connectivity (mesh/MshBlock.cpp:111-432),
//   per-face flux matrices p1OldFaceConvectFlux (rhoSolver/RhoSolver.cpp:90-369),
//   per-cell residual R_c gathered in the order of RhoSolver.cpp:45-56,
//   the updated state p1NewCellQs (RhoSolver.cpp:64),
//   and, for --time-steps, the state after Time::goNextTimeStep loops plus
//   the L-infinity residual lines the reference writes to its log
//   (time/Time.cpp:66-78).
//
// usage: ref_rho MESH OUTDIR [--q0 FILE] [--dt DT] [--remap5to3]
//                [--time-steps N] [--bench N]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "time/Time.h"

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

// The reference reads text with getline and keeps any '\r' (it was written
// for Windows text mode); give it an LF-only copy in the output directory.
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
  std::string q0file;
  double dt = 1.0 / STEP_TIME;
  bool remap5 = false;
  int time_steps = 0, bench = 0;
  for (int i = 3; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "--q0" && i + 1 < argc) q0file = argv[++i];
    else if (a == "--dt" && i + 1 < argc) dt = std::atof(argv[++i]);
    else if (a == "--remap5to3") remap5 = true;
    else if (a == "--time-steps" && i + 1 < argc) time_steps = std::atoi(argv[++i]);
    else if (a == "--bench" && i + 1 < argc) bench = std::atoi(argv[++i]);
    else {
      std::fprintf(stderr, "bad option %s\n", a.c_str());
      return 1;
    }
  }

  std::string lf = lf_copy(mesh_path, out);
  MshBlock mesh;
  mesh.readMsh(lf);
  const int nN = mesh.getNumOfNodes(), nC = mesh.getNumOfCells(),
            nF = mesh.getNumOfFaces(), nI = mesh.getNumOfIntFaces(),
            nZ = mesh.getNumOfFacesInfs();

  if (remap5) {
    // The reference's 2nd-order outlet writes through never-allocated
    // pointers (RhoSolver.cpp:359-361); 2nd-order runs treat outlets as walls.
    auto zi = mesh.getBeginItFacesInfList();
    for (int z = 0; z < nZ; ++z)
      if (zi[z].getType() == 5) zi[z].setType(3);
  }

  // ---- mesh dump ----------------------------------------------------------
  {
    int counts[5] = {nN, nC, nF, nI, nZ};
    dump(out, "counts.i32", counts, sizeof counts);
    std::vector<int> zones;
    auto zi = mesh.getBeginItFacesInfList();
    for (int z = 0; z < nZ; ++z) {
      zones.push_back(zi[z].getNumber());
      zones.push_back(zi[z].getStart());
      zones.push_back(zi[z].getEnd());
      zones.push_back(zi[z].getType());
    }
    dump(out, "zones.i32", zones.data(), zones.size() * 4);

    std::vector<double> nodes(2 * (size_t)nN);
    Node* nl = mesh.getBeginItNodesList();
    for (int i = 0; i < nN; ++i) {
      nodes[2 * i] = nl[i].getCenter()(0);
      nodes[2 * i + 1] = nl[i].getCenter()(1);
    }
    dump(out, "nodes.f64", nodes.data(), nodes.size() * 8);

    Face* fl = mesh.getBeginItFacesList();
    std::vector<int> fnodes(2 * (size_t)nF), fcells(2 * (size_t)nF),
        fdac(nF), ftype(nF);
    std::vector<double> fctr(2 * (size_t)nF), fdir(2 * (size_t)nF), farea(nF),
        feta(nF);
    std::vector<unsigned char> fflag(2 * (size_t)nF);
    for (int i = 0; i < nF; ++i) {
      auto nb = fl[i].getBeginItPNbNodes();
      fnodes[2 * i] = nb[0]->getId();
      fnodes[2 * i + 1] = nb[1]->getId();
      auto cb = fl[i].getBeginItPNbCells();
      fcells[2 * i] = cb[0]->getId();
      fcells[2 * i + 1] = fl[i].getNumOfpNbCells() > 1 ? cb[1]->getId() : -1;
      fdac[i] = fl[i].getDirectAndCells();
      ftype[i] = fl[i].getType();
      fctr[2 * i] = fl[i].getCenter()(0);
      fctr[2 * i + 1] = fl[i].getCenter()(1);
      fdir[2 * i] = fl[i].getDirect()(0);
      fdir[2 * i + 1] = fl[i].getDirect()(1);
      farea[i] = fl[i].getArea();
      feta[i] = fl[i].getEta0();
      fflag[2 * i] = fl[i].getFlagLeftRight()[0] ? 1 : 0;
      fflag[2 * i + 1] = fl[i].getFlagLeftRight()[1] ? 1 : 0;
    }
    dump(out, "face_nodes.i32", fnodes.data(), fnodes.size() * 4);
    dump(out, "face_cells.i32", fcells.data(), fcells.size() * 4);
    dump(out, "face_dac.i32", fdac.data(), fdac.size() * 4);
    dump(out, "face_type.i32", ftype.data(), ftype.size() * 4);
    dump(out, "face_center.f64", fctr.data(), fctr.size() * 8);
    dump(out, "face_direct.f64", fdir.data(), fdir.size() * 8);
    dump(out, "face_area.f64", farea.data(), farea.size() * 8);
    dump(out, "face_eta0.f64", feta.data(), feta.size() * 8);
    dump(out, "face_flag.u8", fflag.data(), fflag.size());

    Cell* cl = mesh.getBeginItCellsList();
    std::vector<int> cptr(nC + 1, 0), cfaces, cnb;
    std::vector<double> cctr(2 * (size_t)nC), cvol(nC), cdof, ceta;
    for (int c = 0; c < nC; ++c) {
      int nf = cl[c].getNumOfNbFaces();
      cptr[c + 1] = cptr[c] + nf;
      auto fb = cl[c].getBeginItPNbFaces();
      auto nbc = cl[c].getBeginItPNbCells();
      VCTDIM* dof = cl[c].getBeginItDirectOfNbFaces();
      NUM* e0 = cl[c].getBeginItEta0C();
      for (int k = 0; k < nf; ++k) {
        cfaces.push_back(fb[k]->getId());
        cnb.push_back(k < cl[c].getNumOfNbCells() ? nbc[k]->getId() : -1);
        cdof.push_back(dof[k](0));
        cdof.push_back(dof[k](1));
        ceta.push_back(e0[k]);
      }
      cctr[2 * c] = cl[c].getCenter()(0);
      cctr[2 * c + 1] = cl[c].getCenter()(1);
      cvol[c] = cl[c].getVolume();
    }
    dump(out, "cell_ptr.i32", cptr.data(), cptr.size() * 4);
    dump(out, "cell_faces.i32", cfaces.data(), cfaces.size() * 4);
    dump(out, "cell_nbcells.i32", cnb.data(), cnb.size() * 4);
    dump(out, "cell_dof.f64", cdof.data(), cdof.size() * 8);
    dump(out, "cell_eta0c.f64", ceta.data(), ceta.size() * 8);
    dump(out, "cell_center.f64", cctr.data(), cctr.size() * 8);
    dump(out, "cell_volume.f64", cvol.data(), cvol.size() * 8);

    int nb1 = mesh.getNumOfBond1Cells(), nb2 = mesh.getNumOfBond2Cells(),
        nin = mesh.getNumOfInnerCells();
    int bcounts[3] = {nin, nb1, nb2};
    dump(out, "bond_counts.i32", bcounts, sizeof bcounts);
    dump(out, "inner.i32", mesh.getBeginItInnerIdList(), (size_t)nin * 4);
    dump(out, "bond1.i32", mesh.getBeginItBond1IdList(), (size_t)nb1 * 4);
    dump(out, "bond2.i32", mesh.getBeginItBond2IdList(), (size_t)nb2 * 4);
  }

  // ---- state ----------------------------------------------------------------
  AllData data;
  data.createAllData(nC, nF);
  std::fstream flog;
  std::string logpath = out + "/time.log";
  flog.open(logpath, std::ios::out | std::ios::trunc);
  Time timeLoop(&mesh, &flog, &data);
  VCTDIMU iniQ;
  iniQ << inirho, inirho * iniu, inirho * iniv, iniE;
  timeLoop.initialization(iniQ);
  if (!q0file.empty()) {
    std::vector<double> q(4 * (size_t)nC);
    FILE* f = std::fopen(q0file.c_str(), "rb");
    if (!f || std::fread(q.data(), 8, q.size(), f) != q.size()) {
      std::fprintf(stderr, "bad q0 file %s\n", q0file.c_str());
      return 2;
    }
    std::fclose(f);
    for (int c = 0; c < nC; ++c)
      for (int m = 0; m < 4; ++m) {
        data.getP1OldCellQs()[c](m) = q[4 * c + m];
        data.getP1NewCellQs()[c](m) = q[4 * c + m];
        data.getPtP1OldNTimeCellQs()[c](m) = q[4 * c + m];
      }
  }
  {
    std::vector<double> q(4 * (size_t)nC);
    for (int c = 0; c < nC; ++c)
      for (int m = 0; m < 4; ++m) q[4 * c + m] = data.getP1OldCellQs()[c](m);
    dump(out, "q0.f64", q.data(), q.size() * 8);
  }

  if (bench > 0) {
    // Time solve() + updateNewToOld() per step, as the CPU baseline.
    RhoSolver warm(&mesh, &flog, &data);
    warm.setDT(dt);
    warm.solve();
    warm.updateNewToOld();
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < bench; ++s) {
      RhoSolver solver(&mesh, &flog, &data);
      solver.setDT(dt);
      solver.solve();
      solver.updateNewToOld();
    }
    auto t1 = std::chrono::steady_clock::now();
    double sec = std::chrono::duration<double>(t1 - t0).count();
    std::printf("BENCH cells=%d steps=%d seconds=%.6f mcups=%.6f threads=%d\n",
                nC, bench, sec, (double)nC * bench / sec / 1e6,
                (int)NUM_CPU_THREADS);
    return 0;
  }

  if (time_steps > 0) {
    for (int s = 0; s < time_steps; ++s) timeLoop.goNextTimeStep();
    std::vector<double> q(4 * (size_t)nC);
    for (int c = 0; c < nC; ++c)
      for (int m = 0; m < 4; ++m) q[4 * c + m] = data.getP1OldCellQs()[c](m);
    dump(out, "q_steps.f64", q.data(), q.size() * 8);
    flog.close();
    return 0;
  }

  // ---- one residual evaluation ---------------------------------------------
  RhoSolver solver(&mesh, &flog, &data);
  solver.setDT(dt);
  solver.solve();
  {
    MTDIMU_DIM* F = data.getP1OldFaceConvectFlux();
    std::vector<double> fl(8 * (size_t)nF);
    for (int i = 0; i < nF; ++i)
      for (int d = 0; d < 2; ++d)
        for (int m = 0; m < 4; ++m) fl[8 * i + 4 * d + m] = F[i](m, d);
    dump(out, "flux.f64", fl.data(), fl.size() * 8);

    // R_c = sum over the cell's faces (stored order) and axes of
    // n_{c,k,d} * F_f(:,d), accumulated in that order from zero.
    Cell* cl = mesh.getBeginItCellsList();
    std::vector<double> R(4 * (size_t)nC);
    for (int c = 0; c < nC; ++c) {
      double r[4] = {0, 0, 0, 0};
      VCTDIM* dof = cl[c].getBeginItDirectOfNbFaces();
      auto fb = cl[c].getBeginItPNbFaces();
      for (int k = 0; k < cl[c].getNumOfNbFaces(); ++k)
        for (int d = 0; d < 2; ++d) {
          double s = dof[k](d);
          const MTDIMU_DIM& Ff = F[fb[k]->getId()];
          for (int m = 0; m < 4; ++m) r[m] += s * Ff(m, d);
        }
      for (int m = 0; m < 4; ++m) R[4 * c + m] = r[m];
    }
    dump(out, "resid.f64", R.data(), R.size() * 8);

    std::vector<double> qn(4 * (size_t)nC), fq(4 * (size_t)nF);
    for (int c = 0; c < nC; ++c)
      for (int m = 0; m < 4; ++m) qn[4 * c + m] = data.getP1NewCellQs()[c](m);
    dump(out, "qnew.f64", qn.data(), qn.size() * 8);
    for (int i = 0; i < nF; ++i)
      for (int m = 0; m < 4; ++m) fq[4 * i + m] = data.getP1OldFaceQs()[i](m);
    dump(out, "faceq.f64", fq.data(), fq.size() * 8);
  }
  flog.close();
  return 0;
}
