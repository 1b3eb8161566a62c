// Oracle harness around the reference's sparse LU-SGS / Gauss-Seidel sweeps
// (test infrastructure only; built into oracle/_ref by build_ref.sh).
//
// Drives lusolver/SparseSolverNUM.cpp (scalar: setELE/addELE :115-140,
// solveILUSGS :144-212, solveGS :214-252) and the block template
// lusolver/SparseSolver.cpp (setD/setL/setU :35-48, solveILU :53-104) on a
// matrix given as an ordered list of insertions, so the duplicate-keeping,
// insertion-ordered column lists of the reference are reproduced exactly.
//
// input (binary, little endian):
//   int32 mode (0 scalar ILU-SGS, 1 scalar GS, 2 block 4x4 ILU), int32 dim,
//   int32 n;  int32 rows[n]; int32 cols[n]; int32 ops[n] (0 set, 1 add);
//   f64 vals[n * B]; f64 b[dim * b]; f64 x0[dim * b]
//   where B = 1 (scalar) or 16 (block, row-major 4x4) and b = 1 or 4.
// output: f64 x[dim * b]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lusolver/sparseSolverNUM.h"
#include "lusolver/sparseSolver.h"
#include "lusolver/sparseSolver.cpp"

template <typename T>
static void rd(FILE* f, T* p, size_t n) {
  if (n && std::fread(p, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "ref_lu: short input\n");
    std::exit(2);
  }
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
    return 1;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[3];
  rd(f, hdr, 3);
  int mode = hdr[0], dim = hdr[1], n = hdr[2];
  std::vector<int> rows(n), cols(n), ops(n);
  rd(f, rows.data(), n);
  rd(f, cols.data(), n);
  rd(f, ops.data(), n);
  const int B = (mode == 2) ? 16 : 1, b = (mode == 2) ? 4 : 1;
  std::vector<double> vals((size_t)n * B), rhs((size_t)dim * b),
      x0((size_t)dim * b);
  rd(f, vals.data(), vals.size());
  rd(f, rhs.data(), rhs.size());
  rd(f, x0.data(), x0.size());
  std::fclose(f);

  std::vector<double> x((size_t)dim * b);
  if (mode == 0 || mode == 1) {
    SparseSolverNUM s(dim, x0.data());
    for (int i = 0; i < n; ++i) {
      if (ops[i] == 1) s.addELE(vals[i], rows[i], cols[i]);
      else s.setELE(vals[i], rows[i], cols[i]);
    }
    for (int i = 0; i < dim; ++i) s.setRHSb(rhs[i], i);
    if (mode == 0) s.solveILUSGS();
    else s.solveGS();
    double* px = s.getPNewX();
    for (int i = 0; i < dim; ++i) x[i] = px[i];
  } else {
    typedef Eigen::Matrix<double, 4, 4> M4;
    typedef Eigen::Matrix<double, 4, 1> V4;
    std::vector<V4> px0(dim);
    for (int i = 0; i < dim; ++i)
      for (int k = 0; k < 4; ++k) px0[i](k) = x0[4 * i + k];
    SparseSolver<M4, V4> s(dim, px0.data());
    for (int i = 0; i < n; ++i) {
      M4 m;
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m(r, c) = vals[(size_t)16 * i + 4 * r + c];
      if (rows[i] == cols[i]) s.setD(m, rows[i]);
      else if (rows[i] > cols[i]) s.setL(m, rows[i], cols[i]);
      else s.setU(m, rows[i], cols[i]);
    }
    for (int i = 0; i < dim; ++i) {
      V4 v;
      for (int k = 0; k < 4; ++k) v(k) = rhs[4 * i + k];
      s.setRHSb(v, i);
    }
    s.solveILU();
    V4* px = s.getItBeginX();
    for (int i = 0; i < dim; ++i)
      for (int k = 0; k < 4; ++k) x[4 * i + k] = px[i](k);
  }
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  std::fwrite(x.data(), 8, x.size(), o);
  std::fclose(o);
  return 0;
}
