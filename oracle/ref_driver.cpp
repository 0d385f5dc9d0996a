// Driver for the reference solver compiled from its own, unmodified sources
// (src/WENOFD.cpp + include/ + utils/ of infinity-07/FD-WENO-EulerEquation)
// against the single-rank MPI shim in mpishim/.  Test infrastructure only: it
// produces the outputs that pin the C restatement (wenofd_oracle.c) and the
// golden fixtures under tests/golden/.
//
// It drives CWENOFD exactly the way CWENOFD::run does (src/WENOFD.cpp:189-299)
// but through the class's public members, so that configurations the
// reference hard-codes can be overridden:
//   * the initial state can be replaced after initializeAve() (--init);
//   * the quadrant states of the Riemann2 case can be replaced (--riemann),
//     keeping its interface at (0.8, 0.8) (utils/equations.hpp:537-592);
//   * the domain can be replaced (--domain), after which m_deltaX/Y and
//     m_grids are recomputed with the formulas of src/WENOFD.cpp:73-106;
//   * boundary types and the end time can be replaced (--bc, --tend).
//
// Usage:  wenofd_ref <config.cfg> <mode> <out-prefix> [options]
// Every mode except fullrun writes <out>.init, the interior initial state.
//   mode rhs      : one assembleRHS(); writes <out>.ghosted (full state with
//                   ghosts after the boundary fill) and <out>.rhs (interior).
//   mode run      : loop calculateDeltaT + RunRK{1,2,3} + m_now += dt
//                   (src/WENOFD.cpp:213-239) until t_end or --steps; writes
//                   <out>.state (interior) and <out>.dts.
//   mode accuracy : as run, then outputAccuracy (src/WENOFD.cpp:1308-1382);
//                   the norms go to <out>.meta.
//   mode fullrun  : CWENOFD::run(option) unchanged, as src/main.cpp does;
//                   the accuracy norms (if any) go to <out>.meta.
// Interior arrays are float64 [4][ELEMNUMX][ELEMNUMY] (ej fastest), the same
// index order as m_Uh[ei][ej].vector[r].
#include <mpi.h>

#include "WENOFD.hpp"  // the reference header, found through -I<reference>/include

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

void write_doubles(const std::string &path, const std::vector<double> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  std::fwrite(v.data(), sizeof(double), v.size(), f);
  std::fclose(f);
}

std::vector<double> read_doubles(const std::string &path, size_t n) {
  std::vector<double> v(n);
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot read " + path);
  if (std::fread(v.data(), sizeof(double), n, f) != n) throw std::runtime_error("short file " + path);
  std::fclose(f);
  return v;
}

std::vector<double> interior(CWENOFD &s, Array2D<Cvector> &a) {
  const int nx = s.m_numPointsX, ny = s.m_numPointsY;
  std::vector<double> v(4 * size_t(nx) * ny);
  for (int r = 0; r < 4; ++r)
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        v[(size_t(r) * nx + i) * ny + j] = a[s.m_startPointX + i][s.m_startPointY + j].vector[r];
  return v;
}

std::vector<double> ghosted(CWENOFD &s, Array2D<Cvector> &a) {
  const int nxt = s.m_totalPointNumX, nyt = s.m_totalPointNumY;
  std::vector<double> v(4 * size_t(nxt) * nyt);
  for (int r = 0; r < 4; ++r)
    for (int i = 0; i < nxt; ++i)
      for (int j = 0; j < nyt; ++j) v[(size_t(r) * nxt + i) * nyt + j] = a[i][j].vector[r];
  return v;
}

// Recompute spacing and node coordinates for an overridden domain with the
// reference's own formulas (src/WENOFD.cpp:73-80, 95-106, 110-121).
void rebuild_grid(CWENOFD &s) {
  EulerEquation *eq = s.equation;
  s.m_deltaX = (eq->xR - eq->xL) / (s.m_worldPointNumX - 1);
  s.m_deltaY = (eq->yR - eq->yL) / (s.m_worldPointNumY - 1);
  const double procXLeft = eq->xL + s.m_startPointX_per_rank[s.m_rank] * s.m_deltaX;
  const double procYLeft = eq->yL;
  const double gx = procXLeft - s.m_deltaX * s.m_ghostCellNum;
  const double gy = procYLeft - s.m_deltaY * s.m_ghostCellNum;
  for (int ei = 0; ei < s.m_totalPointNumX; ++ei)
    for (int ej = 0; ej < s.m_totalPointNumY; ++ej) {
      s.m_grids[ei][ej].m_xCenter = gx + ei * s.m_deltaX;
      s.m_grids[ei][ej].m_yCenter = gy + ej * s.m_deltaY;
    }
  for (int ei = 0; ei < s.m_worldPointNumX + 2 * s.m_ghostCellNum; ++ei)
    for (int ej = 0; ej < s.m_worldPointNumY + 2 * s.m_ghostCellNum; ++ej) {
      s.m_worldGrids[ei][ej].m_xCenter = eq->xL - s.m_ghostCellNum * s.m_deltaX + ei * s.m_deltaX;
      s.m_worldGrids[ei][ej].m_yCenter = eq->yL - s.m_ghostCellNum * s.m_deltaY + ej * s.m_deltaY;
    }
}

void step_once(CWENOFD &s, double dt) {
  switch (s.m_rkMeth) {
    case RK1: s.RunRK1(dt); break;
    case RK2: s.RunRK2(dt); break;
    case RK3: s.RunRK3(dt); break;
    default: throw std::runtime_error("bad RKMETH");
  }
}

bool read_accuracy_csv(const std::string &dir, double out[3]) {
  std::ifstream f(dir + "accuracy_final.csv");
  if (!f.is_open()) return false;
  std::string header, line;
  std::getline(f, header);
  std::getline(f, line);
  for (char &c : line)
    if (c == ',') c = ' ';
  std::istringstream ss(line);
  int n;
  ss >> n >> out[0] >> out[1] >> out[2];  // Linf, L1, L2
  return true;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s <config.cfg> <rhs|run|accuracy|fullrun> <out-prefix> [options]\n", argv[0]);
    return 2;
  }
  const std::string cfg = argv[1], mode = argv[2], out = argv[3];
  std::string init_file;
  bool have_domain = false, have_riemann = false, have_bc = false, have_tend = false;
  double dom[4] = {0, 0, 0, 0}, tend = 0, quad[16];
  int bc[4] = {0, 0, 0, 0};
  long max_steps = -1;
  for (int a = 4; a < argc; ++a) {
    const std::string k = argv[a];
    auto need = [&](int n) {
      if (a + n >= argc) throw std::runtime_error("missing value for " + k);
    };
    if (k == "--init") { need(1); init_file = argv[++a]; }
    else if (k == "--steps") { need(1); max_steps = std::atol(argv[++a]); }
    else if (k == "--tend") { need(1); tend = std::atof(argv[++a]); have_tend = true; }
    else if (k == "--domain") { need(4); for (double &d : dom) d = std::atof(argv[++a]); have_domain = true; }
    else if (k == "--bc") { need(4); for (int &b : bc) b = std::atoi(argv[++a]); have_bc = true; }
    else if (k == "--riemann") { need(16); for (double &q : quad) q = std::atof(argv[++a]); have_riemann = true; }
    else throw std::runtime_error("unknown option " + k);
  }

  int rc = 0;
  try {
    MPI_Init(&argc, &argv);
    EulerEquation *equation = new EulerEquation();
    CConfig config(cfg);
    std::map<std::string, std::string> option;
    config.read(option);
    CWENOFD solver(equation);

    if (mode == "fullrun") {
      solver.run(option);
      double norms[3] = {0, 0, 0};
      const bool have = read_accuracy_csv(solver.m_outputDir, norms);
      std::ofstream meta(out + ".meta");
      meta.precision(17);
      meta << "now=" << solver.m_now << "\n";
      if (have) meta << "linf=" << norms[0] << "\nl1=" << norms[1] << "\nl2=" << norms[2] << "\n";
      write_doubles(out + ".state", interior(solver, solver.m_Uh));
      MPI_Finalize();
      return 0;
    }

    solver.initializeSolver(option);
    if (have_domain) {
      equation->xL = dom[0]; equation->xR = dom[1];
      equation->yL = dom[2]; equation->yR = dom[3];
      rebuild_grid(solver);
    }
    if (have_bc) {
      equation->leftBoundaryCondition = BOUNDARYTYPE(bc[0]);
      equation->rightBoundaryCondition = BOUNDARYTYPE(bc[1]);
      equation->bottomBoundaryCondition = BOUNDARYTYPE(bc[2]);
      equation->topBoundaryCondition = BOUNDARYTYPE(bc[3]);
    }
    if (have_tend) solver.m_outputTime = tend;
    if (have_riemann) {
      // Same quadrant tests as the Riemann2 lambdas (utils/equations.hpp:537-592),
      // values replaced: quad = {rho,u,v,p} for (x<.8,y<.8), (x<.8,y>=.8),
      // (x>=.8,y<.8), (x>=.8,y>=.8).
      std::vector<double> q(quad, quad + 16);
      auto pick = [q](int var) {
        return [q, var](const double x, const double y) {
          int k = (x < 0.8) ? (y < 0.8 ? 0 : 1) : (y < 0.8 ? 2 : 3);
          return q[4 * k + var];
        };
      };
      equation->rho0 = pick(0);
      equation->u0 = pick(1);
      equation->v0 = pick(2);
      equation->pre0 = pick(3);
    }

    solver.m_now = 0;
    solver.m_solverTimer.start();
    solver.initializeAve();
    if (!init_file.empty()) {
      const int nx = solver.m_numPointsX, ny = solver.m_numPointsY;
      std::vector<double> v = read_doubles(init_file, 4 * size_t(nx) * ny);
      for (int r = 0; r < 4; ++r)
        for (int i = 0; i < nx; ++i)
          for (int j = 0; j < ny; ++j)
            solver.m_Uh[solver.m_startPointX + i][solver.m_startPointY + j].vector[r] =
                v[(size_t(r) * nx + i) * ny + j];
    }
    solver.m_mainTimer.start();
    write_doubles(out + ".init", interior(solver, solver.m_Uh));

    std::ofstream meta(out + ".meta");
    meta.precision(17);
    meta << "dx=" << solver.m_deltaX << "\ndy=" << solver.m_deltaY << "\n";

    if (mode == "rhs") {
      solver.assembleRHS();
      write_doubles(out + ".ghosted", ghosted(solver, solver.m_Uh));
      write_doubles(out + ".rhs", interior(solver, solver.m_rhs));
      const double dt = solver.calculateDeltaT();
      meta << "dt=" << dt << "\n";
    } else if (mode == "run" || mode == "accuracy") {
      std::vector<double> dts;
      long count = 0;
      while (std::fabs(solver.m_now - solver.m_outputTime) > 1e-9) {
        if (max_steps >= 0 && count >= max_steps) break;
        const double dt = solver.calculateDeltaT();
        step_once(solver, dt);
        solver.m_now += dt;
        ++count;
        dts.push_back(dt);
      }
      meta << "steps=" << count << "\nnow=" << solver.m_now << "\n";
      write_doubles(out + ".state", interior(solver, solver.m_Uh));
      write_doubles(out + ".dts", dts);
      if (mode == "accuracy") {
        solver.outputAccuracy("final");
        double norms[3] = {0, 0, 0};
        if (read_accuracy_csv(solver.m_outputDir, norms))
          meta << "linf=" << norms[0] << "\nl1=" << norms[1] << "\nl2=" << norms[2] << "\n";
      }
    } else {
      throw std::runtime_error("unknown mode " + mode);
    }
    MPI_Finalize();
  } catch (const std::exception &e) {
    std::fprintf(stderr, "wenofd_ref: %s\n", e.what());
    rc = 1;
  }
  return rc;
}
