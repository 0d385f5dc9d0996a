// Drop-in host class with the public interface of the reference's CWENOFD
// (include/WENOFD.hpp:28-124), running the per-step hot path on one GB300
// through the C ABI (include/wenofd.h).  Method names, config keys, output
// files and their formats follow the reference; the state lives on the GPU
// and m_Uh / m_rhs are host copies refreshed on demand.
//
// Differences from the reference, by design:
//  - one process drives one GPU holding the whole domain: no MPI ranks, slab
//    decomposition or halo exchange (the ghost fill runs on the device);
//  - the time loop in run() is device resident (wenofd_advance);
//  - RunRK1/2/3 must match RKMETH (the device solver is built for one method);
//  - errors throw std::runtime_error instead of calling MPI_Abort / exit;
//  - getFlux() is the README's name for the RHS assembly (assembleBoundaryTerm
//    plus the source term), kept beside assembleRHS();
//  - the output directory is created but the source tree is not copied into
//    it (backupProjectFiles).
#pragma once

#include <chrono>
#include <map>
#include <string>
#include <vector>

#include "EulerEquation.hpp"
#include "wenofd.h"

enum RKMETHOD { RK1 = 0, RK2 = 1, RK3 = 2 };

// CConfig (utils/readConfig.hpp:30-104): `key = value` lines, '#' comments.
class CConfig {
 public:
  explicit CConfig(const std::string &file) : m_inputFileName(file) {}
  // Throws std::runtime_error if the file cannot be opened (the reference exits).
  void read(std::map<std::string, std::string> &option);
  std::string m_inputFileName;
};

class CWENOFD {
 public:
  CWENOFD() {}
  explicit CWENOFD(EulerEquation *equation) : equation(equation) {}
  ~CWENOFD();
  CWENOFD(const CWENOFD &) = delete;
  CWENOFD &operator=(const CWENOFD &) = delete;

  EulerEquation *equation = nullptr;
  int m_varNum = 4;

  int m_worldPointNumX = 0, m_worldPointNumY = 0;
  int m_ghostCellNum = 4;
  int m_startPointX = 4, m_endPointX = 4, m_startPointY = 4, m_endPointY = 4;
  int m_totalPointNumX = 0, m_totalPointNumY = 0;
  double m_deltaX = 0, m_deltaY = 0;
  double m_outputTime = 0, m_now = 0, m_cfl = 0;
  TESTCASETYPE m_testcase = SMOOTH;
  SCHEMETYPE m_scheme = WENOZ;
  RKMETHOD m_rkMeth = RK3;
  int m_precision = 0;  // 0 FP64 (bitwise the reference), 1 FP32 flux arithmetic
  std::string m_outputDir;
  long long m_steps = 0;

  // Interior state and RHS, float64 [4][ELEMNUMX][ELEMNUMY] (ej fastest):
  // element (r, i, j) is the reference's m_Uh[i+4][j+4].vector[r].
  std::vector<double> m_Uh, m_rhs;

  void run(std::map<std::string, std::string> option);
  void initializeSolver(std::map<std::string, std::string> option);
  void initializeAve();
  void assembleRHS();
  std::vector<double> &getFlux();
  double calculateDeltaT();
  void setBoundary();
  void RunRK1(double deltaT);
  void RunRK2(double deltaT);
  void RunRK3(double deltaT);
  void outputAve(std::string prefix);
  void outputError(std::string prefix);
  void outputAccuracy(std::string prefix);

  // node coordinates (m_grids[ei][ej] of the reference; ei, ej include ghosts)
  double nodeX(int ei) const;
  double nodeY(int ej) const;
  // refresh m_Uh from the device / push m_Uh to the device
  void downloadState();
  void uploadState();
  wenofd_solver *handle() { return m_handle; }

 private:
  void ensureHandle();
  void stepWith(RKMETHOD m, double dt);
  void progressLine(long long count, double deltaT, double now, std::chrono::steady_clock::time_point start) const;
  std::map<std::string, std::string> m_option;
  wenofd_solver *m_handle = nullptr;
};
