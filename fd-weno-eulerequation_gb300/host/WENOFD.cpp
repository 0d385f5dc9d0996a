#include "WENOFD.hpp"

#include <chrono>
#include <numeric>
#include <cmath>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>

namespace {

void check(int rc, const char *what) {
  if (rc != WENOFD_OK)
    throw std::runtime_error(std::string(what) + ": " + wenofd_last_error() + " (status " + std::to_string(rc) + ")");
}

// getTimestamp of utils/timer.hpp: local time as YYYYmmdd_HHMMSS.
std::string timestamp() {
  const std::time_t t = std::chrono::system_clock::to_time_t(std::chrono::system_clock::now());
  std::ostringstream ss;
  ss << std::put_time(std::localtime(&t), "%Y%m%d_%H%M%S");
  return ss.str();
}

std::string trim(const std::string &s) {
  const size_t first = s.find_first_not_of(' ');
  if (first == std::string::npos) return std::string();
  size_t last = s.find_last_not_of(' ');
  if (s[last] == '\r') {
    if (last == first) return std::string();
    --last;
  }
  return s.substr(first, last - first + 1);
}

}  // namespace

void CConfig::read(std::map<std::string, std::string> &option) {
  std::ifstream input(m_inputFileName);
  if (!input.is_open()) throw std::runtime_error("Failed to open file" + m_inputFileName);
  std::string line;
  while (std::getline(input, line)) {
    if (line.empty() || line[0] == '#' || line[0] == '\r') continue;
    const size_t eq = line.find('=');
    if (eq == std::string::npos) {
      std::cerr << "Invalid line: " << line << std::endl;
      continue;
    }
    option[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
  }
}

CWENOFD::~CWENOFD() {
  if (m_handle) wenofd_destroy(m_handle);
}

double CWENOFD::nodeX(int ei) const { return (equation->xL + 0 * m_deltaX - m_deltaX * m_ghostCellNum) + ei * m_deltaX; }
double CWENOFD::nodeY(int ej) const { return (equation->yL - m_deltaY * m_ghostCellNum) + ej * m_deltaY; }

// initializeSolver, src/WENOFD.cpp:10-164 (single process, whole domain).
void CWENOFD::initializeSolver(std::map<std::string, std::string> option) {
  if (!equation) throw std::runtime_error("CWENOFD needs an EulerEquation");
  m_option = option;
  m_testcase = TESTCASETYPE(std::stoi(option["TESTCASE"]));
  m_rkMeth = RKMETHOD(std::stoi(option["RKMETH"]));
  const std::uint64_t seed = option.count("SEED") ? std::stoull(option["SEED"]) : 0;
  equation->setEquationParameters(m_testcase, seed);
  m_outputTime = equation->outputtime;
  m_scheme = SCHEMETYPE(std::stoi(option["SCHEME"]));
  m_cfl = std::stod(option["CFL"]);
  m_precision = option.count("PRECISION") ? std::stoi(option["PRECISION"]) : 0;
  m_ghostCellNum = 4;
  m_worldPointNumX = std::stoi(option["ELEMNUMX"]);
  m_worldPointNumY = std::stoi(option["ELEMNUMY"]);
  m_startPointX = m_startPointY = m_ghostCellNum;
  m_endPointX = m_startPointX + m_worldPointNumX;
  m_endPointY = m_startPointY + m_worldPointNumY;
  m_totalPointNumX = m_worldPointNumX + 2 * m_ghostCellNum;
  m_totalPointNumY = m_worldPointNumY + 2 * m_ghostCellNum;
  m_deltaX = (equation->xR - equation->xL) / (m_worldPointNumX - 1);
  m_deltaY = (equation->yR - equation->yL) / (m_worldPointNumY - 1);
  m_outputDir = "./output/" + timestamp() + "_" + TESTCASETYPE_STRINGS[m_testcase] + "_" +
                SCHEMETYPE_STRINGS[m_scheme] + "_" + std::to_string(m_worldPointNumX) + "x" +
                std::to_string(m_worldPointNumY) + "/";
  std::filesystem::create_directories(m_outputDir);
  m_Uh.assign(size_t(4) * m_worldPointNumX * m_worldPointNumY, 0.0);
  m_rhs.assign(m_Uh.size(), 0.0);
  if (m_handle) {
    wenofd_destroy(m_handle);
    m_handle = nullptr;
  }
  m_now = 0;
  m_steps = 0;
}

// The device solver is created from the options and the equation object as
// it stands at first use, so changes a caller makes to the equation after
// initializeSolver (domain, gamma, boundary types, end time) are honoured.
void CWENOFD::ensureHandle() {
  if (m_handle) return;
  std::map<std::string, std::string> kv = m_option;
  auto num = [](double v) {
    std::ostringstream ss;
    ss << std::setprecision(17) << v;
    return ss.str();
  };
  kv["TEND"] = num(m_outputTime);
  kv["XL"] = num(equation->xL);
  kv["XR"] = num(equation->xR);
  kv["YL"] = num(equation->yL);
  kv["YR"] = num(equation->yR);
  kv["GAMMA"] = num(equation->euler_gamma);
  kv["BC_LEFT"] = std::to_string(int(equation->leftBoundaryCondition));
  kv["BC_RIGHT"] = std::to_string(int(equation->rightBoundaryCondition));
  kv["BC_BOTTOM"] = std::to_string(int(equation->bottomBoundaryCondition));
  kv["BC_TOP"] = std::to_string(int(equation->topBoundaryCondition));
  kv["GRAVITY"] = equation->gravity ? "1" : "0";
  std::vector<const char *> keys, vals;
  for (const auto &p : kv) {
    keys.push_back(p.first.c_str());
    vals.push_back(p.second.c_str());
  }
  check(wenofd_create(keys.data(), vals.data(), int(keys.size()), &m_handle), "wenofd_create");
  wenofd_info info;
  check(wenofd_get_info(m_handle, &info), "wenofd_get_info");
  m_deltaX = info.dx;
  m_deltaY = info.dy;
  const bool special = equation->leftBoundaryCondition == SPECIAL || equation->rightBoundaryCondition == SPECIAL ||
                       equation->bottomBoundaryCondition == SPECIAL;
  if (special) {  // getU0 at the fixed boundary nodes (src/WENOFD.cpp:1045-1058, 1092-1102, 1138-1149)
    const int nxt = m_totalPointNumX, nyt = m_totalPointNumY;
    std::vector<double> tab(8 * size_t(nxt) + 8 * size_t(nyt));
    double q[4];
    for (int ei = 0; ei < nxt; ++ei) {
      equation->getU0(nodeX(ei), nodeY(m_startPointY), q);
      for (int r = 0; r < 4; ++r) tab[r * nxt + ei] = q[r];
      equation->getU0(nodeX(ei), nodeY(m_endPointY - 1), q);
      for (int r = 0; r < 4; ++r) tab[4 * nxt + r * nxt + ei] = q[r];
    }
    for (int ej = 0; ej < nyt; ++ej) {
      equation->getU0(nodeX(m_startPointX), nodeY(ej), q);
      for (int r = 0; r < 4; ++r) tab[8 * nxt + r * nyt + ej] = q[r];
      equation->getU0(nodeX(m_endPointX), nodeY(ej), q);
      for (int r = 0; r < 4; ++r) tab[8 * nxt + 4 * nyt + r * nyt + ej] = q[r];
    }
    check(wenofd_set_boundary_values(m_handle, tab.data()), "wenofd_set_boundary_values");
  }
}

// initializeAve, src/WENOFD.cpp:165-188: getU0 at every interior node.
void CWENOFD::initializeAve() {
  ensureHandle();
  if (equation->library_initial_state) {
    check(wenofd_initialize(m_handle), "wenofd_initialize");
    downloadState();
  } else {
    const size_t plane = size_t(m_worldPointNumX) * m_worldPointNumY;
    double q[4];
    for (int i = 0; i < m_worldPointNumX; ++i)
      for (int j = 0; j < m_worldPointNumY; ++j) {
        equation->getU0(nodeX(i + m_ghostCellNum), nodeY(j + m_ghostCellNum), q);
        for (int r = 0; r < 4; ++r) m_Uh[r * plane + size_t(i) * m_worldPointNumY + j] = q[r];
      }
    uploadState();
  }
  check(wenofd_set_time(m_handle, m_now), "wenofd_set_time");
}

void CWENOFD::downloadState() {
  ensureHandle();
  check(wenofd_get_state(m_handle, m_Uh.data()), "wenofd_get_state");
}

void CWENOFD::uploadState() {
  ensureHandle();
  check(wenofd_set_state(m_handle, m_Uh.data()), "wenofd_set_state");
}

void CWENOFD::assembleRHS() {
  ensureHandle();
  check(wenofd_get_flux(m_handle, m_rhs.data()), "wenofd_get_flux");
}

std::vector<double> &CWENOFD::getFlux() {
  assembleRHS();
  return m_rhs;
}

void CWENOFD::setBoundary() {
  ensureHandle();
  check(wenofd_fill_boundary(m_handle), "wenofd_fill_boundary");
}

double CWENOFD::calculateDeltaT() {
  ensureHandle();
  check(wenofd_set_time(m_handle, m_now), "wenofd_set_time");
  double dt = 0;
  check(wenofd_calc_dt(m_handle, &dt), "calculateDeltaT");
  return dt;
}

void CWENOFD::stepWith(RKMETHOD m, double dt) {
  if (m != m_rkMeth) throw std::runtime_error("Error: Invalid Runge-Kutta method for this solver's RKMETH");
  ensureHandle();
  check(wenofd_rk_step(m_handle, dt), "RunRK");
}

void CWENOFD::RunRK1(double deltaT) { stepWith(RK1, deltaT); }
void CWENOFD::RunRK2(double deltaT) { stepWith(RK2, deltaT); }
void CWENOFD::RunRK3(double deltaT) { stepWith(RK3, deltaT); }

// run, src/WENOFD.cpp:189-299, with the time loop on the device.
void CWENOFD::run(std::map<std::string, std::string> option) {
  const auto t0 = std::chrono::steady_clock::now();
  initializeSolver(option);
  m_now = 0;
  initializeAve();
  outputAve("initial");
  std::cout << "Start iteration..." << std::endl;
  const auto t1 = std::chrono::steady_clock::now();
  // The device time loop runs in chunks so that the reference's progress line
  // (src/WENOFD.cpp:243-273: after steps 1, 21, 41, ...) can be printed: the
  // first step alone, then chunks of a multiple of 20 steps that is also a
  // multiple of the steps per graph replay (full replays only).
  long long steps = 0;
  wenofd_info info;
  for (long long chunk = 1;;) {
    long long k = 0;
    check(wenofd_advance(m_handle, chunk, &k), "run");
    steps += k;
    check(wenofd_get_info(m_handle, &info), "wenofd_get_info");
    if (k > 0 && steps % 20 == 1) progressLine(steps, info.dt, info.now, t1);
    if (k < chunk) break;
    const long long K = info.graph_steps > 0 ? info.graph_steps : 1;
    chunk = std::lcm(20LL, K);
  }
  const auto t2 = std::chrono::steady_clock::now();
  m_now = info.now;
  m_steps = info.steps;
  downloadState();
  outputAve("final");
  if (equation->u_exact_exist) {
    outputAccuracy("final");
    outputError("final");
  }
  const double loop_s = std::chrono::duration<double>(t2 - t1).count();
  std::cout << "steps " << steps << ", t = " << m_now << ", loop " << loop_s << " s, "
            << double(m_worldPointNumX) * m_worldPointNumY * steps / loop_s << " cell-updates/s, total "
            << std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() << " s" << std::endl;
}

// The progress line of src/WENOFD.cpp:247-272 (iteration count, deltaT,
// elapsed time, progress with a 50-character bar).
void CWENOFD::progressLine(long long count, double deltaT, double now,
                           std::chrono::steady_clock::time_point start) const {
  const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  const double progress = now / m_outputTime;
  const int barWidth = 50;
  const int pos = static_cast<int>(progress * barWidth);
  std::cout << std::fixed << std::setprecision(2) << "Iteration count: " << count << std::scientific
            << std::setprecision(2) << ", DeltaT: " << deltaT << std::fixed << std::setprecision(2)
            << ", Elapsed time: " << elapsed << " seconds"
            << ", Progress: " << now << "/" << m_outputTime << " (" << (progress * 100.0) << "%)"
            << " [";
  for (int i = 0; i < barWidth; ++i) std::cout << (i < pos ? "=" : (i == pos ? ">" : " "));
  std::cout << "]" << std::endl;
  std::cout.unsetf(std::ios::floatfield);
  std::cout << std::setprecision(6);
}

// outputAve, src/WENOFD.cpp:1161-1238: Tecplot ASCII, point data packing.
// The variables (getVitalVarVal) come from the device
// (wenofd_output_variables); the text is formatted here.
void CWENOFD::outputAve(std::string prefix) {
  const size_t plane = size_t(m_worldPointNumX) * m_worldPointNumY;
  std::vector<double> vars(6 * plane);
  check(wenofd_output_variables(m_handle, vars.data()), "wenofd_output_variables");
  std::string names[6];
  equation->getVitalVarName(names);
  std::ostringstream out;
  out << "TITLE=DGSolution\n"
      << "VARIABLES=X Y ";
  for (int k = 0; k < 6; ++k) out << names[k] << " ";
  out << "\nZONE T=TA, I=" << m_worldPointNumY << ", J=" << m_worldPointNumX << ", DATAPACKING=POINT\n";
  for (int i = 0; i < m_worldPointNumX; ++i)
    for (int j = 0; j < m_worldPointNumY; ++j) {
      out << nodeX(i + m_ghostCellNum) << " " << nodeY(j + m_ghostCellNum) << " ";
      for (int k = 0; k < 6; ++k) out << vars[k * plane + size_t(i) * m_worldPointNumY + j] << " ";
      out << "\n";
    }
  const std::string filename = m_outputDir + "solution_" + prefix + ".plt";
  std::ofstream f(filename, std::ios::binary);
  f << out.str();
  std::cout << "The file " << filename << " has been output successfully..." << std::endl;
}

// outputError, src/WENOFD.cpp:1239-1306.
void CWENOFD::outputError(std::string prefix) {
  downloadState();
  const std::string filename = m_outputDir + "error_" + prefix + ".plt";
  std::ofstream f(filename);
  if (!f.is_open()) {
    std::cout << "Unable to open file" << std::endl;
    return;
  }
  f << "TITLE=DGSolution" << std::endl;
  f << "VARIABLES=X Y error" << std::endl;
  f << "ZONE T=TA, I=" << m_worldPointNumY << ", J=" << m_worldPointNumX << ", DATAPACKING = POINT" << std::endl;
  const size_t plane = size_t(m_worldPointNumX) * m_worldPointNumY;
  double q[4];
  for (int i = 0; i < m_worldPointNumX; ++i)
    for (int j = 0; j < m_worldPointNumY; ++j) {
      for (int r = 0; r < 4; ++r) q[r] = m_Uh[r * plane + size_t(i) * m_worldPointNumY + j];
      const double x = (equation->xL - m_ghostCellNum * m_deltaX) + (i + m_ghostCellNum) * m_deltaX;
      const double y = (equation->yL - m_ghostCellNum * m_deltaY) + (j + m_ghostCellNum) * m_deltaY;
      const double uref = equation->theVarExact(x, y, m_now);
      f << x << " " << y << " " << std::fabs(uref - equation->theVarUh(q)) << " " << std::endl;
    }
  std::cout << "The file " + filename + " has been output successfully..." << std::endl;
}

// outputAccuracy, src/WENOFD.cpp:1308-1382: Linf, L1, L2 of density against
// the exact solution, summed in the reference's node order on the host.
void CWENOFD::outputAccuracy(std::string prefix) {
  downloadState();
  const size_t plane = size_t(m_worldPointNumX) * m_worldPointNumY;
  double e1 = 0, e2 = 0, einf = 0, q[4];
  for (int i = 0; i < m_worldPointNumX; ++i)
    for (int j = 0; j < m_worldPointNumY; ++j) {
      for (int r = 0; r < 4; ++r) q[r] = m_Uh[r * plane + size_t(i) * m_worldPointNumY + j];
      const double uref = equation->theVarExact(nodeX(i + m_ghostCellNum), nodeY(j + m_ghostCellNum), m_now);
      const double err = std::fabs(uref - equation->theVarUh(q));
      e1 += err;
      e2 += std::pow(err, 2);
      if (err > einf) einf = err;
    }
  e1 = e1 / m_worldPointNumX / m_worldPointNumY;
  e2 = std::sqrt(e2 / m_worldPointNumX / m_worldPointNumY);
  const std::string filename = m_outputDir + "accuracy_" + prefix + ".csv";
  std::fstream f(filename, std::ios::out);
  f << "elemNum, Linf-norm (rho), L1-norm (rho), L2-norm (rho)" << std::endl;
  f << m_worldPointNumX << ", ";
  f << std::setprecision(15) << std::setw(20) << std::setiosflags(std::ios::scientific) << einf << ", ";
  f << std::setprecision(15) << std::setw(20) << std::setiosflags(std::ios::scientific) << e1 << ", ";
  f << std::setprecision(15) << std::setw(20) << std::setiosflags(std::ios::scientific) << e2;
  std::cout << "Accuracy verification completed..." << std::endl;
}
