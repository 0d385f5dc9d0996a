// Host-side physics object with the public interface of the reference's
// EulerEquation (utils/equations.hpp:55-699): domain, end time, boundary
// types, gamma, initial-condition lambdas, exact solution, output variables.
// The flux, eigenvector and splitting functions of the reference run on the
// GPU (csrc/physics.cuh); this class only carries the parameters and the
// initial condition that CWENOFD evaluates on the host, as the reference does.
//
// Differences from the reference, by design: state vectors are plain
// double[4] instead of Array1D<double>; two seeded test cases are added
// (RiemannSeeded = 4, ShearLayer = 5).
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>

enum SCHEMETYPE { WENOJS = 0, WENOZ = 1, WENOZP = 2, WENOZPI = 3 };
inline const std::string SCHEMETYPE_STRINGS[] = {"WENOJS", "WENOZ", "WENOZP", "WENOZPI"};

enum TESTCASETYPE { SMOOTH = 0, Riemann1 = 1, Riemann2 = 2, RTI = 3, RiemannSeeded = 4, ShearLayer = 5 };
inline const std::string TESTCASETYPE_STRINGS[] = {"SMOOTH", "Riemann1", "Riemann2", "RTI", "RiemannSeeded",
                                                   "ShearLayer"};

enum BOUNDARYTYPE { PERIOD = 0, SLIP = 1, SPECIAL = 2, SYMMETRIC = 3 };

class EulerEquation {
 public:
  double xL = 0, xR = 1, yL = 0, yR = 1;
  double outputtime = 1;
  BOUNDARYTYPE leftBoundaryCondition = PERIOD, rightBoundaryCondition = PERIOD;
  BOUNDARYTYPE topBoundaryCondition = PERIOD, bottomBoundaryCondition = PERIOD;
  std::function<double(const double, const double, const double)> theVarExact;
  std::function<double(const double *)> theVarUh;
  bool u_exact_exist = false;
  double euler_gamma = 1.4;
  bool gravity = false;  // RTI source term (the reference switches it on TESTCASE in assembleSourceTerm)
  // The shear layer's seeded noise depends on the node index, so its initial
  // state is generated by the library (wenofd_initialize), not by getU0.
  bool library_initial_state = false;
  std::uint64_t seed = 0;

  std::function<double(const double, const double)> u0, v0, pre0, rho0;

  int getVarNum() const { return 4; }

  // setEquationParameters (utils/equations.hpp:400-646) plus the seeded cases.
  void setEquationParameters(TESTCASETYPE type, std::uint64_t seed_value = 0) {
    seed = seed_value;
    gravity = false;
    library_initial_state = false;
    euler_gamma = 1.4;
    u_exact_exist = false;
    theVarUh = [](const double *U) { return U[0]; };
    theVarExact = [](const double, const double, const double) { return 0.0; };
    switch (type) {
      case SMOOTH:
        setDomain(0.0, 2.0, 0.0, 2.0, 1.0, PERIOD, PERIOD, PERIOD, PERIOD);
        rho0 = [](const double x, const double y) { return 1 + 0.2 * std::sin(M_PI * (x + y)); };
        u0 = [](const double, const double) { return 0.7; };
        v0 = [](const double, const double) { return 0.3; };
        pre0 = [](const double, const double) { return 1.0; };
        u_exact_exist = true;
        theVarExact = [](const double x, const double y, const double t) {
          return 1 + 0.2 * std::sin(M_PI * (x + y - t));
        };
        break;
      case Riemann1:
        setDomain(0.0, 2.0, 0.0, 2.0, 0.52, SYMMETRIC, SYMMETRIC, SYMMETRIC, SYMMETRIC);
        setQuadrants(1.0, {0.8, 0.0, 0.0, 1.0, 1.0, 0.7276, 0.0, 1.0, 1.0, 0.0, 0.7276, 1.0, 0.5313, 0.0, 0.0, 0.4});
        break;
      case Riemann2:
        setDomain(0.0, 1.0, 0.0, 1.0, 0.8, SYMMETRIC, SYMMETRIC, SYMMETRIC, SYMMETRIC);
        setQuadrants(0.8, {0.138, 1.206, 1.206, 0.029, 0.5323, 1.206, 0.0, 0.3, 0.5323, 0.0, 1.206, 0.3, 1.5,
                           0.0, 0.0, 1.5});
        break;
      case RTI:
        setDomain(0.0, 0.25, 0.0, 1.0, 1.95, SLIP, SLIP, SPECIAL, SPECIAL);
        euler_gamma = 5.0 / 3.0;
        gravity = true;
        rho0 = [](const double, const double y) { return y <= 0.5 ? 2.0 : 1.0; };
        u0 = [](const double, const double) { return 0.0; };
        pre0 = [](const double, const double y) { return y <= 0.5 ? 1 + 2 * y : y + 1.5; };
        v0 = [this](const double x, const double y) {
          const double c = std::sqrt(euler_gamma * pre0(x, y) / rho0(x, y));
          return -0.025 * c * std::cos(8 * M_PI * x);
        };
        break;
      case RiemannSeeded: {
        // four quadrants drawn from the seed: rho in [0.1,1.5], u,v in
        // [-1.2,1.2], p in [0.03,1.5]; interface (0.8, 0.8)
        setDomain(0.0, 1.0, 0.0, 1.0, 0.3, SYMMETRIC, SYMMETRIC, SYMMETRIC, SYMMETRIC);
        std::uint64_t s = seed_value;
        std::array<double, 16> q;
        for (int k = 0; k < 4; ++k) {
          q[4 * k + 0] = 0.1 + (1.5 - 0.1) * uniform01(s);
          q[4 * k + 1] = -1.2 + (1.2 - -1.2) * uniform01(s);
          q[4 * k + 2] = -1.2 + (1.2 - -1.2) * uniform01(s);
          q[4 * k + 3] = 0.03 + (1.5 - 0.03) * uniform01(s);
        }
        setQuadrants(0.8, q);
        break;
      }
      case ShearLayer:
        setDomain(0.0, 1.0, 0.0, 1.0, 1.0, PERIOD, PERIOD, PERIOD, PERIOD);
        rho0 = [](const double, const double y) { return std::fabs(y - 0.5) < 0.25 ? 2.0 : 1.0; };
        u0 = [](const double, const double y) { return std::fabs(y - 0.5) < 0.25 ? 0.5 : -0.5; };
        v0 = [](const double x, const double) { return 0.01 * std::sin(4 * M_PI * x); };
        pre0 = [](const double, const double) { return 2.5; };
        library_initial_state = true;
        break;
      default:
        throw std::invalid_argument("Invalid example number");
    }
  }

  // getU0 (utils/equations.hpp:649-662)
  void getU0(const double x, const double y, double U[4]) const {
    const double rho = rho0(x, y), u = u0(x, y), v = v0(x, y), pre = pre0(x, y);
    const double E = pre / (euler_gamma - 1.0) + 0.5 * rho * (u * u + v * v);
    U[0] = rho;
    U[1] = rho * u;
    U[2] = rho * v;
    U[3] = E;
  }

  int getVitalVarNum() const { return 6; }
  void getVitalVarName(std::string names[6]) const {
    static const char *n[6] = {"rho", "u", "v", "pre", "c", "E"};
    for (int k = 0; k < 6; ++k) names[k] = n[k];
  }
  // getVitalVarVal (utils/equations.hpp:683-698)
  void getVitalVarVal(const double U[4], double out[6]) const {
    const double rho = U[0], u = U[1] / U[0], v = U[2] / U[0], E = U[3];
    const double pre = (euler_gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
    out[0] = rho;
    out[1] = u;
    out[2] = v;
    out[3] = pre;
    out[4] = std::sqrt(euler_gamma * pre / rho);
    out[5] = E;
  }

 private:
  void setDomain(double xl, double xr, double yl, double yr, double t, BOUNDARYTYPE l, BOUNDARYTYPE r,
                 BOUNDARYTYPE b, BOUNDARYTYPE tp) {
    xL = xl;
    xR = xr;
    yL = yl;
    yR = yr;
    outputtime = t;
    leftBoundaryCondition = l;
    rightBoundaryCondition = r;
    bottomBoundaryCondition = b;
    topBoundaryCondition = tp;
  }

  // quadrant k of (x<c,y<c), (x<c,y>=c), (x>=c,y<c), (x>=c,y>=c)
  void setQuadrants(double c, const std::array<double, 16> &q) {
    auto pick = [c, q](int var) {
      return [c, q, var](const double x, const double y) {
        const int k = (x < c) ? (y < c ? 0 : 1) : (y < c ? 2 : 3);
        return q[4 * k + var];
      };
    };
    rho0 = pick(0);
    u0 = pick(1);
    v0 = pick(2);
    pre0 = pick(3);
  }

  static std::uint64_t splitmix64(std::uint64_t &state) {
    std::uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  static double uniform01(std::uint64_t &state) { return double(splitmix64(state) >> 11) * (1.0 / 9007199254740992.0); }
};
