// Test-case definitions on the host: domain, gamma, boundary types, end
// time and initial condition of each TESTCASE (EulerEquation::
// setEquationParameters and getU0, utils/equations.hpp:400-662), plus the
// two seeded cases the reference has no enum for.
#pragma once

#include <cstdint>
#include <vector>

namespace wenofd {

struct CaseSpec {
  int testcase = 0;
  double xl = 0, xr = 1, yl = 0, yr = 1;
  double t_end = 1, gamma = 1.4;
  int bc_left = 0, bc_right = 0, bc_bottom = 0, bc_top = 0;
  int gravity = 0;      // RTI source term
  int exact = 0;        // u_exact_exist
  double quad[16] = {}; // {rho,u,v,p} per quadrant (x<c,y<c), (x<c,y>=c), (x>=c,y<c), (x>=c,y>=c)
  double interface = 0.8;
  uint64_t seed = 0;
};

// Throws std::invalid_argument for an unknown testcase, as the reference
// does (utils/equations.hpp:643-644).
CaseSpec make_case(int testcase, uint64_t seed);

// Node coordinates with the reference's rounding: (xl - dx*4) + ei*dx
// (src/WENOFD.cpp:76-79, 100-101); ei, ej include the 4 ghost nodes.
double node_x(const CaseSpec &c, double dx, int ei);
double node_y(const CaseSpec &c, double dy, int ej);

// Conserved initial state of one node (getU0).  Not for the shear layer,
// whose noise depends on the node index.
void u0(const CaseSpec &c, double x, double y, double U[4]);

// Interior initial state [4][nx][ny] (initializeAve, src/WENOFD.cpp:165-188).
void initial_state(const CaseSpec &c, int nx, int ny, double dx, double dy, double *out);

// SPECIAL ghost values: getU0 at fixed boundary nodes, tabulated once.
// Layout (nxt = nx+8, nyt = ny+8), each block r-major:
//   [0, 4nxt) bottom per ei at node (ei, 4);  [4nxt, 8nxt) top at (ei, ny+3);
//   [8nxt, +4nyt) left per ej at (4, ej);      [.., +4nyt) right at (nx+4, ej).
std::vector<double> special_table(const CaseSpec &c, int nx, int ny, double dx, double dy);

uint64_t splitmix64(uint64_t &state);
double uniform01(uint64_t &state);

}  // namespace wenofd
