// Driver with the flow of the reference's src/main.cpp:5-33: read
// ./input/config.cfg, build the equation object and the solver, run.
// An optional first argument replaces the config path.
#include <iostream>
#include <map>
#include <string>

#include "WENOFD.hpp"

int main(int argc, char *argv[]) {
  try {
    EulerEquation equation;
    const std::string inputfile = argc > 1 ? argv[1] : "./input/config.cfg";
    std::cout << "Starting to read configuration file..." << std::endl;
    CConfig config(inputfile);
    std::map<std::string, std::string> option;
    config.read(option);
    CWENOFD solver(&equation);
    solver.run(option);
  } catch (const std::exception &e) {
    std::cerr << "Error: " << e.what() << std::endl;
    return 1;
  }
  return 0;
}
