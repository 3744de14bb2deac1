// Command-line form of the CPU oracle (test infrastructure and CPU baseline):
// the same options as run_md_simulation (run_md_simulation.f90:26-55).
#include "oracle.h"

int main(int argc, char** argv) { return orc_run_md_simulation(argc, argv); }
