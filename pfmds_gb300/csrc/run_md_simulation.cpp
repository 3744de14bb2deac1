// The drop-in run_md_simulation executable: see pfmd_run_md_simulation.
#include "../../include/pfmd.h"

int main(int argc, char** argv) { return pfmd_run_md_simulation(argc, argv); }
