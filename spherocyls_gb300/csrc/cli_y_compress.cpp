// spherocyl_y_compress -- the find-jam bisection with resizes of Ly and y alone
// (y_compress_energy_2p); arguments and files as described in cli_jam.hpp.
#include "cli_jam.hpp"

int main(int argc, char** argv) { return cli::jam_main(argc, argv, true); }
