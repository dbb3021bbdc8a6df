// spherocyl_find_jam -- bisection of the packing fraction to a jamming energy
// (find_jam_2p); arguments and files as described in cli_jam.hpp.
#include "cli_jam.hpp"

int main(int argc, char** argv) { return cli::jam_main(argc, argv, false); }
