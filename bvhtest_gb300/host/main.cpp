// bvhTest command-line runner: list | generate FILE CMD... | run CFG (src/main.cpp:97-244); the
// logic lives in libbvhgb (bvhgb_cli_main) so the runner stays a thin executable.
#include "../../include/bvhgb.h"

int main(int argc, char **argv) { return bvhgb_cli_main(argc, argv); }
