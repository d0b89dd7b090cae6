// Test oracle command line: the reference's test_compress_cpu flags and
// output, run by the CPU restatement in wl_port.cpp.  Test infrastructure only.
#include "wl_port.h"

int main(int argc, char **argv) { return orc_main(argc, (const char **)argv); }
