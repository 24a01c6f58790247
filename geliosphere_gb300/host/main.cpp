// The `geliosphere` executable: the reference application's command line
// (main.cpp:22-40) over the GB300 engine.
#include "gelio_host.h"

int main(int argc, char **argv) { return gelio_host_main(argc, argv) == 0 ? 0 : 255; }
