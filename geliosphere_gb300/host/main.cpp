// The `geliosphere` executable: the reference application's command line
// (main.cpp:22-40) over the GB300 engine.
#include "gelio_host.h"

int main(int argc, char **argv) {
  const int rc = gelio_host_main(argc, argv);
  return rc < 0 ? 255 : rc;
}
