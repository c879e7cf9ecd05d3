// hdog_main.cpp -- drop-in for the reference's HDoG3D_main executable
// (src/3D/HDoG3D_main.cpp:260-319): `hdog_main PARAM_FILE`, the parameter JSON that
// script/HDoG_gpu.py writes, one 28-byte record per kept candidate appended to each
// stack's dst_path.  Exit status 2 on usage, parameter or I/O errors (as the reference's
// exit(2) paths), 1 on any other failure, 0 on success.
#include <cstdio>

#include "../../include/hdog.h"

int main(int argc, char **argv) {
  if (argc != 2) {
    std::printf("Usage:\n%s PARAM_FILE\n", argv[0]);
    return 2;
  }
  const int rc = hdog_run_param_file(argv[1], 1);
  if (rc != HDOG_OK) {
    std::fprintf(stderr, "hdog_main: %s\n", hdog_last_error());
    return (rc == HDOG_ERR_IO || rc == HDOG_ERR_PARAM || rc == HDOG_ERR_ARG) ? 2 : 1;
  }
  return 0;
}
