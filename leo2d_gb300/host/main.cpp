// main.cpp - `leo2d file.in`: runs one KPM input on GPU 0 and writes the same
// files the reference's `LEO2D file.in` writes for that path (app/src/main.cpp:23).
// One process, one GPU: no MPI ranks are needed (main.cpp:943-948).
#include <cstdio>
#include <cstdlib>

#include "../../include/leo2d_gpu.h"

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: leo2d file.in [out_dir] [device]\n");
    return 2;
  }
  const char* out = argc > 2 ? argv[2] : ".";
  const int device = argc > 3 ? std::atoi(argv[3]) : 0;
  char msg[1024] = {0};
  const leo2d_status st = leo2d_run_input(argv[1], out, device, msg, sizeof(msg));
  if (st != LEO2D_OK) {
    std::fprintf(stderr, "leo2d: %s: %s\n", leo2d_status_string(st), msg);
    return 1;
  }
  return 0;
}
