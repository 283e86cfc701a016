/*
 * leo2d_ref: runs the reference's unmodified main() (app/src/main.cpp:23,
 * renamed at compile time) on in-process MPI ranks.
 *
 * TEST INFRASTRUCTURE ONLY. The reference refuses to run on one MPI rank
 * (main.cpp:943-948) and uses a master/worker job farm
 * (src/locality.cpp:2694-2771), so this launcher starts LEO2D_REF_RANKS
 * threads (default 2), each with its own rank, and runs main() in every one of
 * them. Ranks exchange messages through mpi_inproc.cpp. Thread stacks are
 * 1 GiB because the reference keeps its Chebyshev vectors in stack arrays
 * (src/locality.cpp:5965-5982, 2939).
 */
#include <pthread.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "mpi.h"

int leo2d_ref_main(int argc, char** argv);

namespace {
struct RankArgs {
  int rank, size, argc;
  char** argv;
  int rc;
};

void* run_rank(void* p) {
  RankArgs* a = static_cast<RankArgs*>(p);
  leo2d_inproc_set_rank(a->rank, a->size);
  a->rc = leo2d_ref_main(a->argc, a->argv);
  return nullptr;
}
}  // namespace

int main(int argc, char** argv) {
  const char* env = std::getenv("LEO2D_REF_RANKS");
  int n = env ? std::atoi(env) : 2;
  if (n < 2) n = 2;
  std::vector<RankArgs> args(n);
  std::vector<pthread_t> th(n);
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, (size_t)1 << 30);
  for (int r = 0; r < n; ++r) {
    args[r] = RankArgs{r, n, argc, argv, 0};
    if (pthread_create(&th[r], &attr, run_rank, &args[r]) != 0) {
      std::fprintf(stderr, "leo2d_ref: cannot start rank %d\n", r);
      return 3;
    }
  }
  for (int r = 0; r < n; ++r) pthread_join(th[r], nullptr);
  return args[0].rc;
}
