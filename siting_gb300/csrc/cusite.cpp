// cusite: drop-in replacement for the reference's command line
//   cusite nrows roi height targets bw nwanted intervis inputfile outputfile
// (siting.cu:746-919, siting.cpp:632-780), running the four stages on the GPU
// through the library's C ABI.  Argument checks print the reference's
// messages as "ERROR: <msg>" on stdout and exit 1 (siting.cpp:22-25,
// 663-695); the stdout timing line keeps the reference's keys; the observers
// file is "x,y\n" per selected observer in index order (siting.cpp:761-765).
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "siting.h"

namespace {

[[noreturn]] void die(const char *msg) {
  std::cout << "ERROR: " << msg << std::endl;
  std::exit(1);
}

double secs(const timeval &a, const timeval &b) {
  return (double)(b.tv_sec - a.tv_sec) + (b.tv_usec - a.tv_usec) / 1e6;
}

}  // namespace

int main(int argc, char **argv) {
  timeval begin, middle, end;
  gettimeofday(&begin, nullptr);
  middle = begin;
  if (argc != 10) {
    std::cout << "argc=" << argc << std::endl;
    die("SITE requires 9 arguments: nrows, roi, oht/tht, ntests, blocksize, nwanted, intervis, "
        "infile, outfile");
  }
  siting_params p;
  p.nrows = std::atoi(argv[1]);
  p.roi = std::atoi(argv[2]);
  p.oht = p.tht = std::atoi(argv[3]);
  p.ntests = std::atoi(argv[4]);
  p.bw = std::atoi(argv[5]);
  p.nwanted0 = std::atoi(argv[6]);
  p.intervis = std::atoi(argv[7]);
  char msg[256];
  if (siting_validate(&p, 0, msg, sizeof msg) != SITING_OK) die(msg);
  siting_geometry g;
  siting_block_geometry(p.nrows, p.bw, p.nwanted0, &g);

  const size_t ncell = (size_t)p.nrows * p.nrows;
  // Page-locked when a device is present (faster upload), plain memory otherwise.
  uint16_t *elevs = nullptr;
  bool pinned = siting_pinned_alloc(ncell * sizeof(uint16_t), (void **)&elevs) == SITING_OK;
  if (!pinned) elevs = static_cast<uint16_t *>(std::malloc(ncell * sizeof(uint16_t)));
  if (!elevs) die("Memory exhausted. Program terminates.");
  std::vector<int32_t> obs(g.nwanted);
  std::vector<uint8_t> selected(g.nwanted);
  if (siting_read_dem(argv[8], p.nrows, elevs) != SITING_OK) die("Input failed");
  gettimeofday(&end, nullptr);
  std::cout << "input:" << secs(middle, end);
  middle = end;

  siting_ctx *ctx = nullptr;
  if (siting_ctx_create(0, 0, &ctx) != SITING_OK) die("no usable CUDA device");
  siting_result r{};
  const int rc = siting_run(ctx, &p, elevs, obs.data(), selected.data(), &r);
  if (rc != SITING_OK) die(siting_last_error(ctx));
  // Stage lines as the reference prints them; device times come from CUDA
  // events around each stage, host copies are counted in the first stage.
  std::cout << " vix:" << (r.ms_h2d + r.ms_vix) / 1e3 << " findmax:" << r.ms_findmax / 1e3
            << " viewshed:" << r.ms_viewshed / 1e3;
  std::cout << " nusedsheds:" << r.nusedsheds << " coverage:" << r.coverage;
  std::cout << " site:" << (r.ms_site + r.ms_d2h) / 1e3;
  gettimeofday(&middle, nullptr);
  if (siting_write_observers(argv[9], p.nrows, g.nwanted, obs.data(), selected.data()) !=
      SITING_OK)
    die("Output failed");
  gettimeofday(&end, nullptr);
  std::cout << " output:" << secs(middle, end);
  std::cout << " total:" << secs(begin, end) << std::endl;
  siting_ctx_destroy(ctx);
  if (pinned)
    siting_pinned_free(elevs);
  else
    std::free(elevs);
  return 0;
}
