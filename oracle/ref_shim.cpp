// Library form of the reference's own CPU program (test infrastructure only).
//
// This translation unit is compiled by oracle/Makefile against the unmodified
// reference source `siting.cpp` found on the include path (the staged,
// git-ignored copy under oracle/_ref/src; it is never committed).  `main` is
// renamed so that the four stage functions can be called one at a time:
//   calc_vix    siting.cpp:192-198
//   find_max    siting.cpp:235-241
//   calc_sheds  siting.cpp:349-360
//   site_it     siting.cpp:501-626
// Built with -DSEQ (sequential tie-break of siting.cpp:553-562) it is the
// deterministic `seqsite`; built with -fopenmp it is `ompsite` in library form,
// used only for timing.  The block geometry of siting.cpp:688-695 lives in
// main(), so it is restated here in ref_geometry() with the same expressions.
#define main siting_ref_main
#include "siting.cpp"
#undef main

#include <cstdio>
#include <cstdint>

extern "C" {

int ref_geometry(int nrows, int blocksize0, int nwanted0, float *blocksize,
                 int *nblocks, int *nwantedperblock, int *nwanted) {
  float bs = (float)nrows / (int)((float)nrows / blocksize0 + 0.5f);
  int nb = (int)(nrows / bs + 0.5f);
  int npb = (int)((float)nwanted0 / square(nb) + 0.99999f);
  int nw = npb * square(nb);
  int lastsize = nrows - (int)(bs * (nb - 1));
  *blocksize = bs;
  *nblocks = nb;
  *nwantedperblock = npb;
  *nwanted = nw;
  return square(lastsize) < npb ? 1 : 0;
}

void ref_calc_vix(int nrows, const uint16_t *elevs, int roi, int oht, int tht,
                  int ntests, uint8_t *vix) {
  calc_vix(nrows, (const usint *)elevs, roi, oht, tht, ntests, vix);
}

void ref_find_max(int nrows, uint8_t *vix, float blocksize, int nwanted,
                  int nblocks, int nwantedperblock, int32_t *obs) {
  find_max(nrows, vix, blocksize, nwanted, nblocks, nwantedperblock, obs);
}

void ref_calc_sheds(int nrows, const uint16_t *elevs, int roi, int oht,
                    int tht, int nsheds, const int32_t *obs, uint64_t *sheds) {
  calc_sheds(nrows, (const usint *)elevs, roi, oht, tht, nsheds, obs,
             (ullint *)sheds);
}

// site_it prints " nusedsheds:N coverage:C" to stdout (siting.cpp:617); the
// caller recovers N from `selected` and C from the union of selected sheds.
void ref_site_it(int nrows, int roi, int intervis, int nsheds,
                 const int32_t *obs, const uint64_t *sheds, char *selected) {
  site_it(nrows, roi, intervis, nsheds, obs, (const ullint *)sheds, selected);
  cout.flush();
}

int ref_main(int argc, char **argv) { return siting_ref_main(argc, argv); }

// Thread count of the OpenMP build's parallel loops (the program itself fixes
// 50 threads in main, siting.cpp:633-636); returns the count in force, 1 for
// the sequential build.
int ref_set_threads(int n) {
#ifdef _OPENMP
  omp_set_dynamic(0);
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

}  // extern "C"
