/* ref_medfilter.c — C harness around the reference's own median filter
 * (src/medfilter.hpp: ConstantTimeMedianFilter), compiled from the header
 * where it lies in the reference tree by oracle/build.py into
 * oracle/_ref/libref_medfilter.so.  Test infrastructure only: it generates
 * the golden median fixtures and checks the oracle's restatement.
 *
 * The call mirrors pguresvt.hpp:69-80: width = Nx, height = Ny, both steps
 * Nx, radius medianSize, one channel, memsize 1 MiB.                       */
#include <stdint.h>
#include "medfilter.hpp"

void ref_median_filter(const uint16_t* src, uint16_t* dst, int nx, int ny, int r) {
  ConstantTimeMedianFilter(src, dst, nx, ny, nx, nx, r, 1, 1024 * 1024);
}
