/* JoinT_gpu: command-line drop-in for `./JoinT param_JoinT.ini`
 * (src/main_jt.c:326-389): reads the reference .ini, the component maps
 * <prefix>_%03d.fits, the frequency table and the mask, runs merge, beam, noise
 * and mask on GPU 0 and writes <prefix_out>_%03d.fits and
 * <prefix_out>_instrument.dat. */
#include <stdio.h>

#include "joint_gpu.h"

int main(int argc, char **argv)
{
  if (argc != 2) {
    fprintf(stderr, "Usage: ./JoinT file_name\n");
    return 1;
  }
  int rc = joint_host_run(argv[1], 0);
  if (rc != GETHI_OK) {
    fprintf(stderr, "CRIME: %s\n", gethi_last_error());
    return 1;
  }
  return 0;
}
