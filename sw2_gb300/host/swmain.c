/* Command line of sw2g-run (see swrun.c): the reference's `SW NPX NPY CASE
 * OUTDIR` (main/Main.c:34-37) on one GPU, one rank. */
#include <stdio.h>
#include <string.h>

int sw2g_run_case(const char *bname, const char *outdir, int fp32, int quiet, int checkpoint, int resume,
                  int device_forcing, int timing);

int main(int argc, char **argv) {
  int fp32 = 0, quiet = 0, checkpoint = 0, resume = -1, device_forcing = 0, timing = 0, a = 1;
  for (; a < argc && argv[a][0] == '-' && argv[a][1] == '-'; a++) {
    if (!strcmp(argv[a], "--fp32")) fp32 = 1;
    else if (!strcmp(argv[a], "--quiet")) quiet = 1;
    else if (!strcmp(argv[a], "--checkpoint")) checkpoint = 1;
    else if (!strcmp(argv[a], "--device-forcing")) device_forcing = 1;
    else if (!strcmp(argv[a], "--timing")) timing = 1;
    else if (!strcmp(argv[a], "--resume") && a + 1 < argc && sscanf(argv[a + 1], "%d", &resume) == 1 && resume >= 0)
      a++;
    else {
      fprintf(stderr, "sw2g-run: unknown option %s\n", argv[a]);
      return 2;
    }
  }
  if (argc - a != 4) {
    fprintf(stderr, "Run as\n  sw2g-run [--fp32] [--quiet] [--checkpoint] [--resume F] npx npy input_file output_folder\n"
                    "with npx = npy = 1 (one GPU); input_file without its .sw extension\n");
    return 2;
  }
  int npx = 0, npy = 0;
  if (sscanf(argv[a], "%d", &npx) != 1 || sscanf(argv[a + 1], "%d", &npy) != 1 || npx != 1 || npy != 1) {
    fprintf(stderr, "sw2g-run: runs one rank on one GPU: npx and npy must be 1\n");
    return 2;
  }
  return sw2g_run_case(argv[a + 2], argv[a + 3], fp32, quiet, checkpoint, resume, device_forcing, timing);
}
