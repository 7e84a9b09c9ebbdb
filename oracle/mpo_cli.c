/*
 * Command-line front end of the CPU oracle (test infrastructure).  The three
 * sub-commands take the reference programs' positional arguments:
 *
 *   mpo_cli genFastqIdx numPartitions numPEFiles numSEFiles numInterleavedFiles files...
 *   mpo_cli genHistograms [--min3] kmerSize numPEFiles numSEFiles numInterleavedFiles files...
 *   mpo_cli metapart [--min3] -o outPrefix fastqBufferSize kmerSize numScans numThreads
 *                    numPEFiles numSEFiles numInterleavedFiles files...
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mp_oracle.h"

static int usage(void)
{
    fprintf(stderr, "usage: mpo_cli genFastqIdx|genHistograms|metapart ...\n");
    return 2;
}

int main(int argc, char **argv)
{
    if (argc < 2) return usage();
    int rc;
    if (!strcmp(argv[1], "genFastqIdx")) {
        if (argc < 7) return usage();
        rc = mpo_fastq_index(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), atoi(argv[5]), argc - 6,
                             (const char *const *)&argv[6]);
    } else if (!strcmp(argv[1], "genHistograms")) {
        int a = 2, min3 = 0;
        if (a < argc && !strcmp(argv[a], "--min3")) { min3 = 1; a++; }
        if (argc - a < 5) return usage();
        rc = mpo_gen_histograms(atoi(argv[a]), min3, atoi(argv[a + 1]), atoi(argv[a + 2]), atoi(argv[a + 3]),
                                argc - a - 4, (const char *const *)&argv[a + 4]);
    } else if (!strcmp(argv[1], "metapart")) {
        int a = 2, min3 = 0;
        const char *out = ".";
        while (a < argc && argv[a][0] == '-') {
            if (!strcmp(argv[a], "--min3")) { min3 = 1; a++; }
            else if (!strcmp(argv[a], "-o") && a + 1 < argc) { out = argv[a + 1]; a += 2; }
            else return usage();
        }
        if (argc - a < 8) return usage();
        rc = mpo_metapart(out, strtoull(argv[a], NULL, 10), atoi(argv[a + 1]), atoi(argv[a + 2]), atoi(argv[a + 3]),
                          min3, atoi(argv[a + 4]), atoi(argv[a + 5]), atoi(argv[a + 6]), argc - a - 7,
                          (const char *const *)&argv[a + 7]);
    } else {
        return usage();
    }
    if (rc) {
        fprintf(stderr, "mpo_cli %s: error %d: %s\n", argv[1], rc, mpo_last_error());
        return 1;
    }
    return 0;
}
