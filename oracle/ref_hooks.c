/*
 * Stage dumper for the reference metapart.c (test infrastructure only).
 *
 * This translation unit includes the unmodified reference source
 * (src/metapart.c, found through -I at build time) and routes every
 * gettimeofday() call of that file through mp_hook_time().  The reference
 * brackets each stage with gettimeofday, so the hook sees the exact points
 * between stages and can dump the reference's globals (sortedKmers, rcvKmers,
 * parent, filteredReads, compSizes) without any edit to the reference.
 *
 * Dumps go to $MP_DUMP_DIR (nothing is written when it is unset):
 *   scan<s>_enum.bin     tuples in enumeration order     (metapart.c:1983, sortKmerList entry)
 *   scan<s>_sorted.bin   tuples after the stable sort    (metapart.c:2274, markMischiefKmers entry)
 *   scan<s>_filtered.bin tuples after the mischief filter (metapart.c:2523, unionFindPar2 entry)
 *   scan<s>_bad.bin      filteredReads after the filter   (same point)
 *   stats<c>_parent.bin  5-byte parent array after printStats call c (metapart.c:3305)
 *   stats<c>_sizes.bin   compSizes after printStats call c
 *   pe_parent.bin / pe_sizes.bin  state after unionFindPeReads (metapart.c:2863)
 * Tuples are the reference's 14-byte records (7 x u16).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

static int mp_hook_time(struct timeval *tv, void *tz, const char *fn, int line);
#define gettimeofday(tv, tz) mp_hook_time((tv), (tz), __func__, __LINE__)
#define main ref_metapart_main
#include "metapart.c"
#undef main
#undef gettimeofday

static int mp_scan_enum = 0, mp_scan_sorted = 0, mp_scan_filtered = 0, mp_stats = 0;

static void mp_dump(const char *name, const void *buf, size_t bytes)
{
    const char *dir = getenv("MP_DUMP_DIR");
    if (!dir || !buf) return;
    char path[1024];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "hook: cannot write %s\n", path); exit(3); }
    if (bytes && fwrite(buf, 1, bytes, f) != bytes) { fprintf(stderr, "hook: short write\n"); exit(3); }
    fclose(f);
}

static int mp_hook_time(struct timeval *tv, void *tz, const char *fn, int line)
{
    char name[256];
    if (strcmp(fn, "sortKmerList") == 0 && line == 1983) {
        snprintf(name, sizeof(name), "scan%d_enum.bin", mp_scan_enum++);
        mp_dump(name, rcvKmers, (size_t)numKmers * 14);
    } else if (strcmp(fn, "markMischiefKmers") == 0 && line == 2274) {
        snprintf(name, sizeof(name), "scan%d_sorted.bin", mp_scan_sorted++);
        mp_dump(name, sortedKmers, (size_t)numKmers * 14);
    } else if (strcmp(fn, "unionFindPar2") == 0 && line == 2523) {
        snprintf(name, sizeof(name), "scan%d_filtered.bin", mp_scan_filtered);
        mp_dump(name, sortedKmers, (size_t)numKmers * 14);
        snprintf(name, sizeof(name), "scan%d_bad.bin", mp_scan_filtered++);
        mp_dump(name, filteredReads, (size_t)numReads);
    } else if (strcmp(fn, "printStats") == 0 && line == 3305) {
        snprintf(name, sizeof(name), "stats%d_parent.bin", mp_stats);
        mp_dump(name, parent, (size_t)numReads * 5);
        snprintf(name, sizeof(name), "stats%d_sizes.bin", mp_stats++);
        mp_dump(name, compSizes, (size_t)numReads * 4);
    } else if (strcmp(fn, "unionFindPeReads") == 0 && line == 2863) {
        mp_dump("pe_parent.bin", parent, (size_t)numReads * 5);
        mp_dump("pe_sizes.bin", compSizes, (size_t)numReads * 4);
    }
    return gettimeofday(tv, tz);
}

int main(int argc, char **argv) { return ref_metapart_main(argc, argv); }
