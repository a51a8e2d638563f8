/*
 * sphrayderv_main.cpp — drop-in replacement of the sphrayderv program (reference: src/sphrayderv.c
 * main) for local earthquakes.  Same interface: the spec-file name is read from stdin; the station
 * list, event file, time files and the six output files are the ones the spec names.  The rays are
 * traced on the GPU (fdgpu_sphrayderv).  The spacing rule of the reference (dq, df below 1e-4 rad
 * replaced by h/rearth) applies unless FDGPU_KEEP_SPACING=1 is set, for fields computed with the
 * spec's own spacing.  Exit status 0 on success, 1 otherwise (the reference aborts instead).
 */
#include "fdgpu.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

int main()
{
    char spec[1024];
    std::printf("Enter parameter specification file: ");
    if (std::scanf("%1023s", spec) != 1) return 1;
    const char *keep = std::getenv("FDGPU_KEEP_SPACING");
    const int rule = (keep && std::strcmp(keep, "1") == 0) ? 0 : 1;
    const int rc = fdgpu_sphrayderv(spec, rule, nullptr, nullptr);
    if (rc != FDGPU_OK) {
        std::fprintf(stderr, "sphrayderv: %s\n", fdgpu_strerror(rc));
        return 1;
    }
    return 0;
}
