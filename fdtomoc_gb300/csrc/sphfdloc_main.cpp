/*
 * sphfdloc_main.cpp — drop-in replacement of the sphfdloc program (reference: src/sphfdloc.c main).
 * Same interface: the spec-file name is read from stdin; the event file, time files and the four
 * report files are the ones the spec names.  The events are located on the GPU (fdgpu_sphfdloc).
 * Exit status 0 on success, 1 otherwise (the reference aborts instead).
 */
#include "fdgpu.h"

#include <cstdio>

int main()
{
    char spec[1024];
    std::printf("Enter parameter specification file: ");
    if (std::scanf("%1023s", spec) != 1) return 1;
    const int rc = fdgpu_sphfdloc(spec, nullptr, nullptr);
    if (rc != FDGPU_OK) {
        std::fprintf(stderr, "sphfdloc: %s\n", fdgpu_strerror(rc));
        return 1;
    }
    return 0;
}
