/*
 * fdgpu_check.cuh — optional index checks for diagnosing a bad access (FD_SELFCHECK builds only).
 *
 * FD_OK(idx, bound, site) is true when 0 <= idx < bound.  In a build with FD_SELFCHECK defined a
 * failing check is counted and the first one recorded (site and index) in a device word the host
 * reads with fdk_selfcheck_read(); the caller then skips or clamps the access, so a bad index shows
 * up as a record instead of a fault.  In normal builds the macro is the constant true.
 */
#ifndef FDGPU_CHECK_CUH
#define FDGPU_CHECK_CUH

#ifdef FD_SELFCHECK
static __device__ unsigned long long fd_selfcheck_words[3];   /* count, first site, first index */

__device__ __forceinline__ bool fd_check_index(long long idx, long long bound, int site)
{
    if (idx >= 0 && idx < bound) return true;
    if (atomicAdd(&fd_selfcheck_words[0], 1ull) == 0ull) {
        fd_selfcheck_words[1] = (unsigned long long)site;
        fd_selfcheck_words[2] = (unsigned long long)idx;
    }
    return false;
}
#define FD_OK(idx, bound, site) fd_check_index((long long)(idx), (long long)(bound), (site))
#else
#define FD_OK(idx, bound, site) true
#endif

#endif
