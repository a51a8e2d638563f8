/*
 * fd_oracle_main.c — command-line driver for the CPU oracle with the reference's interface
 * (src/sphfd.c:200-257): the spec-file name is read from stdin, its "parlist" and "timedir" keys
 * name the par-file list and the output directory, and every "par=<file>" line is one station.
 *
 * TEST INFRASTRUCTURE (the checker); FDO_MODE=fast selects the pruned / tabled evaluation.
 */
#include "fd_oracle.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* First line whose first whitespace-separated field equals name; value = second field
 * (get_vars, lib/common/parseprogs.c:9-79). */
static int spec_get(FILE *fp, const char *name, char *out, size_t cap)
{
    char line[512], a[256], b[256];
    rewind(fp);
    while (fgets(line, sizeof line, fp)) {
        if (sscanf(line, "%255s %255s", a, b) == 2 && strcmp(a, name) == 0) {
            snprintf(out, cap, "%s", b);
            return 1;
        }
    }
    return 0;
}

int main(void)
{
    char spec[512], parlist[512] = "", timedir[512] = "", line[600];
    if (scanf("%511s", spec) != 1) return 2;
    FILE *fs = fopen(spec, "r");
    if (!fs) { fprintf(stderr, "cannot open spec %s\n", spec); return 2; }
    spec_get(fs, "parlist", parlist, sizeof parlist);
    spec_get(fs, "timedir", timedir, sizeof timedir);
    fclose(fs);
    FILE *fl = fopen(parlist, "r");
    if (!fl) { fprintf(stderr, "cannot open parlist %s\n", parlist); return 2; }
    const char *m = getenv("FDO_MODE");
    const int mode = (m && strcmp(m, "fast") == 0) ? FDO_MODE_FAST : FDO_MODE_LITERAL;
    int failures = 0;
    while (fgets(line, sizeof line, fl)) {
        if (line[0] == '\n') break;
        line[strcspn(line, "\n")] = 0;
        char *av[2] = {"sphfd", line};
        fdo_stats st;
        memset(&st, 0, sizeof st);
        int rc = fdo_sphfd(2, av, timedir, mode, &st);
        if (rc) { fprintf(stderr, "%s: error %d\n", line, rc); failures++; continue; }
        if (getenv("FDO_CHANGED"))
            for (int k = 0; k < st.sweeps && k < 64; k++)
                fprintf(stderr, "sweep %d changed %lld updates %lld depth %lld\n", k, (long long)st.changed_per_sweep[k],
                        (long long)st.updates_per_sweep[k], (long long)st.depth_per_sweep[k]);
        fprintf(stderr, "%s: sweeps=%d node_updates=%lld faces=%lld inherit=%lld calls=%lld/%lld/%lld/%lld/%lld skipped=%lld/%lld/%lld/%lld\n",
                line, st.sweeps, (long long)st.node_updates, (long long)st.faces, (long long)st.inherit_points,
                (long long)st.calls[0], (long long)st.calls[1], (long long)st.calls[2], (long long)st.calls[3],
                (long long)st.calls[4], (long long)st.skipped[0], (long long)st.skipped[1], (long long)st.skipped[2],
                (long long)st.skipped[3]);
    }
    fclose(fl);
    return failures ? 1 : 0;
}
