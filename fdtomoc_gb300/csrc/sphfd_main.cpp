/*
 * sphfd_main.cpp — drop-in replacement of the sphfd program's main() (reference: src/sphfd.c:200-257).
 *
 * Same interface: the spec-file name is read from stdin; its "parlist" and "timedir" entries name
 * the list of "par=<file>" lines and the output directory (get_vars semantics,
 * lib/common/parseprogs.c:9-79: the first line whose first field is the key; the value is the
 * second field).  The list ends at EOF or at an empty line, as in the reference.  Instead of one
 * OpenMP thread per par file, every station is solved on the GPU in one batch.  Exit status 0 when
 * every station succeeded, 1 otherwise (the reference aborts instead).
 */
#include "fdgpu.h"

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

static bool spec_get(FILE *fp, const char *key, std::string &out)
{
    char line[1024], a[512], b[512];
    std::rewind(fp);
    while (std::fgets(line, sizeof line, fp)) {
        if (std::sscanf(line, "%511s %511s", a, b) == 2 && std::strcmp(a, key) == 0) {
            out = b;
            return true;
        }
    }
    return false;
}

int main()
{
    char spec[1024];
    std::printf("Input the name spec file\n");
    if (std::scanf("%1023s", spec) != 1) return 2;
    FILE *fs = std::fopen(spec, "r");
    if (!fs) { std::fprintf(stderr, "Error on opening spec file(%s)\n", spec); return 2; }
    std::string parlist, timedir;
    spec_get(fs, "parlist", parlist);
    spec_get(fs, "timedir", timedir);
    std::fclose(fs);
    std::printf("%s\n", parlist.c_str());
    FILE *fl = std::fopen(parlist.c_str(), "r");
    if (!fl) { std::fprintf(stderr, "Error on opening parlist(%s)\n", parlist.c_str()); return 2; }
    std::vector<std::string> entries;
    char line[1024];
    while (std::fgets(line, sizeof line, fl)) {
        if (line[0] == '\n') break;
        line[std::strcspn(line, "\n")] = 0;
        entries.emplace_back(line);
    }
    std::fclose(fl);
    std::vector<char *> av;
    for (auto &e : entries) av.push_back(&e[0]);
    std::vector<int> status(entries.size(), 0);
    fdgpu_sphfd_parlist((int)av.size(), av.data(), timedir.c_str(), status.data());
    int bad = 0;
    for (size_t k = 0; k < entries.size(); k++)
        if (status[k]) {
            std::fprintf(stderr, "%s: %s\n", entries[k].c_str(), fdgpu_strerror(status[k]));
            bad++;
        }
    return bad ? 1 : 0;
}
