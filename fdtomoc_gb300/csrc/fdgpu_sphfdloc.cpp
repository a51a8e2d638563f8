/* sphfdloc's driver around the device search (reference src/sphfdloc.c main): the spec, event file
 * and time files read as the reference reads them, every event located (fdgpu_locate by default),
 * and the four report files written as the reference writes them (:1129-1250).
 *
 * The reference splits the event file into one file per event under eqkdir and reads every time file
 * of timedir; this driver reads the event file directly and the time files its phases name, which
 * gives the same events and tables.  Where the reference asserts (a phase other than P or S, a missing
 * time file) the driver returns an error. */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/fdgpu.h"

namespace {

const double kDegrad = 0.017453292f;   /* src/sphfdloc.c:74-75: float literals */
const double kHpi = 1.570796f;

int leap(int y) { return ((y % 4 == 0 && y % 100 != 0) || y % 400 == 0) ? 1 : 0; }

/* epoch seconds (lib/common/time_process.c:85-109) */
double htoe(int iyear, int iday, int ihour, int imin, double sec)
{
    int days = 0;
    if (iyear > 1970)
        for (int y = 1970; y < iyear; y++) days += 365 + leap(y);
    else if (iyear < 1970)
        for (int y = iyear; y <= 1969; y++) days -= 365 + leap(y);
    days += iday - 1;
    double e = (double)(days * 24 * 60 * 60);
    return e + 3600.0 * ihour + 60.0 * imin + sec;
}

/* and back (lib/common/time_process.c etoh): day of the epoch, then hour, minute, second */
void etoh(double epoch, int *iyear, int *iday, int *ihour, int *imin, double *sec)
{
    int doy = (int)(epoch / 86400.0);
    double left = std::fmod(epoch, 86400.0);
    int hour = 0, minute = 0;
    double second = 0.0;
    if (left != 0.0) {
        if (left < 0) {
            doy -= 1;
            left += 86400;
        }
        hour = (int)(left / 3600);
        left = std::fmod(left, 3600.0);
        minute = (int)(left / 60);
        second = std::fmod(left, 60.0);
    }
    int year;
    if (doy >= 0) {
        year = 1970;
        while (doy >= 365 + leap(year)) {
            doy -= 365 + leap(year);
            year++;
        }
    } else {
        year = 1969;
        while (doy < 0) {
            doy += 365 + leap(year);
            year--;
        }
    }
    *iyear = year;
    *iday = doy + 1;
    *ihour = hour;
    *imin = minute;
    *sec = second;
}

/* geocentric latitude and radius -> geographic latitude and height (WGS84, five fixed-point steps;
 * lib/common/geographic_method.c glathinv with height) */
double glathinv(double xcent, double r, double *h)
{
    const double ap = 6378137.0;
    const double esq = 6.69437978616733379 * 0.001;
    const double rm = r * 1000.0;
    double lat = xcent;
    const double x = rm * std::cos(lat);
    const double z = rm * std::sin(lat);
    double anu = 0.0;
    for (int it = 0; it < 5; it++) {
        const double s = std::sin(lat);
        anu = ap / std::sqrt(1.0 - esq * s * s);
        const double hb = x / std::cos(lat) - anu;
        const double zp = z / (1.0 - esq * (anu / (anu + hb)));
        lat = std::atan2(zp, x);
    }
    *h = x / std::cos(lat) - anu;
    *h = -*h / 1000.0;
    return lat;
}

/* trailing blanks off in place, as the reference's trim() is used (its return value ignored) */
void trim_tail(char *s)
{
    size_t n = std::strlen(s);
    while (n > 0 && (s[n - 1] == ' ' || s[n - 1] == '\t' || s[n - 1] == '\n' || s[n - 1] == '\r' ||
                     s[n - 1] == '\v' || s[n - 1] == '\f'))
        s[--n] = '\0';
}

/* spec variables, get_vars style: the first line whose first field is the name */
struct Spec {
    std::map<std::string, std::vector<std::string>> v;
    bool load(const char *path)
    {
        FILE *f = std::fopen(path, "r");
        if (!f) return false;
        char line[4096];
        while (std::fgets(line, sizeof line, f)) {
            std::vector<std::string> fields;
            char *save = nullptr;
            for (char *t = strtok_r(line, " \t\r\n", &save); t; t = strtok_r(nullptr, " \t\r\n", &save))
                fields.emplace_back(t);
            if (fields.size() < 2) continue;
            const std::string key = fields[0];
            fields.erase(fields.begin());
            v.emplace(key, std::move(fields));
        }
        std::fclose(f);
        return true;
    }
    bool has(const char *k) const { return v.count(k) != 0; }
    std::string str(const char *k, const char *dflt = "") const
    {
        auto it = v.find(k);
        return it == v.end() ? std::string(dflt) : it->second[0];
    }
    template <class T> void get(const char *k, const char *fmt, T *out) const
    {
        if (has(k)) std::sscanf(str(k).c_str(), fmt, out);
    }
    std::vector<int> ints(const char *k, int n) const
    {
        std::vector<int> out;
        auto it = v.find(k);
        if (it == v.end()) return out;
        for (int q = 0; q < n && q < (int)it->second.size(); q++) {
            int x = 0;
            std::sscanf(it->second[q].c_str(), "%d", &x);
            out.push_back(x);
        }
        return out;
    }
};

struct Phase {
    std::string sta;
    int iyr, jday, ihr, imn;
    float sec;
    char phase;
    float rwt;
    int good;
    float obstime, pwt;
};

struct LocEvent {
    int iyr, jday, ihr, imn;
    float sec;
    std::string evid;
    double dpot;
    std::vector<Phase> ph;
};

/* the event file (:566-667): a header line, one line per phase, events separated by a blank line */
int read_events(const std::string &path, std::vector<LocEvent> &out)
{
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) return FDGPU_EIO;
    char line[1024];
    LocEvent *cur = nullptr;
    while (std::fgets(line, sizeof line, f)) {
        trim_tail(line);
        if (line[0] == '\0') {
            cur = nullptr;
            continue;
        }
        if (!cur) {
            LocEvent e{};
            float xlat = 0, xlon = 0, dep = 0;
            char evid[256] = "";
            std::sscanf(line, "%d %d %d %d %f %f %f %f %255s", &e.iyr, &e.jday, &e.ihr, &e.imn, &e.sec, &xlat, &xlon,
                        &dep, evid);
            e.evid = evid;
            e.dpot = htoe(e.iyr, e.jday, e.ihr, e.imn, (double)e.sec);
            out.push_back(e);
            cur = &out.back();
            continue;
        }
        Phase p{};
        char sta[256] = "", rest[128] = "";
        std::sscanf(line, "%255s %d %d %d %d %f %99[^\n]", sta, &p.iyr, &p.jday, &p.ihr, &p.imn, &p.sec, rest);
        p.good = 1;
        if (rest[0] == '*') {
            p.good = 0;
            rest[0] = ' ';
            trim_tail(rest);
        }
        std::sscanf(rest, "%c %f", &p.phase, &p.rwt);
        if (p.phase == '0') p.phase = 'P';
        else if (p.phase == '1') p.phase = 'S';
        if (p.phase != 'P' && p.phase != 'S') {
            std::fclose(f);
            return FDGPU_EPAR;   /* the reference asserts */
        }
        p.sta = sta;
        p.pwt = 1.f / (p.rwt * p.rwt);
        const double tarr = htoe(p.iyr, p.jday, p.ihr, p.imn, (double)p.sec);
        p.obstime = (float)(tarr - cur->dpot);
        cur->ph.push_back(p);
    }
    std::fclose(f);
    return FDGPU_OK;
}

}  // namespace

namespace {

/* the default locator: the fields to the device, fdgpu_locate on a context of device 0 */
int gpu_locator(void *, const fdgpu_loc_grid *g, const float *const *h_fields, int nfields, int nev,
                const int *obs_offset, fdgpu_loc_obs *obs, float *resmin, float *tps, fdgpu_loc_result *results)
{
    fdgpu_ctx *ctx = nullptr;
    int rc = fdgpu_create(0, &ctx);
    if (rc) return rc;
    const size_t n = (size_t)g->nx * g->ny * g->nz;
    std::vector<float *> d(nfields, nullptr);
    for (int k = 0; k < nfields && rc == 0; k++)
        if (cudaMalloc(&d[k], n * sizeof(float)) != cudaSuccess ||
            cudaMemcpy(d[k], h_fields[k], n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
            rc = FDGPU_ECUDA;
    if (rc == 0)
        rc = fdgpu_locate(ctx, g, (const float *const *)d.data(), nfields, nev, obs_offset, obs, resmin, tps, results,
                          nullptr);
    for (float *p : d)
        if (p) cudaFree(p);
    fdgpu_destroy(ctx);
    return rc;
}

std::string fmt(const char *f, ...) __attribute__((format(printf, 1, 2)));
std::string fmt(const char *f, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, f);
    std::vsnprintf(buf, sizeof buf, f, ap);
    va_end(ap);
    return buf;
}

bool write_file(const std::string &path, const std::string &data)
{
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
    return std::fclose(f) == 0 && ok;
}

}  // namespace

extern "C" int fdgpu_sphfdloc(const char *specfile, fdgpu_loc_locator locator, void *user)
{
    if (!specfile) return FDGPU_EINVAL;
    Spec sp;
    if (!sp.load(specfile)) return FDGPU_EIO;
    for (const char *k : {"nxc", "nyc", "nzc", "h", "leqsfil", "fsumfil", "outlfil", "fhedfil", "fdatfil"})
        if (!sp.has(k)) return FDGPU_EPAR;
    int nxc = 0, nyc = 0, nzc = 0;
    double h = 0, x0 = 0, y0 = 0, z0 = 0;
    sp.get("nxc", "%d", &nxc);
    sp.get("nyc", "%d", &nyc);
    sp.get("nzc", "%d", &nzc);
    sp.get("h", "%lf", &h);
    sp.get("x0", "%lf", &x0);
    sp.get("y0", "%lf", &y0);
    sp.get("z0", "%lf", &z0);
    if (nxc < 2 || nyc < 2 || nzc < 2 || !(h > 0)) return FDGPU_EPAR;
    const std::vector<int> igx = sp.ints("igridx", nxc - 1), igy = sp.ints("igridy", nyc - 1),
                           igz = sp.ints("igridz", nzc - 1);
    if ((int)igx.size() != nxc - 1 || (int)igy.size() != nyc - 1 || (int)igz.size() != nzc - 1) return FDGPU_EPAR;
    int nx = 1, ny = 1, nz = 1;
    for (int v : igx) nx += v;
    for (int v : igy) ny += v;
    for (int v : igz) nz += v;

    /* the grid and the search parameters (:150-400), the reference's defaults where the spec is silent */
    fdgpu_loc_grid g;
    fdgpu_loc_grid_from_spec(&g, nx, ny, nz, x0, y0, z0, h);
    int ivs = 1, kmin = 0, ndiv = g.ndiv, ndiv2 = g.ndiv2;
    sp.get("ivs", "%d", &ivs);
    if (ivs != 0 && ivs != 1) ivs = 0;
    g.ivs = ivs;
    sp.get("vpvs", "%f", &g.vpvs);
    sp.get("nthres", "%d", &g.nthres);
    sp.get("resthres", "%f", &g.resthres);
    sp.get("resthrep", "%f", &g.resthrep);
    sp.get("stdmax", "%f", &g.stdmax);
    if (sp.has("kmin")) {
        sp.get("kmin", "%d", &kmin);
        g.kmin = kmin - 1;
    }
    sp.get("ndiv", "%d", &ndiv);
    g.ndiv = ndiv <= 0 ? 1 : ndiv;
    sp.get("ndiv2", "%d", &ndiv2);
    g.ndiv2 = ndiv2 <= 0 ? 1 : ndiv2;

    std::vector<LocEvent> events;
    int rc = read_events(sp.str("leqsfil"), events);
    if (rc) return rc;

    /* phases, and the time files they name (:627-640: "<station>.ptimes" or ".stimes" in timedir) */
    const std::string timedir = sp.str("timedir", "./ttimes");
    std::map<std::string, int> fidx;
    std::vector<std::string> files;
    std::vector<fdgpu_loc_obs> obs;
    std::vector<int> off(1, 0);
    for (const LocEvent &e : events) {
        for (const Phase &p : e.ph) {
            const std::string key = p.sta + (p.phase == 'P' ? ".ptimes" : ".stimes");
            auto it = fidx.find(key);
            if (it == fidx.end()) it = fidx.emplace(key, (int)files.size()).first, files.push_back(key);
            fdgpu_loc_obs o{};
            o.field = it->second;
            o.obstime = p.obstime;
            o.pwt = p.pwt;
            o.phase = p.phase;
            o.good = (char)p.good;
            obs.push_back(o);
        }
        off.push_back((int)obs.size());
    }
    const int nev = (int)events.size();
    for (int e = 0; e < nev; e++)
        if (off[e + 1] == off[e]) return FDGPU_EPAR;   /* an event without phases */
    const size_t n = (size_t)nx * ny * nz;
    std::vector<std::vector<float>> fields(files.size(), std::vector<float>(n));
    std::vector<const float *> fptr;
    for (size_t k = 0; k < files.size(); k++) {
        FILE *f = std::fopen((timedir + "/" + files[k]).c_str(), "rb");
        if (!f) return FDGPU_EIO;
        char head[4] = {0, 0, 0, 0};
        const size_t got = std::fread(head, 1, 4, f);
        std::fseek(f, (got == 4 && std::memcmp(head, "HEAD", 4) == 0) ? 232 : 0, SEEK_SET);
        const size_t rd = std::fread(fields[k].data(), sizeof(float), n, f);
        std::fclose(f);
        if (rd != n) return FDGPU_EIO;
        fptr.push_back(fields[k].data());
    }

    /* the search */
    std::vector<float> resmin(obs.size() + 1), tps(obs.size() + 1);
    std::vector<fdgpu_loc_result> res(nev + 1);
    if (nev > 0) {
        rc = (locator ? locator : gpu_locator)(user, &g, fptr.data(), (int)fptr.size(), nev, off.data(), obs.data(),
                                               resmin.data(), tps.data(), res.data());
        if (rc) return rc;
    }

    /* the reports (:1129-1250) */
    std::string fhd, dat, sum, out;
    for (int ev = 0; ev < nev; ev++) {
        const LocEvent &E = events[ev];
        const fdgpu_loc_result &r = res[ev];
        const int b = off[ev], nsta = off[ev + 1] - off[ev];
        const float xlon = (float)(r.exm / kDegrad);
        double ezmr = 0;
        const double lat = glathinv(kHpi - r.eym, g.z0r - (r.ezm - g.z0), &ezmr);
        const float xlat = (float)(lat / kDegrad);
        int iyr, jday, ihr, imn;
        double dsec;
        etoh(E.dpot + r.avrmin, &iyr, &jday, &ihr, &imn, &dsec);
        const float sec = (float)dsec;
        const double stdmin = r.stdmin;
        std::vector<float> res_dm(nsta);
        for (int i = 0; i < nsta; i++) res_dm[i] = resmin[b + i] - r.avrmin;
        const char *id = E.evid.c_str();
        if (r.status == 1) {
            if (std::isinf(r.stdmin))
                out += fmt("%4d %3d %2d %2d %8.4f %9.5f %10.5f %8.4f %12s    **********\n", iyr, jday, ihr, imn,
                           (double)sec, (double)xlat, (double)xlon, ezmr, id);
            else
                out += fmt("%4d %3d %2d %2d %8.4f %9.5f %10.5f %8.4f %12s %13.3f\n", iyr, jday, ihr, imn, (double)sec,
                           (double)xlat, (double)xlon, ezmr, id, stdmin);
            for (int j = 0; j < nsta; j++) {
                const Phase &p = E.ph[j];
                const float tarr = (float)(p.obstime + E.dpot);
                int y2, d2, h2, m2;
                double s2;
                etoh(tarr, &y2, &d2, &h2, &m2, &s2);
                out += fmt("%s %4d %3d %2d %2d %7.3f*%c %15.3f %10.3f\n", p.sta.c_str(), y2, d2, h2, m2, s2, p.phase,
                           (double)p.rwt, (double)res_dm[j]);
            }
            out += "\n";
            continue;
        }
        if (r.status != 0) continue;   /* stdmin above stdmax: nothing is written */
        const std::string line = fmt("%4d %3d %2d %2d %8.4f %9.5f %10.5f %8.4f %12s %13.3f\n", iyr, jday, ihr, imn,
                                     (double)sec, (double)xlat, (double)xlon, ezmr, id, stdmin);
        dat += line;
        fhd += line;
        if (r.ngood < nsta)
            out += fmt("%4d %3d %2d %2d %8.4f %9.5f %10.5f %8.4f %12s %13.3f\n", iyr, jday, ihr, imn, (double)sec,
                       r.exm, r.eym, ezmr, id, stdmin);
        sum += "\n\n";
        sum += fmt("  Minimum Standard Deviation   : %12.8f\n", stdmin);
        sum += fmt("  Info Density Maximum for event %12d\n", ev);
        sum += fmt("%4d %3d %2d %2d %8.4f  %8.5f %10.5f %8.4f %12s %13.3f\n", iyr, jday, ihr, imn, (double)sec, r.exm,
                   r.eym, ezmr, id, stdmin);
        sum += fmt(" Event ID: %7s\n", id);
        sum += fmt("  Minimum Standard Deviation   : %12.8f\n", stdmin);
        sum += "  Maximum Sigma                :   2.51547135E+15\n";
        sum += "  Total Sigma                  :    0.0000000    \n";
        sum += fmt("  Optimal Grid point (nx,ny,nz): %12d %11d %11d\n", r.nxx + 1, r.nyy + 1, r.nzz + 1);
        sum += fmt("  Average residual             :   %10.8f\n", (double)r.avrmin);
        sum += fmt("  Hypocenter (lat, lon ,z )    :   %12.3f  %12.3f  %12.3f\n\n", (double)xlat, (double)xlon, ezmr);
        sum += "  Station statistics at this point: \n";
        sum += " Code  Ph  Demeaned    True   Expected  Used   Tobs     Tcalc     To-Tc \n";
        sum += "           Residual   Weight   Uncert.  Flag    Abs      Abs     \n\n";
        for (int i = 0; i < nsta; i++) {
            const Phase &p = E.ph[i];
            const float wt = p.pwt;
            sum += fmt("%4s   %c %10.4f %9.3E %9.4f %3d %9.4f %9.4f %9.4f\n", p.sta.c_str(), p.phase, (double)res_dm[i],
                       (double)wt, 1.0 / std::sqrt(wt), (int)obs[b + i].good, (double)p.obstime, (double)tps[b + i],
                       (double)(float)(p.obstime - tps[b + i]));
        }
        sum += "\n";
        for (int j = 0; j < nsta; j++) {
            const Phase &p = E.ph[j];
            int y2, d2, h2, m2;
            double s2;
            etoh(p.obstime + E.dpot, &y2, &d2, &h2, &m2, &s2);
            const std::string t = fmt(obs[b + j].good ? "%-6s%4d %3d %2d %2d %7.3f %c %15.3f %10.3f\n"
                                                      : "%-6s%4d %3d %2d %2d %7.3f*%c %15.3f %10.3f\n",
                                      p.sta.c_str(), y2, d2, h2, m2, s2, p.phase, (double)p.rwt, (double)res_dm[j]);
            if (!obs[b + j].good) out += t;
            dat += t;
        }
        dat += " \n";
    }
    const bool ok = write_file(sp.str("fhedfil"), fhd) && write_file(sp.str("fdatfil"), dat) &&
                    write_file(sp.str("fsumfil"), sum) && write_file(sp.str("outlfil"), out);
    return ok ? FDGPU_OK : FDGPU_EIO;
}
