/* sphrayderv's driver around the device rays (reference src/sphrayderv.c main): the spec, station and
 * event files read as the reference reads them, the observations handed to a tracer (fdgpu_raytrace by
 * default), and the six inversion files written from the results with the reference's bookkeeping.
 *
 * The bookkeeping is the reference's own state, kept across events: the per-event unknown numbering
 * (kbl, mhit, mndex, mndm: reset only when an event's first phase reaches its station,
 * :1565-1569), the run-wide hit index (mbl, nhit, indx, jndx, :1578-1595), and the per-event matrix
 * vmp (zeroed only for the event's first kbl rows, :2262-2268).  Local earthquakes only (ivpvs 0,
 * nomat 0); the data-out, error-summary and log texts are not written. */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/fdgpu.h"

namespace {

const double kDegrad = 0.017453292f;   /* src/sphrayderv.c:84: float literals */
const double kHpi = 1.570796f;
const float kRearthF = 6371.0f;

/* geographic -> geocentric latitude (lib/common/geographic_method.c:7-16) */
double glat(double hlat)
{
    const double halfpi = 1.570796f, polfac = 0.010632f, elfac = 0.993277f;
    if (halfpi - std::fabs(hlat) >= (double)0.05) return std::atan(elfac * std::sin(hlat) / std::cos(hlat));
    return hlat / elfac - std::fabs(polfac) * (hlat >= 0 ? 1 : -1);
}

int isleap(int y) { return (y % 4 == 0 && y % 100 != 0) || y % 400 == 0 ? 1 : 0; }

/* epoch seconds (lib/common/time_process.c:85-109) */
double htoe(int iyear, int iday, int ihour, int imin, double sec)
{
    int days = 0;
    if (iyear > 1970)
        for (int i = 1970; i < iyear; i++) days += 365 + isleap(i);
    else if (iyear < 1970)
        for (int i = iyear; i <= 1969; i++) days -= 365 + isleap(i);
    days += iday - 1;
    double e = (double)(days * 24 * 60 * 60);
    return e + 3600.0 * ihour + 60.0 * imin + sec;
}

/* leading and trailing blanks off */
std::string trim(const char *s)
{
    size_t b = 0, e = std::strlen(s);
    while (b < e && (s[b] == ' ' || s[b] == '\t' || s[b] == '\n' || s[b] == '\r')) b++;
    while (e > b && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\n' || s[e - 1] == '\r')) e--;
    return std::string(s + b, e - b);
}

/* spec variables, get_vars style (lib/common/parseprogs.c:9-79): the first line whose first field
 * is the name; its fields after the name */
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
            v.emplace(key, std::move(fields));   /* the first definition stays */
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
    int i(const char *k, int dflt) const
    {
        int x = dflt;
        if (has(k)) std::sscanf(str(k).c_str(), "%d", &x);
        return x;
    }
    double d(const char *k, double dflt) const
    {
        double x = dflt;
        if (has(k)) std::sscanf(str(k).c_str(), "%lf", &x);
        return x;
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

struct Station {
    std::string name;
    double xs, ys, zs;
    float tc[2];
};

struct Pick {
    std::string sta;
    int iyr, jday, ihr, imn;
    float sec;
    char phase;
    float rwt;
};

struct Event {
    int kyr, kday, khr, kmn;
    float esec;
    double xlat, xlon;
    float dep;
    std::vector<Pick> picks;
};

/* station list (:818-851) */
bool read_stations(const std::string &path, std::vector<Station> &out)
{
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    char line[1024], name[256];
    while (std::fgets(line, sizeof line, f)) {
        if (trim(line).empty()) break;
        double sty = 0, stx = 0;
        int ielev = 0;
        float slat = 0, slon = 0, tc0 = 0, tc1 = 0;
        if (std::sscanf(line, "%lf %lf %d %255s %f %f %f %f", &sty, &stx, &ielev, name, &slat, &slon, &tc0, &tc1) < 8)
            break;
        stx = slon;
        sty = slat;
        Station s;
        s.name = name;
        s.xs = (float)(stx * kDegrad);
        s.ys = (float)(kHpi - glat(sty * kDegrad));
        s.zs = -(float)(ielev / 1000.f);
        s.tc[0] = tc0;
        s.tc[1] = tc1;
        out.push_back(s);
    }
    std::fclose(f);
    return true;
}

/* local earthquake file (:880-1048): a header line per event, one line per phase, a blank line */
bool read_events(const std::string &path, std::vector<Event> &out)
{
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    char line[1024];
    Event *cur = nullptr;
    while (std::fgets(line, sizeof line, f)) {
        const std::string t = trim(line);
        if (t.empty()) {
            cur = nullptr;
            continue;
        }
        if (!cur) {
            Event e{};
            char evid[256];
            std::sscanf(line, "%d %d %d %d %f %lf %lf %f %255s", &e.kyr, &e.kday, &e.khr, &e.kmn, &e.esec, &e.xlat,
                        &e.xlon, &e.dep, evid);
            out.push_back(e);
            cur = &out.back();
            continue;
        }
        Pick p{};
        char sta[256], rest[256] = "", ph[8] = "";
        std::sscanf(t.c_str(), "%255s %d %d %d %d %f %99[^\n]", sta, &p.iyr, &p.jday, &p.ihr, &p.imn, &p.sec, rest);
        if (rest[0] == '*') rest[0] = ' ';
        std::sscanf(rest, " %c %f", ph, &p.rwt);
        p.sta = sta;
        p.phase = ph[0] == '0' ? 'P' : ph[0] == '1' ? 'S' : ph[0];
        cur->picks.push_back(p);
    }
    std::fclose(f);
    return true;
}

/* the reference's bookkeeping and its six files */
struct Assembler {
    int maxvarc;
    std::vector<char> mhit;
    std::vector<long long> mndex, nhit, indx;
    std::vector<int> mndm, jndx;
    int kbl = 0, nev = 0;
    std::unordered_map<long long, float> vmp;
    std::unordered_map<int, float> dat;
    std::string dts, res, dth, bok;

    explicit Assembler(int nxyzc)
        : maxvarc(nxyzc), mhit(2 * (size_t)nxyzc + 8, 0), mndex(2 * (size_t)nxyzc + 8, 0), nhit(2 * (size_t)nxyzc + 8, 0),
          indx(2 * (size_t)nxyzc + 8, 0), mndm(2 * (size_t)nxyzc + 8, 0)
    {
    }

    static long long key(long long jnd, long long k) { return (jnd << 24) | k; }

    void put_i(std::string &s, int v) { s.append(reinterpret_cast<const char *>(&v), 4); }
    void put_f(std::string &s, float v) { s.append(reinterpret_cast<const char *>(&v), 4); }

    /* rows[i] = (observation index or -1, phase index) */
    void event(bool inside, const std::vector<std::pair<int, int>> &rows, const fdgpu_ray_result *r,
               const long long *off, const int *idx, const float *du)
    {
        nev++;
        if (!inside) return;
        const int nsta = (int)rows.size();
        std::vector<int> isgood(nsta, 0), inbk(nsta, 0);
        std::map<std::pair<int, int>, float> vm;
        std::map<std::pair<int, int>, int> ind;
        std::map<int, const float *> am;
        for (int i = 0; i < nsta; i++) {
            const int o = rows[i].first, iph = rows[i].second;
            if (o < 0) continue;
            isgood[i] = 1;
            if (r[o].status != FDGPU_RAY_OK) {
                isgood[i] = 0;
                continue;
            }
            if (i == 0) {
                kbl = 0;
                std::fill(mhit.begin(), mhit.end(), 0);
            }
            const float wet = r[o].wet;
            dat[i] = (float)(r[o].dt * wet);
            am[i] = r[o].am;
            int nbk = 0;
            for (long long q = off[o]; q < off[o] + r[o].nnz; q++) {
                const int j = idx[q] + (iph == 1 ? maxvarc : 0);
                vm[{nbk, i}] = du[q] * wet;
                ind[{nbk, i}] = j;
                nbk++;
                if (!mhit[j]) {
                    mndm[kbl] = j;
                    mndex[j] = kbl;
                    mhit[j] = 1;
                    kbl++;
                }
                if (nhit[j] == 0) {
                    indx[j] = (long long)jndx.size();
                    jndx.push_back(j);
                }
                nhit[j]++;
            }
            inbk[i] = nbk;
        }
        for (int j1 = 0; j1 < nsta; j1++)
            for (int j2 = 0; j2 < kbl; j2++) {
                auto it = vmp.find(key(j2, j1));
                if (it != vmp.end()) it->second = 0.0f;
            }
        for (int k = 0; k < nsta; k++)
            if (isgood[k])
                for (int j1 = 0; j1 < inbk[k]; j1++) {
                    const long long jnd = mndex[ind[{j1, k}]];
                    float &cell = vmp[key(jnd, k)];
                    cell = cell + vm[{j1, k}];
                }
        int nwrt = 0;
        for (int j1 = 0; j1 < nsta; j1++) {
            if (!isgood[j1]) continue;
            std::vector<int> ja;
            for (int i1 = 0; i1 < kbl; i1++) {
                auto it = vmp.find(key(i1, j1));
                if (it != vmp.end() && it->second != 0) ja.push_back(i1);
            }
            if (ja.empty()) continue;
            put_i(dts, (int)ja.size());
            for (int i1 : ja) {
                put_i(dts, (int)indx[mndm[i1]] + 1);
                put_f(dts, vmp[key(i1, j1)]);
            }
            put_f(res, dat[j1]);
            char buf[64];
            for (int q = 0; q < 4; q++) {
                std::snprintf(buf, sizeof buf, "%f\n", (double)am[j1][q]);
                dth += buf;
            }
            nwrt++;
        }
        char buf[64];
        std::snprintf(buf, sizeof buf, "%d %d\n", nev, nwrt);
        bok += buf;
    }
};

}  // namespace

namespace {

/* the default tracer: the fields to the device, fdgpu_raytrace on a context of device 0 */
int gpu_tracer(void *, const fdgpu_ray_grid *g, const float *const *h_fields, int nfields, int nobs,
               const fdgpu_ray_obs *obs, fdgpu_ray_result *res, long long *off, int *idx, float *du,
               long long total_cap)
{
    fdgpu_ctx *ctx = nullptr;
    int rc = fdgpu_create(0, &ctx);
    if (rc) return rc;
    const size_t n = (size_t)g->nx * g->ny * g->nz;
    std::vector<float *> d(nfields, nullptr);
    for (int k = 0; k < nfields && rc == 0; k++) {
        if (cudaMalloc(&d[k], n * sizeof(float)) != cudaSuccess ||
            cudaMemcpy(d[k], h_fields[k], n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
            rc = FDGPU_ECUDA;
    }
    if (rc == 0)
        rc = fdgpu_raytrace(ctx, g, (const float *const *)d.data(), nfields, nobs, obs, 0, 0, res, off, idx, du,
                            total_cap, nullptr);
    for (float *p : d)
        if (p) cudaFree(p);
    fdgpu_destroy(ctx);
    return rc;
}

bool write_file(const std::string &path, const std::string &data)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
    return std::fclose(f) == 0 && ok;
}

}  // namespace

extern "C" int fdgpu_sphrayderv(const char *specfile, int spacing_rule, fdgpu_ray_tracer tracer, void *user)
{
    if (!specfile) return FDGPU_EINVAL;
    Spec sp;
    if (!sp.load(specfile)) return FDGPU_EIO;
    for (const char *k : {"nxc", "nyc", "nzc", "h", "stafile", "locdfil", "dtdsfil", "resfile", "hitfile", "dtdhfil",
                          "bookfil", "sclefil"})
        if (!sp.has(k)) return FDGPU_EPAR;
    if (sp.i("ivpvs", 0) == 1 || sp.i("dotel", 0) == 1 || sp.i("doshot", 0) == 1 || sp.i("nomat", 0) == 1)
        return FDGPU_EINVAL;   /* local earthquakes only */
    int ivs = sp.i("ivs", 1);
    if (ivs != 0 && ivs != 1) ivs = 0;
    const int nxc = sp.i("nxc", 0), nyc = sp.i("nyc", 0), nzc = sp.i("nzc", 0);
    const double h = sp.d("h", 0);
    if (nxc < 2 || nyc < 2 || nzc < 2 || !(h > 0)) return FDGPU_EPAR;
    const std::vector<int> igx = sp.ints("igridx", nxc - 1), igy = sp.ints("igridy", nyc - 1),
                           igz = sp.ints("igridz", nzc - 1);
    if ((int)igx.size() != nxc - 1 || (int)igy.size() != nyc - 1 || (int)igz.size() != nzc - 1) return FDGPU_EPAR;

    /* the grid (:470-525, :779-788) */
    int nx = 1, ny = 1, nz = 1;
    for (int v : igx) nx += v;
    for (int v : igy) ny += v;
    for (int v : igz) nz += v;
    const double x0 = sp.d("x0", 0) * kDegrad;
    const double y0 = kHpi - glat(sp.d("y0", 0) * kDegrad);
    const double z0 = sp.d("z0", 0);
    double dq = sp.d("dq", 0) * kDegrad, df = sp.d("df", 0) * kDegrad;
    if (std::fabs(dq) < 0.0001 && (spacing_rule || dq == 0)) dq = h / kRearthF;
    if (std::fabs(df) < 0.0001 && (spacing_rule || df == 0)) df = std::fabs(h / (kRearthF * std::sin(y0)));
    std::vector<float> gx(nxc), gy(nyc), gz(nzc);
    gx[0] = x0;
    gy[0] = y0;
    gz[0] = z0;
    for (int q = 1; q < nxc; q++) gx[q] = gx[q - 1] + df * igx[q - 1];
    for (int q = 1; q < nyc; q++) gy[q] = gy[q - 1] + dq * igy[q - 1];
    for (int q = 1; q < nzc; q++) gz[q] = gz[q - 1] + h * igz[q - 1];
    fdgpu_ray_grid g{nx, ny, nz, nxc, nyc, nzc, x0, y0, z0, h, dq, df, gx.data(), gy.data(), gz.data()};

    std::vector<Station> stations;
    std::vector<Event> events;
    if (!read_stations(sp.str("stafile"), stations) || !read_events(sp.str("locdfil"), events)) return FDGPU_EIO;
    std::map<std::string, int> by_name;
    for (int k = 0; k < (int)stations.size(); k++) by_name.emplace(stations[k].name, k);

    /* observations of the events inside the model, and the time fields they need */
    std::vector<fdgpu_ray_obs> obs;
    std::vector<std::pair<bool, std::vector<std::pair<int, int>>>> plan;
    std::vector<std::string> files;
    std::map<std::string, int> fidx;
    const std::string timedir = sp.str("timedir", "./ttimes");
    for (const Event &e : events) {
        const double ex = e.xlon * kDegrad, ey = kHpi - glat(e.xlat * kDegrad), ez = e.dep;
        const int ies = (int)((ex - x0) / df), jes = (int)((ey - y0) / dq), kes = (int)((ez - z0) / h);
        const bool inside = !((ex < x0 || ies >= nx - 1) || (ey < y0 || jes >= ny - 1) || (ez < z0 || kes >= nz - 1));
        std::vector<std::pair<int, int>> rows;
        if (inside) {
            const double dpot = htoe(e.kyr, e.kday, e.khr, e.kmn, e.esec);
            for (const Pick &p : e.picks) {
                const int iph = p.phase == 'S' ? 1 : 0;
                auto st = by_name.find(p.sta);
                if (st == by_name.end()) {
                    rows.emplace_back(-1, iph);
                    continue;
                }
                const Station &s = stations[st->second];
                const std::string file = timedir + "/" + p.sta + ((p.phase == 'P' || ivs == 0) ? ".ptimes" : ".stimes");
                auto fi = fidx.find(file);
                if (fi == fidx.end()) fi = fidx.emplace(file, (int)files.size()).first, files.push_back(file);
                const double tarr = htoe(p.iyr, p.jday, p.ihr, p.imn, p.sec);
                fdgpu_ray_obs o{};
                o.ex = ex;
                o.ey = ey;
                o.ez = ez;
                o.xs = s.xs;
                o.ys = s.ys;
                o.zs = s.zs;
                o.field = fi->second;
                o.phase = iph;
                o.obstime = (float)(tarr - dpot);
                o.pwt = 1.f / (p.rwt * p.rwt);
                o.tc = s.tc[iph];
                rows.emplace_back((int)obs.size(), iph);
                obs.push_back(o);
            }
        }
        plan.emplace_back(inside, rows);
    }

    /* the time files (:1160-1218): a 232-byte header when the file starts with HEAD */
    const size_t n = (size_t)nx * ny * nz;
    std::vector<std::vector<float>> fields(files.size(), std::vector<float>(n));
    std::vector<const float *> fptr;
    for (size_t k = 0; k < files.size(); k++) {
        FILE *f = std::fopen(files[k].c_str(), "rb");
        if (!f) return FDGPU_EIO;
        char head[4] = {0, 0, 0, 0};
        const size_t got = std::fread(head, 1, 4, f);
        std::fseek(f, (got == 4 && std::memcmp(head, "HEAD", 4) == 0) ? 232 : 0, SEEK_SET);
        const size_t rd = std::fread(fields[k].data(), sizeof(float), n, f);
        std::fclose(f);
        if (rd != n) return FDGPU_EIO;
        fptr.push_back(fields[k].data());
    }

    /* the rays */
    const int nobs = (int)obs.size();
    std::vector<fdgpu_ray_result> res(nobs > 0 ? nobs : 1);
    std::vector<long long> off((size_t)nobs + 1, 0);
    long long total_cap = 192ll * (nobs > 0 ? nobs : 1);
    std::vector<int> idx;
    std::vector<float> du;
    if (!tracer) tracer = gpu_tracer;
    for (int attempt = 0; nobs > 0; attempt++) {
        idx.assign((size_t)total_cap, 0);
        du.assign((size_t)total_cap, 0.f);
        const int rc = tracer(user, &g, fptr.data(), (int)fptr.size(), nobs, obs.data(), res.data(), off.data(),
                              idx.data(), du.data(), total_cap);
        if (rc == FDGPU_ETOOBIG && attempt == 0 && off[nobs] > total_cap) {
            total_cap = off[nobs];
            continue;
        }
        if (rc) return rc;
        break;
    }

    /* the files */
    Assembler A(nxc * nyc * nzc);
    for (const auto &pl : plan) A.event(pl.first, pl.second, res.data(), off.data(), idx.data(), du.data());
    const int mbl = (int)A.jndx.size();
    A.put_i(A.dts, -1);
    A.put_i(A.dts, mbl);
    for (int j : A.jndx) A.put_i(A.dts, j);
    std::string msc, hit;
    char buf[64];
    std::snprintf(buf, sizeof buf, "%d\n", mbl);
    msc = buf;
    std::snprintf(buf, sizeof buf, "%d", mbl);
    hit = buf;
    for (int j : A.jndx) {
        std::snprintf(buf, sizeof buf, "%d\n", j);
        msc += buf;
        std::snprintf(buf, sizeof buf, "%d %lld\n", j, A.nhit[j]);
        hit += buf;
    }
    A.bok += "-2 -2\n";
    const bool ok = write_file(sp.str("dtdsfil"), A.dts) && write_file(sp.str("resfile"), A.res) &&
                    write_file(sp.str("dtdhfil"), A.dth) && write_file(sp.str("bookfil"), A.bok) &&
                    write_file(sp.str("sclefil"), msc) && write_file(sp.str("hitfile"), hit);
    return ok ? FDGPU_OK : FDGPU_EIO;
}
