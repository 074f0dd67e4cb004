// Configuration text files in the reference's format, IO::SaveConfiguration
// (IO/SaveConfiguration.cpp:3-56) and IO::LoadConfiguration
// (IO/LoadConfiguration.cpp:3-120), for checkpoints exchanged with reference runs.
//
//   links:  "x y z mu v_0 v_1 ... v_{n-1} " per link (SU(2): the 4 quaternion
//           reals; SU(3): re and im of the 9 entries in storage order,
//           SUNc/SU{2,3}/GroupOperations.cpp MatrixToString), a trailing blank;
//   fields: "x y z mu e^0 ... e^{NA-1}" per link;
// both z-, y-, x-, mu-major as the reference loops, at 15 significant digits
// (OUTPUT_PRECISION = digits10, Definitions.cpp:21-22).  Host code only: the
// arrays are the reference's AoS layouts that tcym_lattice_upload/download take.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/tcym.h"
#include "tcym_internal.h"

namespace {

int reals_per_link(int nc) { return nc == 2 ? 4 : 18; }
int reals_per_field(int nc) { return nc == 2 ? 3 : 8; }

bool valid(int nc, int nx, int ny, int nz) { return (nc == 2 || nc == 3) && nx > 0 && ny > 0 && nz > 0; }

int write_file(const char *path, const std::string &text) {
    std::FILE *f = std::fopen(path, "wb");
    if (!f) return TCYM_ERR_ARG;
    const size_t n = std::fwrite(text.data(), 1, text.size(), f);
    const int closed = std::fclose(f);
    return (n == text.size() && closed == 0) ? TCYM_OK : TCYM_ERR_ARG;
}

bool read_file(const char *path, std::string &text) {
    std::ifstream in(path, std::ios::binary);
    if (!in) return false;
    std::ostringstream ss;
    ss << in.rdbuf();
    text = ss.str();
    return true;
}

// One record per non-empty line: four integers then `n` reals.  Fills out[]
// at the record's (site, mu); each link exactly once.
int parse(const std::string &text, int n, int nx, int ny, int nz, double *out, const char *what) {
    const int64_t V = (int64_t)nx * ny * nz;
    std::vector<unsigned char> seen((size_t)(3 * V), 0);
    int64_t count = 0;
    const char *p = text.c_str(), *end = p + text.size();
    while (p < end) {
        const char *eol = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
        if (!eol) eol = end;
        std::string line(p, eol);
        p = eol + 1;
        size_t k = 0;
        while (k < line.size() && (line[k] == ' ' || line[k] == '\t' || line[k] == '\r')) ++k;
        if (k == line.size()) continue;  // empty line
        const char *s = line.c_str();
        char *q = nullptr;
        long c[4];
        for (int i = 0; i < 4; ++i) {
            errno = 0;
            c[i] = std::strtol(s, &q, 10);
            if (q == s || errno) {
                std::fprintf(stderr, "tcym: %s file: bad coordinates in \"%s\"\n", what, line.c_str());
                return TCYM_ERR_ARG;
            }
            s = q;
        }
        if (c[0] < 0 || c[0] >= nx || c[1] < 0 || c[1] >= ny || c[2] < 0 || c[2] >= nz || c[3] < 0 || c[3] > 2) {
            std::fprintf(stderr, "tcym: %s file: link outside the lattice in \"%s\"\n", what, line.c_str());
            return TCYM_ERR_ARG;
        }
        const int64_t link = 3 * (c[0] + (int64_t)nx * (c[1] + (int64_t)ny * c[2])) + c[3];
        for (int i = 0; i < n; ++i) {
            errno = 0;
            const double v = std::strtod(s, &q);
            if (q == s || errno == ERANGE) {
                std::fprintf(stderr, "tcym: %s file: expected %d values in \"%s\"\n", what, n, line.c_str());
                return TCYM_ERR_ARG;
            }
            out[link * n + i] = v;
            s = q;
        }
        if (seen[(size_t)link]++) {
            std::fprintf(stderr, "tcym: %s file: link given twice in \"%s\"\n", what, line.c_str());
            return TCYM_ERR_ARG;
        }
        ++count;
    }
    if (count != 3 * V) {
        std::fprintf(stderr, "tcym: %s file: %lld of %lld links present\n", what, (long long)count,
                     (long long)(3 * V));
        return TCYM_ERR_ARG;
    }
    return TCYM_OK;
}

std::string format(int n, int nx, int ny, int nz, const double *in, bool trailing_blank) {
    std::ostringstream os;
    os.precision(15);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x)
                for (int mu = 0; mu < 3; ++mu) {
                    const int64_t link = 3 * (x + (int64_t)nx * (y + (int64_t)ny * z)) + mu;
                    os << x << " " << y << " " << z << " " << mu;
                    for (int i = 0; i < n; ++i) os << " " << in[link * n + i];
                    os << (trailing_blank ? " \n" : "\n");
                }
    return os.str();
}

}  // namespace

extern "C" int tcym_write_configuration(int nc, int nx, int ny, int nz, const double *U_aos, const double *E_aos,
                                        const char *ufile, const char *efile) {
    if (!valid(nc, nx, ny, nz) || (ufile && !U_aos) || (efile && !E_aos)) return TCYM_ERR_ARG;
    int r = TCYM_OK;
    if (ufile && (r = write_file(ufile, format(reals_per_link(nc), nx, ny, nz, U_aos, true)))) return r;
    if (efile && (r = write_file(efile, format(reals_per_field(nc), nx, ny, nz, E_aos, false)))) return r;
    return TCYM_OK;
}

extern "C" int tcym_read_configuration(int nc, int nx, int ny, int nz, double *U_aos, double *E_aos,
                                       const char *ufile, const char *efile) {
    if (!valid(nc, nx, ny, nz) || (ufile && !U_aos) || (efile && !E_aos)) return TCYM_ERR_ARG;
    std::string text;
    int r;
    if (ufile) {
        if (!read_file(ufile, text)) return TCYM_ERR_ARG;
        if ((r = parse(text, reals_per_link(nc), nx, ny, nz, U_aos, "link"))) return r;
    }
    if (efile) {
        if (!read_file(efile, text)) return TCYM_ERR_ARG;
        if ((r = parse(text, reals_per_field(nc), nx, ny, nz, E_aos, "field"))) return r;
    }
    return TCYM_OK;
}

extern "C" int tcym_lattice_save(tcym_lattice lat, const char *ufile, const char *efile) {
    if (!lat) return TCYM_ERR_ARG;
    const size_t links = 3 * (size_t)lat->g.V;
    std::vector<double> U(ufile ? links * reals_per_link(lat->nc) : 0), E(efile ? links * reals_per_field(lat->nc) : 0);
    int r = tcym_lattice_download(lat, ufile ? U.data() : nullptr, efile ? E.data() : nullptr);
    if (r) return r;
    r = tcym_write_configuration(lat->nc, lat->g.nx, lat->g.ny, lat->g.nz, U.data(), E.data(), ufile, efile);
    if (r) tcym_set_error(lat->ctx, "tcym_lattice_save: cannot write the configuration files");
    return r;
}

extern "C" int tcym_lattice_load(tcym_lattice lat, const char *ufile, const char *efile) {
    if (!lat) return TCYM_ERR_ARG;
    const size_t links = 3 * (size_t)lat->g.V;
    std::vector<double> U(ufile ? links * reals_per_link(lat->nc) : 0), E(efile ? links * reals_per_field(lat->nc) : 0);
    int r = tcym_read_configuration(lat->nc, lat->g.nx, lat->g.ny, lat->g.nz, U.data(), E.data(), ufile, efile);
    if (r) {
        tcym_set_error(lat->ctx, "tcym_lattice_load: unreadable or incomplete configuration files");
        return r;
    }
    return tcym_lattice_upload(lat, ufile ? U.data() : nullptr, efile ? E.data() : nullptr);
}
