// rans::save (post.h:58-180): the ASCII VTU file of a state on a mesh.
//
// The text is the reference's, byte for byte: the same elements, the same
// indentation (including the connectivity block's trailing indent before
// its closing tag), integer separators of two spaces, node coordinates as
// std::to_string formats them ("%f") and cell data in fixed notation with
// 16 digits (both through std::to_chars, which gives printf's text).  The
// derived fields follow solution (core.h:119-164) with the same operand
// order.
//
// The reference appends every number to one std::string through a
// stringstream.  Here each block is formatted by OpenMP threads into
// per-chunk buffers over fixed row ranges and written in row order, so the
// bytes do not depend on the thread count.
#include <omp.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "afx_host.hpp"

namespace afx {
namespace {

// printf-style append (a heap buffer when the text is long, e.g. huge values
// in fixed notation)
void app(std::string& s, const char* fmt, ...) {
    char buf[128];
    va_list ap;
    va_start(ap, fmt);
    const int k = std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (k < 0) throw Error(1, "vtu: formatting failed");
    if (k < (int)sizeof(buf)) {
        s.append(buf, (size_t)k);
        return;
    }
    std::vector<char> big((size_t)k + 1);
    va_start(ap, fmt);
    std::vsnprintf(big.data(), big.size(), fmt, ap);
    va_end(ap);
    s.append(big.data(), (size_t)k);
}

// x in fixed notation with prec digits: std::to_chars gives printf's text
// ("%.*f": exact binary value, correctly rounded), several times faster
void fixed(std::string& s, double x, int prec) {
    char buf[400];  // sign + 309 integer digits + point + 16 digits fit
    const auto r = std::to_chars(buf, buf + sizeof(buf), x, std::chars_format::fixed, prec);
    if (r.ec != std::errc()) throw Error(1, "vtu: formatting failed");
    s.append(buf, (size_t)(r.ptr - buf));
}
void uint_(std::string& s, unsigned v) {
    char buf[16];
    const auto r = std::to_chars(buf, buf + sizeof(buf), v);
    s.append(buf, (size_t)(r.ptr - buf));
}

struct File {
    std::FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
    void put(const std::string& s) {
        if (!s.empty() && std::fwrite(s.data(), 1, s.size(), f) != s.size()) throw Error(1, "vtu: write failed");
    }
};

// rows [0, n) formatted by fmt(i, out), written in row order; chunks of rows
// are formatted in parallel, a bounded number of chunks at a time
template <class F>
void rows(File& out, long long n, F fmt) {
    const long long chunk = 1 << 14;
    const long long nch = (n + chunk - 1) / chunk;
    const long long group = std::max(1, 4 * omp_get_max_threads());
    std::vector<std::string> buf;
    for (long long g0 = 0; g0 < nch; g0 += group) {
        const long long g1 = std::min(nch, g0 + group);
        buf.assign((size_t)(g1 - g0), std::string());
#pragma omp parallel for schedule(dynamic, 1)
        for (long long c = g0; c < g1; ++c) {
            std::string& s = buf[(size_t)(c - g0)];
            s.reserve((size_t)chunk * 24);
            const long long i1 = std::min(n, (c + 1) * chunk);
            for (long long i = c * chunk; i < i1; ++i) fmt(i, s);
        }
        for (const std::string& s : buf) out.put(s);
    }
}

}  // namespace

void write_vtu(const HostMesh& m, const double* q, const double* wall_dist, double gamma, double R,
               const std::string& path) {
    File out;
    out.f = std::fopen(path.c_str(), "wb");
    if (!out.f) throw Error(1, "cannot write " + path);
    const long long nn = (long long)m.nodesX.size(), nc = (long long)m.nRealCells;
    std::string h;
    h += "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n";
    h += "  <UnstructuredGrid>\n";
    app(h, "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", nn, nc);
    h += "      <Points>\n";
    h += "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n";
    out.put(h);
    rows(out, nn, [&](long long i, std::string& s) {
        s += "          ";
        fixed(s, m.nodesX[i], 6);
        s += ' ';
        fixed(s, m.nodesY[i], 6);
        s += " 0.0\n";
    });
    out.put("        </DataArray>\n"
            "      </Points>\n"
            "      <Cells>\n"
            "        <DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n"
            "          ");
    rows(out, nc, [&](long long i, std::string& s) {
        const int k = m.cellsIsTriangle[i] ? 3 : 4;
        for (int j = 0; j < k; ++j) {
            uint_(s, (unsigned)m.cellsNodes[i][j]);
            s += "  ";
        }
        s += "\n          ";
    });
    out.put("        </DataArray>\n"
            "        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n"
            "          ");
    std::vector<unsigned> off((size_t)nc);
    unsigned acc = 0;
    for (long long i = 0; i < nc; ++i) off[i] = acc += m.cellsIsTriangle[i] ? 3u : 4u;
    rows(out, nc, [&](long long i, std::string& s) {
        uint_(s, off[i]);
        s += "  ";
    });
    out.put("\n"
            "        </DataArray>\n"
            "        <DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n"
            "          ");
    rows(out, nc, [&](long long i, std::string& s) { s += m.cellsIsTriangle[i] ? "5  " : "9  "; });
    out.put("\n"
            "        </DataArray>\n"
            "      </Cells>\n"
            "      <CellData Scalars=\"scalars\">\n");
    auto block = [&](const char* name, auto value) {
        std::string t = "        <DataArray type=\"Float32\" Name=\"";
        t += name;
        t += "\" Format=\"ascii\">\n";
        out.put(t);
        rows(out, nc, [&](long long i, std::string& s) {
            s += "          ";
            fixed(s, value(i), 16);
            s += '\n';
        });
        out.put("        </DataArray>\n");
    };
    // solution (core.h:119-164)
    auto rho = [&](long long i) { return q[4 * i]; };
    auto rhou = [&](long long i) { return q[4 * i + 1]; };
    auto rhov = [&](long long i) { return q[4 * i + 2]; };
    auto rhoe = [&](long long i) { return q[4 * i + 3]; };
    auto p = [&](long long i) {
        return (gamma - 1) * (rhoe(i) - 0.5 / rho(i) * (rhou(i) * rhou(i) + rhov(i) * rhov(i)));
    };
    auto c = [&](long long i) { return std::sqrt(gamma * p(i) / rho(i)); };
    block("Wall Distance", [&](long long i) { return wall_dist ? wall_dist[i] : 0.0; });
    block("Mach", [&](long long i) { return std::sqrt(rhou(i) * rhou(i) + rhov(i) * rhov(i)) / (rho(i) * c(i)); });
    block("Density", rho);
    block("Pressure", p);
    block("Temperature", [&](long long i) { return p(i) / (R * rho(i)); });
    out.put("        <DataArray type=\"Float32\" Name=\"Velocity\" NumberOfComponents=\"3\" Format=\"ascii\">\n");
    rows(out, nc, [&](long long i, std::string& s) {
        s += "          ";
        fixed(s, rhou(i) / rho(i), 16);
        s += ' ';
        fixed(s, rhov(i) / rho(i), 16);
        s += " 0.0\n";
    });
    out.put("        </DataArray>\n"
            "      </CellData>\n"
            "    </Piece>\n"
            "  </UnstructuredGrid>\n"
            "</VTKFile>");
    if (std::fflush(out.f) != 0) throw Error(1, "vtu: write failed");
}

}  // namespace afx
