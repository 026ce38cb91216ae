// Mesh load, finite-volume metrics and the GPU layout of the rans library.
//
// The numbering reproduces AeroFLEX's mesh class exactly (edges numbered in
// the order cells first meet them, mesh.h:317-341; second cell = the last
// other cell to list the edge, mesh.h:344-375; ghosts appended per boundary
// edge, mesh.h:744-787), and the metrics use the reference's formulas in the
// same operand order (mesh.h:378-453), so every FP64 metric is bit-identical
// to the reference's definition.  The edge build itself is a stable radix
// sort of half-edges instead of the reference's std::map, which keeps the
// 4.2M-cell channel mesh to well under a second.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <unordered_map>

#include "afx_host.hpp"

namespace afx {

// ------------------------------------------------------------- gmsh 4.1
namespace {

struct LineReader {
    std::string buf;
    size_t pos = 0;
    bool next(const char*& b, const char*& e) {
        if (pos >= buf.size()) return false;
        size_t nl = buf.find('\n', pos);
        if (nl == std::string::npos) nl = buf.size();
        b = buf.data() + pos;
        e = buf.data() + nl;
        if (e > b && e[-1] == '\r') --e;
        pos = nl + 1;
        return true;
    }
};

// Space-separated tokens; integers read like std::stoi (leading integer part).
struct Tok {
    const char* p;
    const char* e;
    bool next(const char*& tb, const char*& te) {
        while (p < e && *p == ' ') ++p;
        if (p >= e) return false;
        tb = p;
        while (p < e && *p != ' ') ++p;
        te = p;
        return true;
    }
};

long tok_int(const char* b, const char* e) {
    std::string s(b, e);
    char* end = nullptr;
    long v = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str()) throw Error(3, "gmsh: expected an integer, got '" + s + "'");
    return v;
}

double tok_double(const char* b, const char* e) {
    std::string s(b, e);
    char* end = nullptr;
    double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str()) throw Error(3, "gmsh: expected a number, got '" + s + "'");
    return v;
}

std::vector<long> ints(const char* b, const char* e) {
    std::vector<long> v;
    Tok t{b, e};
    const char *tb, *te;
    while (t.next(tb, te)) v.push_back(tok_int(tb, te));
    return v;
}

}  // namespace

// One pass with the semantics of read_entities / read_nodes /
// read_boundaries / read_elements (mesh.h:457-738).
HostMesh load_gmsh(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(1, "cannot open mesh file " + path);
    LineReader lr;
    {
        std::ostringstream ss;
        ss << f.rdbuf();
        lr.buf = ss.str();
    }
    HostMesh m;
    std::map<uint32_t, std::string> physicalNames;
    std::map<uint32_t, uint32_t> entityPhys;
    std::unordered_map<uint32_t, uint32_t> nodeRef;
    std::vector<uint32_t> bndTag;
    std::string section;
    long ns = 0, nss = 0, node_nss = 0;
    long n_points = 0, n_curves = 0;
    long node_start = 0, node_n = 0;
    std::vector<uint32_t> block_tags;
    long el_start = 0, el_n = 0, block_dim = 0;
    uint32_t block_phys = 0;
    const char *b, *e;
    while (lr.next(b, e)) {
        if (e > b && *b == '$') {
            section.assign(b + 1, e);
            ns = 1;
            nss += 1;
            node_nss += 1;
            continue;
        }
        if (section == "PhysicalNames") {
            if (ns > 1) {
                Tok t{b, e};
                const char *t0b, *t0e, *t1b, *t1e, *t2b, *t2e;
                if (!t.next(t0b, t0e) || !t.next(t1b, t1e) || !t.next(t2b, t2e))
                    throw Error(3, "gmsh: bad $PhysicalNames line");
                std::string name(t2b, t2e);
                name.erase(std::remove(name.begin(), name.end(), '"'), name.end());
                physicalNames[(uint32_t)(tok_int(t1b, t1e) + 1000 * tok_int(t0b, t0e))] = name;
            }
        } else if (section == "Entities") {
            if (ns == 1) {
                auto l = ints(b, e);
                if (l.size() < 4) throw Error(3, "gmsh: bad $Entities header");
                n_points = l[0];
                n_curves = l[1] + l[0];
                nss = 0;
            } else if (nss <= n_points) {
            } else if (nss <= n_curves) {
                auto l = ints(b, e);
                if (l.size() < 9) throw Error(3, "gmsh: curve entity without a physical tag");
                entityPhys[(uint32_t)l[0]] = (uint32_t)(l[8] + 1000);
            }
        } else if (section == "Nodes") {
            if (ns == 1) {
                node_start = 1;
                node_nss = 0;
            } else if (ns > node_start + 2 * node_n) {
                auto l = ints(b, e);
                if (l.size() < 4) throw Error(3, "gmsh: bad node block header");
                node_n = l[3];
                node_start = ns;
                block_tags.assign(node_n, 0);
                node_nss = 0;
            } else if (node_nss <= node_n) {
                block_tags[node_nss - 1] = (uint32_t)(tok_int(b, e) - 1);
            } else {
                uint32_t tag = block_tags[node_nss - 1 - node_n];
                Tok t{b, e};
                const char *xb, *xe, *yb, *ye;
                if (!t.next(xb, xe) || !t.next(yb, ye)) throw Error(3, "gmsh: bad node coordinates");
                nodeRef[tag] = (uint32_t)m.nodesX.size();
                m.nodesX.push_back(tok_double(xb, xe));
                m.nodesY.push_back(tok_double(yb, ye));
            }
        } else if (section == "Elements") {
            if (ns == 1) {
                el_start = 1;
                el_n = 0;
            } else if (ns > el_start + el_n) {
                auto l = ints(b, e);
                if (l.size() < 4) throw Error(3, "gmsh: bad element block header");
                block_dim = l[0];
                if (block_dim == 1) {
                    auto it = entityPhys.find((uint32_t)l[1]);
                    if (it == entityPhys.end()) throw Error(3, "gmsh: boundary entity without physical group");
                    block_phys = it->second;
                }
                el_n = l[3];
                el_start = ns;
            } else if (block_dim == 1 || block_dim == 2) {
                auto li = ints(b, e);
                size_t nn = li.size() - 1;
                auto node = [&](long t) {
                    auto it = nodeRef.find((uint32_t)(t - 1));
                    if (it == nodeRef.end()) throw Error(3, "gmsh: element references an unknown node");
                    return it->second;
                };
                if (block_dim == 1 && nn == 2) {
                    m.bnd0.push_back(node(li[1]));
                    m.bnd1.push_back(node(li[2]));
                    bndTag.push_back(block_phys);
                } else if (block_dim == 2 && nn != 2) {
                    if (nn != 3 && nn != 4)
                        throw Error(3, "size of input array " + std::to_string(nn) + " not equal to 4");
                    std::array<uint32_t, 4> c{0, 0, 0, 0};
                    for (size_t i = 0; i < nn; ++i) c[i] = node(li[i + 1]);
                    m.cellsNodes.push_back(c);
                    m.cellsIsTriangle.push_back(nn == 3);
                }
            }
        }
        ns += 1;
        nss += 1;
        node_nss += 1;
    }
    for (uint32_t t : bndTag) {
        auto it = physicalNames.find(t);
        if (it == physicalNames.end()) throw Error(3, "gmsh: boundary physical tag without a name");
        m.bndName.push_back(it->second);
    }
    m.finalize();
    return m;
}

// -------------------------------------------------------------- finalize
namespace {

// Stable LSD radix sort of (key, payload) by key.
void radix_sort(std::vector<uint64_t>& key, std::vector<uint32_t>& val, int key_bits) {
    const size_t n = key.size();
    std::vector<uint64_t> k2(n);
    std::vector<uint32_t> v2(n);
    for (int shift = 0; shift < key_bits; shift += 16) {
        std::vector<size_t> cnt(65537, 0);
        for (size_t i = 0; i < n; ++i) cnt[((key[i] >> shift) & 0xFFFF) + 1]++;
        for (int d = 0; d < 65536; ++d) cnt[d + 1] += cnt[d];
        for (size_t i = 0; i < n; ++i) {
            size_t d = (key[i] >> shift) & 0xFFFF;
            size_t o = cnt[d]++;
            k2[o] = key[i];
            v2[o] = val[i];
        }
        key.swap(k2);
        val.swap(v2);
    }
}

}  // namespace

// Cell and edge metrics of the real cells from the node coordinates
// (mesh.h:378-453); the cell arrays hold the real cells afterwards.
void HostMesh::compute_metrics() {
    const uint32_t N = nRealCells;
    const uint32_t E = (uint32_t)edgesNodes.size();
    cellsAreas.assign(N, 0.);
    cellsCentersX.assign(N, 0.);
    cellsCentersY.assign(N, 0.);
    edgesLengths.assign(E, 0.);
    edgesNormalsX.assign(E, 0.);
    edgesNormalsY.assign(E, 0.);
    edgesCentersX.assign(E, 0.);
    edgesCentersY.assign(E, 0.);
#pragma omp parallel for
    for (long i = 0; i < (long)N; ++i) {
        double cx = 0., cy = 0.;
        uint32_t n = cellsIsTriangle[i] ? 3 : 4;
        for (uint32_t j = 0; j < n; ++j) {
            cx += nodesX[cellsNodes[i][j]] / ((double)n);
            cy += nodesY[cellsNodes[i][j]] / ((double)n);
        }
        cellsCentersX[i] = cx;
        cellsCentersY[i] = cy;
    }
#pragma omp parallel for
    for (long i = 0; i < (long)E; ++i) {
        const uint32_t a = edgesNodes[i][0], b = edgesNodes[i][1];
        edgesCentersX[i] = (nodesX[b] + nodesX[a]) * 0.5;
        edgesCentersY[i] = (nodesY[b] + nodesY[a]) * 0.5;
        double dex = nodesX[b] - nodesX[a];
        double dey = nodesY[b] - nodesY[a];
        double l = std::sqrt(dex * dex + dey * dey);
        edgesLengths[i] = l;
        edgesNormalsX[i] = -dey / l;
        edgesNormalsY[i] = dex / l;
        double dot = edgesNormalsX[i] * (edgesCentersX[i] - cellsCentersX[edgesCells[i][0]]) +
                     edgesNormalsY[i] * (edgesCentersY[i] - cellsCentersY[edgesCells[i][0]]);
        if (dot < 0) {
            edgesNormalsX[i] *= -1.;
            edgesNormalsY[i] *= -1.;
        }
    }
#pragma omp parallel for
    for (long i = 0; i < (long)N; ++i) {
        const auto& n = cellsNodes[i];
        double x1 = nodesX[n[0]], x2 = nodesX[n[1]], x3 = nodesX[n[2]];
        double y1 = nodesY[n[0]], y2 = nodesY[n[1]], y3 = nodesY[n[2]];
        if (cellsIsTriangle[i]) {
            cellsAreas[i] = 0.5 * std::fabs(x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2));
        } else {
            double x4 = nodesX[n[3]], y4 = nodesY[n[3]];
            cellsAreas[i] = 0.5 * std::fabs(x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2)) +
                            0.5 * std::fabs(x1 * (y3 - y4) + x3 * (y4 - y1) + x4 * (y1 - y3));
        }
    }

}

// New node coordinates, same topology: metrics and ghost-cell geometry
// (mesh.h:744-787) recomputed with the formulas of finalize().
void HostMesh::update_nodes(const double* x, const double* y) {
    std::copy(x, x + nodesX.size(), nodesX.begin());
    std::copy(y, y + nodesY.size(), nodesY.begin());
    compute_metrics();
    for (size_t b = 0; b < boundaryEdges.size(); ++b) {
        const uint32_t e = boundaryEdges[b];
        const uint32_t cell = edgesCells[e][0];
        double area = cellsAreas[cell];
        double dx = edgesCentersX[e] - cellsCentersX[cell];
        double dy = edgesCentersY[e] - cellsCentersY[cell];
        double dist = std::sqrt(dx * dx + dy * dy);
        double cx = edgesCentersX[e] + dist * edgesNormalsX[e];
        double cy = edgesCentersY[e] + dist * edgesNormalsY[e];
        cellsAreas.push_back(area);
        cellsCentersX.push_back(cx);
        cellsCentersY.push_back(cy);
    }
}

void HostMesh::finalize() {
    const uint32_t N = (uint32_t)cellsNodes.size();
    const uint64_t NN = nodesX.size();
    if (N == 0) throw Error(3, "mesh has no cells");
    for (auto& c : cellsNodes)
        for (int j = 0; j < 4; ++j)
            if (c[j] >= NN) throw Error(3, "cell references a node out of range");
    nRealCells = N;

    // half-edges in the order add_cell_edges meets them (mesh.h:317-341)
    std::vector<uint64_t> key;
    std::vector<uint32_t> pos;
    key.reserve((size_t)N * 4);
    pos.reserve((size_t)N * 4);
    for (uint32_t i = 0; i < N; ++i) {
        uint32_t size = cellsIsTriangle[i] ? 3 : 4;
        for (uint32_t j = 0; j < size; ++j) {
            uint32_t a = cellsNodes[i][j], b = cellsNodes[i][(j < size - 1) ? j + 1 : 0];
            key.push_back((uint64_t)std::min(a, b) * NN + std::max(a, b));
            pos.push_back(4 * i + j);
        }
    }
    int bits = 0;
    while (bits < 64 && (NN * NN >> bits) > 0) bits += 16;
    radix_sort(key, pos, bits);

    // first occurrence creates the edge; ids follow first-occurrence order
    const size_t H = key.size();
    std::vector<uint8_t> first(4 * (size_t)N, 0);
    for (size_t s = 0; s < H;) {
        size_t t = s;
        while (t < H && key[t] == key[s]) ++t;
        first[pos[s]] = 1;
        s = t;
    }
    std::vector<uint32_t> id_of_first(4 * (size_t)N, 0xFFFFFFFFu);
    uint32_t E = 0;
    for (size_t p = 0; p < first.size(); ++p)
        if (first[p]) id_of_first[p] = E++;
    edgesNodes.assign(E, {0, 0});
    edgesCells.assign(E, {0, 0});
    cellsEdges.assign(N, {0, 0, 0, 0});
    std::vector<uint8_t> has_second(E, 0);
    std::vector<uint64_t> ukey(E);
    for (size_t s = 0; s < H;) {
        size_t t = s;
        while (t < H && key[t] == key[s]) ++t;
        const uint32_t p0 = pos[s];
        const uint32_t eid = id_of_first[p0];
        const uint32_t c0 = p0 / 4, j0 = p0 % 4;
        const uint32_t size = cellsIsTriangle[c0] ? 3 : 4;
        edgesNodes[eid] = {cellsNodes[c0][j0], cellsNodes[c0][(j0 < size - 1) ? j0 + 1 : 0]};
        edgesCells[eid] = {c0, 0};
        ukey[eid] = key[s];
        // convert_node_face_info (mesh.h:344-375): the last other cell wins
        for (size_t u = s; u < t; ++u) {
            const uint32_t c = pos[u] / 4;
            cellsEdges[c][pos[u] % 4] = eid;  // cellsEdges(i, j): local edge j of cell i
            if (c != c0) {
                edgesCells[eid][1] = c;
                has_second[eid] = 1;
            }
        }
        s = t;
    }

    compute_metrics();

    // ghost cells (mesh.h:744-787)
    std::vector<uint64_t> skey(ukey);
    std::vector<uint32_t> sid(E);
    std::iota(sid.begin(), sid.end(), 0u);
    radix_sort(skey, sid, bits);
    std::vector<uint8_t> is_bnd(E, 0);
    boundaryEdges.clear();
    boundaryEdgesPhysicals.clear();
    for (size_t i = 0; i < bnd0.size(); ++i) {
        const uint32_t nmin = std::min(bnd0[i], bnd1[i]), nmax = std::max(bnd0[i], bnd1[i]);
        const uint64_t k = (uint64_t)nmin * NN + nmax;
        auto it = std::lower_bound(skey.begin(), skey.end(), k);
        if (it == skey.end() || *it != k)
            throw Error(3, "invalid edge ref (" + std::to_string(nmin) + ", " + std::to_string(nmax) + ")");
        const uint32_t e = sid[it - skey.begin()];
        if (is_bnd[e]) throw Error(3, "boundary edge listed twice (" + std::to_string(nmin) + ", " +
                                          std::to_string(nmax) + ")");
        is_bnd[e] = 1;
        const uint32_t cell = edgesCells[e][0];
        double area = cellsAreas[cell];
        double dx = edgesCentersX[e] - cellsCentersX[cell];
        double dy = edgesCentersY[e] - cellsCentersY[cell];
        double dist = std::sqrt(dx * dx + dy * dy);
        double cx = edgesCentersX[e] + dist * edgesNormalsX[e];
        double cy = edgesCentersY[e] + dist * edgesNormalsY[e];
        cellsAreas.push_back(area);
        cellsCentersX.push_back(cx);
        cellsCentersY.push_back(cy);
        cellsIsTriangle.push_back(1);
        cellsNodes.push_back({nmin, nmax, 0, 0});
        edgesCells[e][1] = (uint32_t)cellsAreas.size() - 1;
        boundaryEdges.push_back(e);
        boundaryEdgesPhysicals.push_back(bndName.at(i));
    }
    for (uint32_t e = 0; e < E; ++e)
        if (!has_second[e] && !is_bnd[e])
            throw Error(3, "edge (" + std::to_string(edgesNodes[e][0]) + ", " + std::to_string(edgesNodes[e][1]) +
                               ") has one cell and is not a listed boundary edge");
    wall_dist.assign(cellsAreas.size(), 0.);
}

// --------------------------------------------------------------- layout
namespace {

// Hilbert index of (x, y) on a 2^16 x 2^16 grid.
uint32_t hilbert(uint32_t x, uint32_t y) {
    uint32_t d = 0;
    for (uint32_t s = 1u << 15; s > 0; s >>= 1) {
        uint32_t rx = (x & s) > 0, ry = (y & s) > 0;
        d += s * s * ((3 * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = s - 1 - x;
                y = s - 1 - y;
            }
            std::swap(x, y);
        }
    }
    return d;
}

}  // namespace

DeviceLayout build_layout(const HostMesh& m) {
    DeviceLayout L;
    const int N = (int)m.nRealCells;
    const int E = (int)m.edgesCells.size();
    const int B = (int)m.boundaryEdges.size();
    L.n_cells = N;
    L.n_faces = E;
    L.n_bnd = B;

    // cells along a Hilbert curve of their centroids, within each segment
    // (a batch of independent cases keeps each case's cells contiguous)
    std::vector<int> seg = m.segments;
    if (seg.empty()) seg = {0, N};
    std::vector<uint64_t> hk(N);
    std::vector<uint32_t> hv(N);
    for (size_t sg = 0; sg + 1 < seg.size(); ++sg) {
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
        for (int i = seg[sg]; i < seg[sg + 1]; ++i) {
            xmin = std::min(xmin, m.cellsCentersX[i]);
            xmax = std::max(xmax, m.cellsCentersX[i]);
            ymin = std::min(ymin, m.cellsCentersY[i]);
            ymax = std::max(ymax, m.cellsCentersY[i]);
        }
        const double span = std::max(std::max(xmax - xmin, ymax - ymin), 1e-300);
        for (int i = seg[sg]; i < seg[sg + 1]; ++i) {
            uint32_t gx = (uint32_t)std::min(65535.0, std::floor((m.cellsCentersX[i] - xmin) / span * 65535.0));
            uint32_t gy = (uint32_t)std::min(65535.0, std::floor((m.cellsCentersY[i] - ymin) / span * 65535.0));
            hk[i] = ((uint64_t)sg << 32) | hilbert(gx, gy);
            hv[i] = (uint32_t)i;
        }
    }
    radix_sort(hk, hv, seg.size() > 2 ? 48 : 32);
    L.cell_old.assign(hv.begin(), hv.end());
    L.cell_new.assign(N, 0);
    for (int i = 0; i < N; ++i) L.cell_new[L.cell_old[i]] = i;

    // boundary index of each edge
    std::vector<int> bnd_of_edge(E, -1);
    for (int b = 0; b < B; ++b) bnd_of_edge[m.boundaryEdges[b]] = b;

    // faces ordered by the first device cell they touch
    std::vector<uint64_t> fk(E);
    std::vector<uint32_t> fv(E);
    for (int e = 0; e < E; ++e) {
        uint32_t a = L.cell_new[m.edgesCells[e][0]];
        uint32_t c1 = m.edgesCells[e][1];
        uint32_t b = c1 < (uint32_t)N ? L.cell_new[c1] : a;
        fk[e] = std::min(a, b);
        fv[e] = (uint32_t)e;
    }
    radix_sort(fk, fv, 32);
    L.face_edge.assign(fv.begin(), fv.end());
    std::vector<int> face_of_edge(E);
    for (int f = 0; f < E; ++f) face_of_edge[L.face_edge[f]] = f;

    // per-cell face slots in ascending reference edge id: +(face+1) when the
    // cell is the face's cell 0, -(face+1) when it is cell 1; the other cell
    // (device id, or -(b+1) for boundary b) beside it
    L.cslot.assign(4 * (size_t)N, 0);
    L.cnbr.assign(4 * (size_t)N, 0);
    std::vector<uint8_t> cnt(N, 0);
    for (int e = 0; e < E; ++e) {
        const uint32_t c0 = m.edgesCells[e][0], c1 = m.edgesCells[e][1];
        const uint32_t cs[2] = {c0, c1};
        const int other_of_c0 = c1 < (uint32_t)N ? L.cell_new[c1] : -(bnd_of_edge[e] + 1);
        for (int s = 0; s < 2; ++s) {
            if (cs[s] >= (uint32_t)N) continue;
            if (s == 1 && c1 == c0) continue;
            const int nc = L.cell_new[cs[s]];
            if (cnt[nc] >= 4) throw Error(3, "cell " + std::to_string(cs[s]) + " has more than 4 faces");
            const size_t k = 4 * (size_t)nc + cnt[nc]++;
            L.cslot[k] = s == 0 ? face_of_edge[e] + 1 : -(face_of_edge[e] + 1);
            L.cnbr[k] = s == 0 ? other_of_c0 : L.cell_new[c0];
        }
    }

    // face records
    L.fcell.assign(2 * (size_t)E, 0);
    L.bface.assign(B, 0);
    for (int f = 0; f < E; ++f) {
        const uint32_t e = L.face_edge[f];
        const uint32_t i = m.edgesCells[e][0], j = m.edgesCells[e][1];
        L.fcell[2 * f] = L.cell_new[i];
        L.fcell[2 * f + 1] = j < (uint32_t)N ? L.cell_new[j] : -(bnd_of_edge[e] + 1);
    }
    for (int b = 0; b < B; ++b) L.bface[b] = face_of_edge[m.boundaryEdges[b]];
    fill_layout_geometry(m, L);
    return L;
}

void fill_layout_geometry(const HostMesh& m, DeviceLayout& L) {
    const long E = L.n_faces;
    const int N = L.n_cells;
    L.fn.assign(2 * (size_t)E, 0.);
    L.fLg.assign(2 * (size_t)E, 0.);
    L.fd0.assign(2 * (size_t)E, 0.);
    L.fd1.assign(2 * (size_t)E, 0.);
    L.ft.assign(4 * (size_t)E, 0.);
#pragma omp parallel for
    for (long f = 0; f < E; ++f) {
        const uint32_t e = L.face_edge[f];
        const uint32_t i = m.edgesCells[e][0], j = m.edgesCells[e][1];
        L.fn[2 * f] = m.edgesNormalsX[e];
        L.fn[2 * f + 1] = m.edgesNormalsY[e];
        // Green-Gauss face weight, solver.h:436-444
        const double dxif = m.edgesCentersX[e] - m.cellsCentersX[i];
        const double dyif = m.edgesCentersY[e] - m.cellsCentersY[i];
        const double dif = std::sqrt(dxif * dxif + dyif * dyif);
        const double dxij = m.cellsCentersX[i] - m.cellsCentersX[j];
        const double dyij = m.cellsCentersY[i] - m.cellsCentersY[j];
        const double dij = std::sqrt(dxij * dxij + dyij * dyij);
        L.fLg[2 * f] = m.edgesLengths[e];
        L.fLg[2 * f + 1] = dif / dij;
        // reconstruction offsets, solver.h:774-778 (also the limiter's, solver.h:541-542)
        L.fd0[2 * f] = m.edgesCentersX[e] - m.cellsCentersX[i];
        L.fd0[2 * f + 1] = m.edgesCentersY[e] - m.cellsCentersY[i];
        L.fd1[2 * f] = m.edgesCentersX[e] - m.cellsCentersX[j];
        L.fd1[2 * f + 1] = m.edgesCentersY[e] - m.cellsCentersY[j];
        // face-gradient direction of average_gradients, solver.h:369-376
        double t0 = m.cellsCentersX[i] + m.cellsCentersX[j];
        double t1 = m.cellsCentersY[i] + m.cellsCentersY[j];
        const double lij = std::sqrt(t0 * t0 + t1 * t1);
        t0 /= lij;
        t1 /= lij;
        L.ft[4 * f] = t0;
        L.ft[4 * f + 1] = t1;
        L.ft[4 * f + 2] = lij;
    }
    L.area.assign(N, 0.);
    for (int i = 0; i < N; ++i) L.area[i] = m.cellsAreas[L.cell_old[i]];
}

}  // namespace afx
