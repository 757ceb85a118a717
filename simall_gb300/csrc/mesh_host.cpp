// Host preprocessing that feeds the pressure path: the structured hex box as
// an unstructured SoA mesh and reverse Cuthill-McKee renumbering.
//
// simall_mesh_cartesian produces exactly what CartesianMesher::generate +
// ConnectivityBuilder::build + Mesh::compute_geometry produce
// (src/meshing/CartesianMesher.cpp:13-101, Connectivity.cpp:45-115,
// MeshStorage.cpp:21-97): the same face numbering, owners, node order per
// face and bit-identical geometry.  It gets there without the reference's
// hash of sorted face-node tuples: for a structured box the first cell to
// list a face is known in closed form (cell (i,j,k) creates its -Z face only
// when k == 0, its -Y face only when j == 0, its -X face only when i == 0, and
// always its three + faces), so faces are numbered in one sweep, O(1) memory
// per face and no node connectivity stored.
#include "simall_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr uint64_t kBoundary = ~0ull;

struct P3 {
    double x, y, z;
};

// Node-average centroid and Newell fan area of a 4-node face, in the
// reference's operation order (MeshStorage.cpp:33-62).
inline void quad_geometry(const P3 (&v)[4], P3 &c, P3 &a)
{
    double cx = 0.0, cy = 0.0, cz = 0.0;
    for (int i = 0; i < 4; ++i) {
        cx += v[i].x;
        cy += v[i].y;
        cz += v[i].z;
    }
    const double inv = 1.0 / 4.0;
    cx *= inv;
    cy *= inv;
    cz *= inv;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int i = 0; i < 4; ++i) {
        const P3 &pa = v[i], &pb = v[(i + 1) & 3];
        const double ax = pa.x - cx, ay = pa.y - cy, az = pa.z - cz;
        const double bx = pb.x - cx, by = pb.y - cy, bz = pb.z - cz;
        const double crx = ay * bz - az * by;
        const double cry = az * bx - ax * bz;
        const double crz = ax * by - ay * bx;
        sx = sx + crx * 0.5;
        sy = sy + cry * 0.5;
        sz = sz + crz * 0.5;
    }
    c = {cx, cy, cz};
    a = {sx, sy, sz};
}

}  // namespace

extern "C" int simall_mesh_cartesian(int Nx, int Ny, int Nz, double ex, double ey, double ez, const double *ndx,
                                     const double *ndy, const double *ndz, uint64_t *owner, uint64_t *neighbor,
                                     double *area_x, double *area_y, double *area_z, double *cen_x, double *cen_y,
                                     double *cen_z, uint32_t *zone, double *volume, double *ccx, double *ccy,
                                     double *ccz, int32_t *cfOff, uint64_t *cfIdx)
{
    if (Nx <= 0 || Ny <= 0 || Nz <= 0 || !owner || !neighbor || !area_x || !area_y || !area_z || !cen_x || !cen_y ||
        !cen_z || !zone || !volume || !ccx || !ccy || !ccz || !cfOff || !cfIdx)
        return SIMALL_ERR_INVALID_ARGUMENT;
    const int64_t nC = static_cast<int64_t>(Nx) * Ny * Nz;
    if (6 * nC > INT32_MAX)
        return SIMALL_ERR_INVALID_ARGUMENT;
    const double dx = ex / Nx, dy = ey / Ny, dz = ez / Nz;
    const int64_t Px = Nx + 1, Py = Ny + 1;
    auto node = [&](int i, int j, int k) -> P3 {
        const int64_t id = ((static_cast<int64_t>(k) * Py) + j) * Px + i;
        P3 p{0.0 + i * dx, 0.0 + j * dy, 0.0 + k * dz};
        if (ndx) {
            p.x += ndx[id];
            p.y += ndy[id];
            p.z += ndz[id];
        }
        return p;
    };
    // face ids of the + faces of the previous cells, needed by their neighbours
    std::vector<int64_t> plusZ(static_cast<size_t>(Nx) * Ny), plusY(static_cast<size_t>(Nx));
    int64_t plusX = -1;
    int64_t nF = 0, e = 0, c = 0;
    cfOff[0] = 0;
    auto make_face = [&](const P3 (&v)[4], int64_t cell) -> int64_t {
        P3 cc, aa;
        quad_geometry(v, cc, aa);
        const int64_t f = nF++;
        owner[f] = static_cast<uint64_t>(cell);
        neighbor[f] = kBoundary;
        area_x[f] = aa.x;
        area_y[f] = aa.y;
        area_z[f] = aa.z;
        cen_x[f] = cc.x;
        cen_y[f] = cc.y;
        cen_z[f] = cc.z;
        return f;
    };
    for (int k = 0; k < Nz; ++k)
        for (int j = 0; j < Ny; ++j)
            for (int i = 0; i < Nx; ++i, ++c) {
                const P3 n0 = node(i, j, k), n1 = node(i + 1, j, k), n2 = node(i + 1, j + 1, k),
                         n3 = node(i, j + 1, k), n4 = node(i, j, k + 1), n5 = node(i + 1, j, k + 1),
                         n6 = node(i + 1, j + 1, k + 1), n7 = node(i, j + 1, k + 1);
                int64_t f;
                // -Z {n0,n3,n2,n1}
                if (k == 0) {
                    const P3 v[4] = {n0, n3, n2, n1};
                    f = make_face(v, c);
                } else {
                    f = plusZ[static_cast<size_t>(j) * Nx + i];
                    neighbor[f] = static_cast<uint64_t>(c);
                }
                cfIdx[e++] = static_cast<uint64_t>(f);
                {  // +Z {n4,n5,n6,n7}
                    const P3 v[4] = {n4, n5, n6, n7};
                    f = make_face(v, c);
                    plusZ[static_cast<size_t>(j) * Nx + i] = f;
                    cfIdx[e++] = static_cast<uint64_t>(f);
                }
                // -Y {n0,n1,n5,n4}
                if (j == 0) {
                    const P3 v[4] = {n0, n1, n5, n4};
                    f = make_face(v, c);
                } else {
                    f = plusY[i];
                    neighbor[f] = static_cast<uint64_t>(c);
                }
                cfIdx[e++] = static_cast<uint64_t>(f);
                {  // +Y {n3,n7,n6,n2}
                    const P3 v[4] = {n3, n7, n6, n2};
                    f = make_face(v, c);
                    plusY[i] = f;
                    cfIdx[e++] = static_cast<uint64_t>(f);
                }
                // -X {n0,n4,n7,n3}
                if (i == 0) {
                    const P3 v[4] = {n0, n4, n7, n3};
                    f = make_face(v, c);
                } else {
                    f = plusX;
                    neighbor[f] = static_cast<uint64_t>(c);
                }
                cfIdx[e++] = static_cast<uint64_t>(f);
                {  // +X {n1,n2,n6,n5}
                    const P3 v[4] = {n1, n2, n6, n5};
                    f = make_face(v, c);
                    plusX = f;
                    cfIdx[e++] = static_cast<uint64_t>(f);
                }
                cfOff[c + 1] = static_cast<int32_t>(e);
            }
    // cell volume and centroid by the divergence theorem (MeshStorage.cpp:65-96)
    for (int64_t q = 0; q < nC; ++q) {
        double V = 0.0, wx = 0.0, wy = 0.0, wz = 0.0;
        for (int32_t t = cfOff[q]; t < cfOff[q + 1]; ++t) {
            const uint64_t f = cfIdx[t];
            const double sgn = (owner[f] == static_cast<uint64_t>(q)) ? 1.0 : -1.0;
            const double d = cen_x[f] * area_x[f] + cen_y[f] * area_y[f] + cen_z[f] * area_z[f];
            const double dv = sgn * d / 3.0;
            V += dv;
            wx = wx + cen_x[f] * dv * (3.0 / 4.0);
            wy = wy + cen_y[f] * dv * (3.0 / 4.0);
            wz = wz + cen_z[f] * dv * (3.0 / 4.0);
        }
        volume[q] = V;
        ccx[q] = ccy[q] = ccz[q] = 0.0;
        if (V != 0.0) {
            ccx[q] = wx / V;
            ccy[q] = wy / V;
            ccz[q] = wz / V;
        }
    }
    // zones from face centroids (CartesianMesher.cpp:66-89): interior 0,
    // xMin 1, xMax 2, yMin 3, yMax 4, zMin 5, zMax 6; else the builder's 1
    const double tol = 1e-9;
    for (int64_t f = 0; f < nF; ++f) {
        if (neighbor[f] != kBoundary) {
            zone[f] = 0;
            continue;
        }
        const double cx = cen_x[f], cy = cen_y[f], cz = cen_z[f];
        uint32_t z = 1;
        if (std::abs(cx - 0.0) < tol)
            z = 1;
        else if (std::abs(cx - (0.0 + ex)) < tol)
            z = 2;
        else if (std::abs(cy - 0.0) < tol)
            z = 3;
        else if (std::abs(cy - (0.0 + ey)) < tol)
            z = 4;
        else if (std::abs(cz - 0.0) < tol)
            z = 5;
        else if (std::abs(cz - (0.0 + ez)) < tol)
            z = 6;
        zone[f] = z;
    }
    return SIMALL_OK;
}

// Reverse Cuthill-McKee (MeshOps.cpp:547-676): BFS from the lowest-index
// unvisited cell of minimum degree, unvisited neighbours in ascending id then
// stably by degree, order reversed; cell arrays permuted, faces remapped.
extern "C" int simall_mesh_rcm(int64_t nC, int64_t nF, uint64_t *owner, uint64_t *neighbor, double *volume,
                               double *ccx, double *ccy, double *ccz, int32_t *cfOff, uint64_t *cfIdx, int64_t *stats)
{
    if (nC < 0 || nF < 0 || !owner || !neighbor || !volume || !ccx || !ccy || !ccz || !cfOff || !cfIdx)
        return SIMALL_ERR_INVALID_ARGUMENT;
    auto bandwidth = [&]() {
        uint64_t bw = 0;
        for (int64_t f = 0; f < nF; ++f) {
            if (neighbor[f] == kBoundary)
                continue;
            const uint64_t a = owner[f], b = neighbor[f];
            const uint64_t d = a > b ? a - b : b - a;
            bw = std::max(bw, d);
        }
        return static_cast<int64_t>(bw);
    };
    const int64_t bw0 = bandwidth();
    if (nC == 0) {
        if (stats) {
            stats[0] = bw0;
            stats[1] = bw0;
            stats[2] = 0;
        }
        return SIMALL_OK;
    }
    // adjacency CSR from interior faces, sorted and unique per cell
    std::vector<int64_t> off(static_cast<size_t>(nC) + 1, 0);
    for (int64_t f = 0; f < nF; ++f) {
        if (neighbor[f] == kBoundary)
            continue;
        const uint64_t a = owner[f], b = neighbor[f];
        if (a >= static_cast<uint64_t>(nC) || b >= static_cast<uint64_t>(nC))
            continue;
        off[a + 1]++;
        off[b + 1]++;
    }
    for (int64_t q = 0; q < nC; ++q)
        off[q + 1] += off[q];
    std::vector<int64_t> adj(static_cast<size_t>(off[nC])), fill(off.begin(), off.end() - 1);
    for (int64_t f = 0; f < nF; ++f) {
        if (neighbor[f] == kBoundary)
            continue;
        const uint64_t a = owner[f], b = neighbor[f];
        if (a >= static_cast<uint64_t>(nC) || b >= static_cast<uint64_t>(nC))
            continue;
        adj[fill[a]++] = static_cast<int64_t>(b);
        adj[fill[b]++] = static_cast<int64_t>(a);
    }
    std::vector<int64_t> deg(static_cast<size_t>(nC));
    for (int64_t q = 0; q < nC; ++q) {
        auto b0 = adj.begin() + off[q], b1 = adj.begin() + fill[q];
        std::sort(b0, b1);
        deg[q] = std::unique(b0, b1) - b0;
    }
    std::vector<uint8_t> seen(static_cast<size_t>(nC), 0);
    std::vector<int64_t> order;
    order.reserve(static_cast<size_t>(nC));
    std::vector<int64_t> queue(static_cast<size_t>(nC)), nb;
    // the minimum-degree seed search scans from cell 0 for every component
    while (static_cast<int64_t>(order.size()) < nC) {
        int64_t seed = -1;
        for (int64_t q = 0; q < nC; ++q) {
            if (seen[q])
                continue;
            if (seed < 0 || deg[q] < deg[seed])
                seed = q;
        }
        if (seed < 0)
            break;
        int64_t qh = 0, qt = 0;
        queue[qt++] = seed;
        seen[seed] = 1;
        while (qh < qt) {
            const int64_t q = queue[qh++];
            order.push_back(q);
            nb.clear();
            for (int64_t t = off[q]; t < off[q] + deg[q]; ++t) {
                const int64_t v = adj[t];
                if (!seen[v]) {
                    nb.push_back(v);
                    seen[v] = 1;
                }
            }
            std::stable_sort(nb.begin(), nb.end(), [&](int64_t a, int64_t b) { return deg[a] < deg[b]; });
            for (int64_t v : nb)
                queue[qt++] = v;
        }
    }
    std::reverse(order.begin(), order.end());
    std::vector<int64_t> newPos(static_cast<size_t>(nC), -1);
    for (size_t k = 0; k < order.size(); ++k)
        newPos[order[k]] = static_cast<int64_t>(k);
    for (int64_t q = 0; q < nC; ++q)
        if (newPos[q] < 0)
            newPos[q] = q;
    std::vector<double> tmp(static_cast<size_t>(nC));
    for (double *arr : {volume, ccx, ccy, ccz}) {
        for (int64_t q = 0; q < nC; ++q)
            tmp[newPos[q]] = arr[q];
        std::memcpy(arr, tmp.data(), static_cast<size_t>(nC) * sizeof(double));
    }
    const int64_t ncf = cfOff[nC];
    std::vector<int32_t> offNew(static_cast<size_t>(nC) + 1, 0);
    std::vector<uint64_t> idxNew(static_cast<size_t>(ncf));
    int64_t w = 0;
    for (int64_t q = 0; q < nC; ++q) {
        const int64_t src = order[q];
        for (int32_t t = cfOff[src]; t < cfOff[src + 1]; ++t)
            idxNew[w++] = cfIdx[t];
        offNew[q + 1] = static_cast<int32_t>(w);
    }
    std::memcpy(cfOff, offNew.data(), offNew.size() * sizeof(int32_t));
    std::memcpy(cfIdx, idxNew.data(), idxNew.size() * sizeof(uint64_t));
    for (int64_t f = 0; f < nF; ++f) {
        owner[f] = static_cast<uint64_t>(newPos[owner[f]]);
        if (neighbor[f] != kBoundary)
            neighbor[f] = static_cast<uint64_t>(newPos[neighbor[f]]);
    }
    if (stats) {
        stats[0] = bw0;
        stats[1] = bandwidth();
        stats[2] = static_cast<int64_t>(order.size());
    }
    return SIMALL_OK;
}
