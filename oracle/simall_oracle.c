/*
 * simall_oracle.c -- TEST INFRASTRUCTURE, not product code.
 *
 * A plain-C, serial restatement of the SimAll reference algorithms on the
 * pressure-correction path.  It is the checker the CUDA library is compared
 * against: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  Parity of this restatement with the reference itself is
 * pinned by tests/test_oracle_vs_reference.py (live, where the reference
 * compiles) and tests/test_oracle_golden.py (committed fixtures made by
 * tests/golden/make_golden.py from the compiled reference).
 *
 * Floating-point operations are written in the same order as the reference
 * and the file is compiled with -ffp-contract=off, so results are bit-exact
 * with the reference on any IEEE-754 host (x86_64 without FMA, aarch64 with
 * contraction off).
 *
 * Index conventions: cell ids are int64, a boundary face has neighbor == -1
 * (the reference's kBoundaryCell = ~0ull, src/meshing/MeshStorage.hpp:35).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_BOUNDARY (-1)

/* std::max(a, b) as the reference evaluates it: (a < b) ? b : a */
#define STD_MAX(a, b) (((a) < (b)) ? (b) : (a))

/* ------------------------------------------------------------------ helpers */

static void *xmalloc(size_t n)
{
    void *p = malloc(n ? n : 1);
    if (!p)
        abort();
    return p;
}

static void sort4(int64_t *k)
{
    for (int i = 1; i < 4; ++i) {
        int64_t v = k[i];
        int j = i - 1;
        while (j >= 0 && k[j] > v) {
            k[j + 1] = k[j];
            --j;
        }
        k[j + 1] = v;
    }
}

/* ------------------------------------------------------------------ mesh topology */

/*
 * Structured hex grid as an unstructured SoA mesh.
 * Follows CartesianMesher::generate (src/meshing/CartesianMesher.cpp:13-58):
 * node (i,j,k) at origin + (i*dx, j*dy, k*dz), node id ((k*Py)+j)*Px+i; cell
 * faces in the order -Z{n0,n3,n2,n1}, +Z{n4,n5,n6,n7}, -Y{n0,n1,n5,n4},
 * +Y{n3,n7,n6,n2}, -X{n0,n4,n7,n3}, +X{n1,n2,n6,n5}.
 * Then ConnectivityBuilder::build (src/meshing/Connectivity.cpp:45-115): a
 * face is keyed by its sorted node tuple; the first cell to list it creates it
 * (owner = that cell, nodes in that cell's order), the second sets neighbor;
 * each cell's face list keeps its descriptor order.  The lookup here is an
 * open-addressing table keyed by the sorted tuple.
 *
 * Outputs (caller-allocated): nodes x/y/z [nNodes]; fnOff [nF+1]; fnIdx [4nF];
 * owner/neighbor [nF]; cfOff [nC+1]; cfIdx [6nC].  Returns nF.
 */
int64_t orc_cartesian_topology(int Nx, int Ny, int Nz, double ex, double ey, double ez, double *nx,
                               double *ny, double *nz, int32_t *fnOff, int64_t *fnIdx, int64_t *owner,
                               int64_t *neighbor, int32_t *cfOff, int64_t *cfIdx)
{
    const double dx = ex / Nx, dy = ey / Ny, dz = ez / Nz;
    const int64_t Px = Nx + 1, Py = Ny + 1, Pz = Nz + 1;
    int64_t p = 0;
    for (int64_t k = 0; k < Pz; ++k)
        for (int64_t j = 0; j < Py; ++j)
            for (int64_t i = 0; i < Px; ++i) {
                nx[p] = 0.0 + (double)(int)i * dx;
                ny[p] = 0.0 + (double)(int)j * dy;
                nz[p] = 0.0 + (double)(int)k * dz;
                ++p;
            }
    const int64_t nC = (int64_t)Nx * Ny * Nz;
    const int64_t maxF = 6 * nC;
    /* hash table of face ids keyed by the face's sorted node tuple (the key
     * of a stored face is recomputed from its node list) */
    int64_t cap = 1;
    while (cap < 2 * maxF)
        cap <<= 1;
    int64_t *hval = (int64_t *)xmalloc((size_t)cap * sizeof(int64_t));
    for (int64_t s = 0; s < cap; ++s)
        hval[s] = -1;
    int64_t nF = 0, ncf = 0;
    int64_t c = 0;
    cfOff[0] = 0;
    for (int64_t k = 0; k < Nz; ++k)
        for (int64_t j = 0; j < Ny; ++j)
            for (int64_t i = 0; i < Nx; ++i, ++c) {
#define PID(a, b, d) ((((d) * Py) + (b)) * Px + (a))
                const int64_t n0 = PID(i, j, k), n1 = PID(i + 1, j, k), n2 = PID(i + 1, j + 1, k),
                              n3 = PID(i, j + 1, k), n4 = PID(i, j, k + 1), n5 = PID(i + 1, j, k + 1),
                              n6 = PID(i + 1, j + 1, k + 1), n7 = PID(i, j + 1, k + 1);
#undef PID
                const int64_t fv[6][4] = {{n0, n3, n2, n1}, {n4, n5, n6, n7}, {n0, n1, n5, n4},
                                          {n3, n7, n6, n2}, {n0, n4, n7, n3}, {n1, n2, n6, n5}};
                for (int q = 0; q < 6; ++q) {
                    int64_t key[4] = {fv[q][0], fv[q][1], fv[q][2], fv[q][3]};
                    sort4(key);
                    uint64_t h = 1469598103934665603ull;
                    for (int t = 0; t < 4; ++t)
                        h = (h ^ (uint64_t)key[t]) * 1099511628211ull;
                    int64_t s = (int64_t)(h & (uint64_t)(cap - 1));
                    for (;;) {
                        const int64_t cand = hval[s];
                        if (cand < 0) {
                            /* new face */
                            const int64_t fid = nF++;
                            hval[s] = fid;
                            fnOff[fid] = (int32_t)(4 * fid);
                            for (int t = 0; t < 4; ++t)
                                fnIdx[4 * fid + t] = fv[q][t];
                            owner[fid] = c;
                            neighbor[fid] = ORC_BOUNDARY;
                            cfIdx[ncf++] = fid;
                            break;
                        }
                        int64_t ck[4] = {fnIdx[4 * cand], fnIdx[4 * cand + 1], fnIdx[4 * cand + 2],
                                         fnIdx[4 * cand + 3]};
                        sort4(ck);
                        if (memcmp(ck, key, sizeof(key)) == 0) {
                            neighbor[cand] = c;
                            cfIdx[ncf++] = cand;
                            break;
                        }
                        s = (s + 1) & (cap - 1);
                    }
                }
                cfOff[c + 1] = (int32_t)ncf;
            }
    fnOff[nF] = (int32_t)(4 * nF);
    free(hval);
    return nF;
}

/*
 * Face areas/centroids and cell volumes/centroids.
 * Follows Mesh::compute_geometry (src/meshing/MeshStorage.cpp:21-97):
 * face centroid = node average (sum then * 1/n); area = sum over the fan of
 * 0.5 * (pa-c) x (pb-c); V = sum sgn*(xf.af)/3; C = sum xf*dv*(3/4) / V.
 */
void orc_compute_geometry(int64_t nC, int64_t nF, const double *nx, const double *ny, const double *nz,
                          const int32_t *fnOff, const int64_t *fnIdx, const int64_t *owner,
                          const int32_t *cfOff, const int64_t *cfIdx, double *ax, double *ay, double *az,
                          double *fcx, double *fcy, double *fcz, double *vol, double *ccx, double *ccy,
                          double *ccz)
{
    for (int64_t f = 0; f < nF; ++f) {
        ax[f] = ay[f] = az[f] = 0.0;
        fcx[f] = fcy[f] = fcz[f] = 0.0;
        const int32_t s = fnOff[f], e = fnOff[f + 1];
        if (e - s < 3)
            continue;
        double cx = 0.0, cy = 0.0, cz = 0.0;
        for (int32_t i = s; i < e; ++i) {
            const int64_t n = fnIdx[i];
            cx += nx[n];
            cy += ny[n];
            cz += nz[n];
        }
        const double inv = 1.0 / (double)(e - s);
        cx *= inv;
        cy *= inv;
        cz *= inv;
        fcx[f] = cx;
        fcy[f] = cy;
        fcz[f] = cz;
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int32_t i = s; i < e; ++i) {
            const int64_t a = fnIdx[i];
            const int64_t b = fnIdx[(i + 1 < e) ? i + 1 : s];
            const double pax = nx[a] - cx, pay = ny[a] - cy, paz = nz[a] - cz;
            const double pbx = nx[b] - cx, pby = ny[b] - cy, pbz = nz[b] - cz;
            const double crx = pay * pbz - paz * pby;
            const double cry = paz * pbx - pax * pbz;
            const double crz = pax * pby - pay * pbx;
            sx = sx + crx * 0.5;
            sy = sy + cry * 0.5;
            sz = sz + crz * 0.5;
        }
        ax[f] = sx;
        ay[f] = sy;
        az[f] = sz;
    }
    for (int64_t c = 0; c < nC; ++c) {
        double V = 0.0, wx = 0.0, wy = 0.0, wz = 0.0;
        for (int32_t i = cfOff[c]; i < cfOff[c + 1]; ++i) {
            const int64_t f = cfIdx[i];
            const double sgn = (owner[f] == c) ? 1.0 : -1.0;
            const double d = fcx[f] * ax[f] + fcy[f] * ay[f] + fcz[f] * az[f];
            const double dv = sgn * d / 3.0;
            V += dv;
            wx = wx + fcx[f] * dv * (3.0 / 4.0);
            wy = wy + fcy[f] * dv * (3.0 / 4.0);
            wz = wz + fcz[f] * dv * (3.0 / 4.0);
        }
        vol[c] = V;
        ccx[c] = ccy[c] = ccz[c] = 0.0;
        if (V != 0.0) {
            ccx[c] = wx / V;
            ccy[c] = wy / V;
            ccz[c] = wz / V;
        }
    }
}

/*
 * Boundary zones by face centroid, tol 1e-9, origin 0.
 * Follows CartesianMesher::generate (src/meshing/CartesianMesher.cpp:60-89):
 * interior faces 0; xMin=1 xMax=2 yMin=3 yMax=4 zMin=5 zMax=6; a boundary
 * face matching none keeps the ConnectivityBuilder default 1
 * (src/meshing/Connectivity.cpp:108-110).
 */
void orc_classify_zones(int64_t nF, const int64_t *neighbor, const double *fcx, const double *fcy,
                        const double *fcz, double ex, double ey, double ez, uint32_t *zone)
{
    const double tol = 1e-9;
    for (int64_t f = 0; f < nF; ++f) {
        if (neighbor[f] != ORC_BOUNDARY) {
            zone[f] = 0;
            continue;
        }
        const double cx = fcx[f], cy = fcy[f], cz = fcz[f];
        uint32_t z = 1;
        if (fabs(cx - 0.0) < tol)
            z = 1;
        else if (fabs(cx - (0.0 + ex)) < tol)
            z = 2;
        else if (fabs(cy - 0.0) < tol)
            z = 3;
        else if (fabs(cy - (0.0 + ey)) < tol)
            z = 4;
        else if (fabs(cz - 0.0) < tol)
            z = 5;
        else if (fabs(cz - (0.0 + ez)) < tol)
            z = 6;
        zone[f] = z;
    }
}

/* ------------------------------------------------------------------ RCM */

static int64_t bandwidth(int64_t nF, const int64_t *owner, const int64_t *neighbor)
{
    int64_t bw = 0;
    for (int64_t f = 0; f < nF; ++f) {
        if (neighbor[f] == ORC_BOUNDARY)
            continue;
        const int64_t d = owner[f] > neighbor[f] ? owner[f] - neighbor[f] : neighbor[f] - owner[f];
        if (d > bw)
            bw = d;
    }
    return bw;
}

static int cmp_i64(const void *a, const void *b)
{
    const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/*
 * Reverse Cuthill-McKee renumbering, in place.
 * Follows renumber_cells_cuthill_mckee (src/meshing/MeshOps.cpp:547-676):
 * adjacency from interior faces (sorted, unique); repeatedly seed BFS at the
 * lowest-index unvisited cell of minimum degree; enqueue unvisited
 * neighbours in ascending id, then stably ordered by ascending degree (the
 * reference's std::sort on <=16 elements is an insertion sort, hence
 * stable); reverse the visit order; permute cell volume/centroids and the
 * cell->face CSR; remap face owner/neighbor.  Face arrays keep their order.
 * Writes newPos[old] = new and stats {bwBefore, bwAfter, permuted}.
 */
void orc_rcm(int64_t nC, int64_t nF, int64_t *owner, int64_t *neighbor, double *vol, double *ccx,
             double *ccy, double *ccz, int32_t *cfOff, int64_t *cfIdx, int64_t *newPos, int64_t *stats)
{
    stats[0] = bandwidth(nF, owner, neighbor);
    if (nC == 0) {
        stats[1] = stats[2] = 0;
        return;
    }
    int64_t *deg = (int64_t *)calloc((size_t)nC + 1, sizeof(int64_t));
    for (int64_t f = 0; f < nF; ++f) {
        if (neighbor[f] == ORC_BOUNDARY)
            continue;
        const int64_t a = owner[f], b = neighbor[f];
        if (a >= nC || b >= nC)
            continue;
        deg[a]++;
        deg[b]++;
    }
    int64_t *aoff = (int64_t *)xmalloc(((size_t)nC + 1) * sizeof(int64_t));
    aoff[0] = 0;
    for (int64_t c = 0; c < nC; ++c)
        aoff[c + 1] = aoff[c] + deg[c];
    int64_t *adj = (int64_t *)xmalloc((size_t)(aoff[nC] ? aoff[nC] : 1) * sizeof(int64_t));
    int64_t *fill = (int64_t *)calloc((size_t)nC, sizeof(int64_t));
    for (int64_t f = 0; f < nF; ++f) {
        if (neighbor[f] == ORC_BOUNDARY)
            continue;
        const int64_t a = owner[f], b = neighbor[f];
        if (a >= nC || b >= nC)
            continue;
        adj[aoff[a] + fill[a]++] = b;
        adj[aoff[b] + fill[b]++] = a;
    }
    /* sort + unique per cell; degree = unique count */
    for (int64_t c = 0; c < nC; ++c) {
        int64_t *v = adj + aoff[c];
        const int64_t m = fill[c];
        qsort(v, (size_t)m, sizeof(int64_t), cmp_i64);
        int64_t u = 0;
        for (int64_t t = 0; t < m; ++t)
            if (u == 0 || v[u - 1] != v[t])
                v[u++] = v[t];
        deg[c] = u;
    }
    uint8_t *seen = (uint8_t *)calloc((size_t)nC, 1);
    int64_t *order = (int64_t *)xmalloc((size_t)nC * sizeof(int64_t));
    int64_t *queue = (int64_t *)xmalloc((size_t)nC * sizeof(int64_t));
    int64_t *nb = (int64_t *)xmalloc(((size_t)nC + 1) * sizeof(int64_t));
    int64_t no = 0;
    while (no < nC) {
        int64_t seed = -1;
        for (int64_t c = 0; c < nC; ++c) {
            if (seen[c])
                continue;
            if (seed < 0 || deg[c] < deg[seed])
                seed = c;
        }
        if (seed < 0)
            break;
        int64_t qh = 0, qt = 0;
        queue[qt++] = seed;
        seen[seed] = 1;
        while (qh < qt) {
            const int64_t c = queue[qh++];
            order[no++] = c;
            int64_t m = 0;
            for (int64_t t = 0; t < deg[c]; ++t) {
                const int64_t n = adj[aoff[c] + t];
                if (!seen[n]) {
                    nb[m++] = n;
                    seen[n] = 1;
                }
            }
            for (int64_t t = 1; t < m; ++t) { /* stable insertion sort by degree */
                const int64_t v = nb[t];
                int64_t s = t - 1;
                while (s >= 0 && deg[nb[s]] > deg[v]) {
                    nb[s + 1] = nb[s];
                    --s;
                }
                nb[s + 1] = v;
            }
            for (int64_t t = 0; t < m; ++t)
                queue[qt++] = nb[t];
        }
    }
    for (int64_t a = 0, b = no - 1; a < b; ++a, --b) {
        const int64_t t = order[a];
        order[a] = order[b];
        order[b] = t;
    }
    for (int64_t c = 0; c < nC; ++c)
        newPos[c] = -1;
    for (int64_t k = 0; k < no; ++k)
        newPos[order[k]] = k;
    for (int64_t c = 0; c < nC; ++c)
        if (newPos[c] < 0)
            newPos[c] = c;
    double *tmp = (double *)xmalloc((size_t)nC * sizeof(double));
    double *arrs[4] = {vol, ccx, ccy, ccz};
    for (int a = 0; a < 4; ++a) {
        for (int64_t c = 0; c < nC; ++c)
            tmp[newPos[c]] = arrs[a][c];
        memcpy(arrs[a], tmp, (size_t)nC * sizeof(double));
    }
    free(tmp);
    const int64_t ncf = cfOff[nC];
    int32_t *offNew = (int32_t *)xmalloc(((size_t)nC + 1) * sizeof(int32_t));
    int64_t *idxNew = (int64_t *)xmalloc((size_t)(ncf ? ncf : 1) * sizeof(int64_t));
    int64_t w = 0;
    offNew[0] = 0;
    for (int64_t q = 0; q < nC; ++q) {
        const int64_t c = order[q];
        for (int32_t t = cfOff[c]; t < cfOff[c + 1]; ++t)
            idxNew[w++] = cfIdx[t];
        offNew[q + 1] = (int32_t)w;
    }
    memcpy(cfOff, offNew, ((size_t)nC + 1) * sizeof(int32_t));
    memcpy(cfIdx, idxNew, (size_t)ncf * sizeof(int64_t));
    free(offNew);
    free(idxNew);
    for (int64_t f = 0; f < nF; ++f) {
        owner[f] = newPos[owner[f]];
        if (neighbor[f] != ORC_BOUNDARY)
            neighbor[f] = newPos[neighbor[f]];
    }
    stats[1] = bandwidth(nF, owner, neighbor);
    stats[2] = no;
    free(deg);
    free(aoff);
    free(adj);
    free(fill);
    free(seen);
    free(order);
    free(queue);
    free(nb);
}

/* ------------------------------------------------------------------ sparsity + assembly */

/*
 * CSR pattern of the pressure-correction matrix.
 * Follows SimpleAlgorithm::build_sparsity (src/solver/SimpleAlgorithm.cpp:49-98)
 * without periodic twins: row c = sorted unique {c} U {other cell of each of
 * c's faces that is not a boundary}.  With colIdx == NULL only rowPtr is
 * filled; returns nnz.
 */
/* SimpleAlgorithm::build_periodic_pairs (src/solver/SimpleAlgorithm.cpp:101-186):
 * periodicZones[0..nP) are the zones of the Periodic boundary specs in spec
 * order (duplicates kept; a face joins the first listed entry of its zone).
 * Boundary faces are grouped by that entry in face order; entries are paired
 * (0,1), (2,3), ...; the translation is mean(B) - mean(A) of the face
 * centroids (sums in face order, times 1/size); each face of A, in order,
 * takes the face of B whose centroid is nearest to its own plus the
 * translation (squared distance, first minimum in B's order), and
 * twin[a] = b, twin[b] = a -- a later face of A choosing the same b rewrites
 * twin[b].  twin[f] = -1 elsewhere (fewer than two periodic entries: all). */
void orc_periodic_pairs(int64_t nF, const int64_t *neighbor, const uint32_t *zone, const double *fcx,
                        const double *fcy, const double *fcz, int nP, const uint32_t *periodicZones, int32_t *twin)
{
    for (int64_t f = 0; f < nF; ++f)
        twin[f] = -1;
    if (nP < 2)
        return;
    int64_t *cnt = (int64_t *)calloc((size_t)nP + 1, sizeof(int64_t));
    int32_t *grp = (int32_t *)xmalloc((size_t)nF * sizeof(int32_t) + 8);
    for (int64_t f = 0; f < nF; ++f) {
        grp[f] = -1;
        if (neighbor[f] != ORC_BOUNDARY)
            continue;
        for (int i = 0; i < nP; ++i)
            if (periodicZones[i] == zone[f]) {
                grp[f] = i;
                cnt[i + 1]++;
                break;
            }
    }
    for (int i = 0; i < nP; ++i)
        cnt[i + 1] += cnt[i];
    int64_t *list = (int64_t *)xmalloc((size_t)(cnt[nP] + 1) * sizeof(int64_t));
    int64_t *fill = (int64_t *)xmalloc((size_t)(nP + 1) * sizeof(int64_t));
    for (int i = 0; i <= nP; ++i)
        fill[i] = cnt[i];
    for (int64_t f = 0; f < nF; ++f)
        if (grp[f] >= 0)
            list[fill[grp[f]]++] = f;
    for (int z = 0; z + 1 < nP; z += 2) {
        const int64_t *A = list + cnt[z], *B = list + cnt[z + 1];
        const int64_t nA = cnt[z + 1] - cnt[z], nB = cnt[z + 2] - cnt[z + 1];
        if (nA == 0 || nB == 0)
            continue;
        double Ax = 0, Ay = 0, Az = 0, Bx = 0, By = 0, Bz = 0;
        for (int64_t i = 0; i < nA; ++i) {
            Ax += fcx[A[i]];
            Ay += fcy[A[i]];
            Az += fcz[A[i]];
        }
        for (int64_t i = 0; i < nB; ++i) {
            Bx += fcx[B[i]];
            By += fcy[B[i]];
            Bz += fcz[B[i]];
        }
        const double invA = 1.0 / (double)nA, invB = 1.0 / (double)nB;
        const double tx = Bx * invB - Ax * invA, ty = By * invB - Ay * invA, tz = Bz * invB - Az * invA;
        for (int64_t i = 0; i < nA; ++i) {
            const int64_t fa = A[i];
            int64_t best = -1;
            double bestd2 = DBL_MAX;
            const double ax = fcx[fa] + tx, ay = fcy[fa] + ty, az = fcz[fa] + tz;
            for (int64_t j = 0; j < nB; ++j) {
                const int64_t fb = B[j];
                const double d2 = (fcx[fb] - ax) * (fcx[fb] - ax) + (fcy[fb] - ay) * (fcy[fb] - ay) +
                                  (fcz[fb] - az) * (fcz[fb] - az);
                if (d2 < bestd2) {
                    bestd2 = d2;
                    best = fb;
                }
            }
            if (best >= 0) {
                twin[fa] = (int32_t)best;
                twin[best] = (int32_t)fa;
            }
        }
    }
    free(cnt);
    free(grp);
    free(list);
    free(fill);
}

int64_t orc_build_sparsity(int64_t nC, const int64_t *owner, const int64_t *neighbor,
                           const int32_t *cfOff, const int64_t *cfIdx, int32_t *rowPtr, int32_t *colIdx,
                           const int32_t *twin)
{
    int64_t nnz = 0;
    int64_t buf[64];
    rowPtr[0] = 0;
    for (int64_t c = 0; c < nC; ++c) {
        int m = 0;
        buf[m++] = c;
        for (int32_t t = cfOff[c]; t < cfOff[c + 1]; ++t) {
            const int64_t f = cfIdx[t];
            const int64_t oth = (owner[f] == c) ? neighbor[f] : owner[f];
            if (oth != ORC_BOUNDARY) {
                if (m < 64)
                    buf[m++] = oth;
            } else if (twin && twin[f] >= 0 && m < 64) {  /* periodic: the twin face's owner (:71-72) */
                buf[m++] = owner[twin[f]];
            }
        }
        for (int i = 1; i < m; ++i) {
            const int64_t v = buf[i];
            int j = i - 1;
            while (j >= 0 && buf[j] > v) {
                buf[j + 1] = buf[j];
                --j;
            }
            buf[j + 1] = v;
        }
        int u = 0;
        for (int i = 0; i < m; ++i)
            if (u == 0 || buf[u - 1] != buf[i])
                buf[u++] = buf[i];
        if (colIdx)
            for (int i = 0; i < u; ++i)
                colIdx[nnz + i] = (int32_t)buf[i];
        nnz += u;
        rowPtr[c + 1] = (int32_t)nnz;
    }
    return nnz;
}

/* find_col (src/solver/SimpleAlgorithm.cpp:23-29) */
static int32_t find_col(const int32_t *rowPtr, const int32_t *colIdx, int64_t row, int64_t col)
{
    for (int32_t k = rowPtr[row]; k < rowPtr[row + 1]; ++k)
        if (colIdx[k] == col)
            return k;
    return -1;
}

/* add_at (src/solver/SimpleAlgorithm.cpp:30-35) */
static void add_at(const int32_t *rowPtr, const int32_t *colIdx, double *values, int64_t row, int64_t col,
                   double v)
{
    const int32_t k = find_col(rowPtr, colIdx, row, col);
    if (k >= 0)
        values[k] += v;
}

/*
 * Pressure-correction Laplacian, SIMPLE variant, no periodic twins.
 * Follows SimpleAlgorithm::assemble_pressure_correction
 * (src/solver/SimpleAlgorithm.cpp:358-447):
 *   interior face: coef = rho*|A|^2 / max(0.5*(max(aP_o,1e-30)+max(aP_n,1e-30))*|d.A|, 1e-30),
 *                  d = C_n - C_o, added +oo, -on, +nn, -no;
 *   boundary face in a pressure zone (isPressure[zone] != 0, i.e. PressureOutlet
 *                  or PressureInlet): coef = rho*|A|^2 / max(max(aP_o,1e-30)*|d.A|, 1e-30),
 *                  d = face centroid - C_o, added +oo, anyDirichlet = 1;
 *   every face: rhs_o -= phi_f, rhs_n += phi_f (interior);
 *   no Dirichlet face: A[0,0] *= 1e6 and rhs[0] = 0.
 * values/rhs are overwritten.  Returns anyDirichlet.
 */
int orc_assemble(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *ax,
                 const double *ay, const double *az, const double *fcx, const double *fcy, const double *fcz,
                 const uint32_t *zone, const double *ccx, const double *ccy, const double *ccz,
                 const uint8_t *isPressure, int nZones, double rho, const double *aP, const double *phi,
                 const int32_t *rowPtr, const int32_t *colIdx, double *values, double *rhs, const int32_t *twin)
{
    const int64_t nnz = rowPtr[nC];
    for (int64_t k = 0; k < nnz; ++k)
        values[k] = 0.0;
    for (int64_t c = 0; c < nC; ++c)
        rhs[c] = 0.0;
    int anyDirichlet = 0;
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        const double Ax = ax[f], Ay = ay[f], Az = az[f];
        const double Amag2 = Ax * Ax + Ay * Ay + Az * Az;
        if (n != ORC_BOUNDARY) {
            const double dx = ccx[n] - ccx[o];
            const double dy = ccy[n] - ccy[o];
            const double dz = ccz[n] - ccz[o];
            const double ddotA = fabs(dx * Ax + dy * Ay + dz * Az);
            const double dOwn = STD_MAX(aP[o], 1e-30), dNbr = STD_MAX(aP[n], 1e-30);
            const double aPf = 0.5 * (dOwn + dNbr);
            const double den = aPf * ddotA;
            const double coef = rho * Amag2 / STD_MAX(den, 1e-30);
            add_at(rowPtr, colIdx, values, o, o, coef);
            add_at(rowPtr, colIdx, values, o, n, -coef);
            add_at(rowPtr, colIdx, values, n, n, coef);
            add_at(rowPtr, colIdx, values, n, o, -coef);
        } else {
            const uint32_t zz = zone[f];
            if (twin && twin[f] >= 0) {  /* periodic face (:411-419): owner and the twin face's owner */
                const int64_t tw = owner[twin[f]];
                const double dx = fcx[f] - ccx[o];
                const double dy = fcy[f] - ccy[o];
                const double dz = fcz[f] - ccz[o];
                const double ddotA = fabs(dx * Ax + dy * Ay + dz * Az);
                const double den = STD_MAX(aP[o], 1e-30) * ddotA;
                const double coef = rho * Amag2 / STD_MAX(den, 1e-30);
                add_at(rowPtr, colIdx, values, o, o, coef);
                add_at(rowPtr, colIdx, values, o, tw, -coef);
            } else if ((int)zz < nZones && isPressure[zz]) {
                const double dx = fcx[f] - ccx[o];
                const double dy = fcy[f] - ccy[o];
                const double dz = fcz[f] - ccz[o];
                const double ddotA = fabs(dx * Ax + dy * Ay + dz * Az);
                const double den = STD_MAX(aP[o], 1e-30) * ddotA;
                const double coef = rho * Amag2 / STD_MAX(den, 1e-30);
                add_at(rowPtr, colIdx, values, o, o, coef);
                anyDirichlet = 1;
            }
        }
        rhs[o] -= phi[f];
        if (n != ORC_BOUNDARY)
            rhs[n] += phi[f];
    }
    if (!anyDirichlet && nC > 0) {
        const int32_t kd = find_col(rowPtr, colIdx, 0, 0);
        if (kd >= 0)
            values[kd] *= 1.0e6;
        rhs[0] = 0.0;
    }
    return anyDirichlet;
}

/* ------------------------------------------------------------------ BLAS-1 + SpMV */

/* SIMPLEC denominator, SimpleAlgorithm.cpp:380-390 and 401-409: per cell
 * max(aP_c - sum_{k != c} |a_mom,ck|, 1e-30), the sum in column order from
 * 0.0.  Passing den as aP to orc_assemble gives the SIMPLEC system, because
 * the assembly's own max(aP, 1e-30) leaves den unchanged. */
void orc_simplec_denominator(int64_t nC, const int32_t *rowPtr, const int32_t *colIdx, const double *mom,
                             const double *aP, double *den)
{
    for (int64_t c = 0; c < nC; ++c) {
        double sumOff = 0.0;
        for (int32_t k = rowPtr[c]; k < rowPtr[c + 1]; ++k)
            if (colIdx[k] != (int32_t)c)
                sumOff += fabs(mom[k]);
        den[c] = STD_MAX(aP[c] - sumOff, 1e-30);
    }
}

/* dot / norm2 / axpy (src/solver/LinearSolvers.cpp:25-43) */
double orc_dot(int64_t n, const double *a, const double *b)
{
    double s = 0;
    for (int64_t i = 0; i < n; ++i)
        s += a[i] * b[i];
    return s;
}

static double norm2(int64_t n, const double *a) { return sqrt(orc_dot(n, a, a)); }

static void axpy(int64_t n, double alpha, const double *x, double *y)
{
    for (int64_t i = 0; i < n; ++i)
        y[i] += alpha * x[i];
}

/* CSRMatrix::spmv (src/solver/CSRMatrix.hpp:24-35) */
void orc_spmv(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, const double *x,
              double *y)
{
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int32_t k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            s += values[k] * x[colIdx[k]];
        y[i] = s;
    }
}

/* ------------------------------------------------------------------ preconditioners */

/* JacobiPreconditioner::setup (src/solver/LinearSolvers.cpp:54-65): first
 * diagonal entry of each row, 1/a_ii, or 1.0 when zero or missing. */
void orc_jacobi_setup(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values,
                      double *invDiag)
{
    for (int64_t i = 0; i < n; ++i) {
        invDiag[i] = 1.0;
        for (int32_t k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                invDiag[i] = (values[k] != 0.0) ? 1.0 / values[k] : 1.0;
                break;
            }
    }
}

/* ILU0Preconditioner::setup (src/solver/LinearSolvers.cpp:81-122): IKJ
 * in-place ILU(0) on the pattern; rows below a missing diagonal or a zero
 * pivot are skipped for that k.  lu and diagPtr are outputs. */
void orc_ilu0_setup(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, double *lu,
                    int32_t *diagPtr)
{
    memcpy(lu, values, (size_t)rowPtr[n] * sizeof(double));
    for (int64_t i = 0; i < n; ++i) {
        diagPtr[i] = -1;
        for (int32_t k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                diagPtr[i] = k;
                break;
            }
    }
    for (int64_t i = 1; i < n; ++i) {
        for (int32_t kp = rowPtr[i]; kp < rowPtr[i + 1]; ++kp) {
            const int32_t k = colIdx[kp];
            if (k >= i)
                break;
            if (diagPtr[k] < 0)
                continue;
            const double piv = lu[diagPtr[k]];
            if (piv == 0.0)
                continue;
            const double m = lu[kp] / piv;
            lu[kp] = m;
            for (int32_t jp = diagPtr[k] + 1; jp < rowPtr[k + 1]; ++jp) {
                const int32_t j = colIdx[jp];
                for (int32_t qp = kp + 1; qp < rowPtr[i + 1]; ++qp) {
                    if (colIdx[qp] == j) {
                        lu[qp] -= m * lu[jp];
                        break;
                    }
                    if (colIdx[qp] > j)
                        break;
                }
            }
        }
    }
}

/* ILU0Preconditioner::apply (src/solver/LinearSolvers.cpp:123-151): forward
 * unit-lower sweep, then backward sweep z_i = s/u_ii (or s when u_ii is
 * zero or missing).  y is caller scratch of length n. */
void orc_ilu0_apply(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *lu,
                    const int32_t *diagPtr, const double *r, double *z, double *y)
{
    for (int64_t i = 0; i < n; ++i) {
        double s = r[i];
        for (int32_t kp = rowPtr[i]; kp < rowPtr[i + 1]; ++kp) {
            const int32_t j = colIdx[kp];
            if (j >= i)
                break;
            s -= lu[kp] * y[j];
        }
        y[i] = s;
    }
    for (int64_t i = 0; i < n; ++i)
        z[i] = 0.0;
    for (int64_t i = n - 1; i >= 0; --i) {
        double s = y[i];
        const int32_t kd = diagPtr[i];
        for (int32_t kp = kd + 1; kp < rowPtr[i + 1]; ++kp)
            s -= lu[kp] * z[colIdx[kp]];
        z[i] = (kd >= 0 && lu[kd] != 0.0) ? s / lu[kd] : s;
    }
}

/* SsorPreconditioner::setup (src/solver/LinearSolvers.cpp:168-186): the first
 * diagonal entry of each row, diag = a_ii and invDiag = 1/a_ii (1.0 when the
 * entry is zero); diag = invDiag = 1.0 when the row has none. */
void orc_ssor_setup(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, double *diag,
                    double *invDiag)
{
    for (int64_t i = 0; i < n; ++i) {
        diag[i] = 1.0;
        invDiag[i] = 1.0;
        for (int32_t k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                diag[i] = values[k];
                invDiag[i] = (values[k] != 0.0) ? 1.0 / values[k] : 1.0;
                break;
            }
    }
}

/* SsorPreconditioner::apply (src/solver/LinearSolvers.cpp:188-231):
 *   forward   y_i = (w r_i - sum_{j<i} (w a_ij) y_j) invDiag_i  (columns
 *             ascending, stopping at the first j >= i);
 *   scale     v_i = (diag_i y_i) / w;
 *   backward  z_i = ((v_i - sum_{j>i} a_ij z_j) w) invDiag_i, rows n-1 .. 0;
 *   z *= (2 - w).
 * make_preconditioner builds it with w = 1 (:247-248).  y, v: caller scratch. */
void orc_ssor_apply(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values,
                    const double *diag, const double *invDiag, double omega, const double *r, double *z, double *y,
                    double *v)
{
    for (int64_t i = 0; i < n; ++i)
        y[i] = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double s = omega * r[i];
        for (int32_t kp = rowPtr[i]; kp < rowPtr[i + 1]; ++kp) {
            const int32_t j = colIdx[kp];
            if (j >= i)
                break;
            s -= omega * values[kp] * y[j];
        }
        y[i] = s * invDiag[i];
    }
    const double scale = (2.0 - omega);
    for (int64_t i = 0; i < n; ++i)
        v[i] = diag[i] * y[i] / omega;
    for (int64_t i = 0; i < n; ++i)
        z[i] = 0.0;
    for (int64_t i = n - 1; i >= 0; --i) {
        double s = v[i];
        for (int32_t kp = rowPtr[i]; kp < rowPtr[i + 1]; ++kp) {
            const int32_t j = colIdx[kp];
            if (j <= i)
                continue;
            s -= values[kp] * z[j];
        }
        z[i] = s * omega * invDiag[i];
    }
    for (int64_t i = 0; i < n; ++i)
        z[i] *= scale;
}

/* ------------------------------------------------------------------ AMG */

/*
 * AMGPreconditioner (src/solver/AMGPreconditioner.cpp), with the defaults
 * make_preconditioner constructs it with (theta 0.25, 10 levels, one pre- and
 * one post-sweep, coarse threshold 32; AMGPreconditioner.hpp:39-43).
 * Ruge-Stueben: strong couplings -a_ij >= theta max_k(-a_ik) (:43-67),
 * greedy C/F split by the largest lambda = |S_i^T| (+1 for each new F point
 * that i influences), the smallest index on ties (:69-113), direct
 * interpolation P_ij = -a_ij / a_ii onto C neighbours (:115-151), R = P^T
 * (:153-174), Galerkin A_c = R (A P) with each product row accumulated in the
 * order its terms are met and its columns sorted (:176-246), a dense LU with
 * partial pivoting of the coarsest operator whose row swaps are not applied to
 * the right-hand side in the solve, as the reference does (:296-322,
 * :354-377), and a V-cycle of symmetric Gauss-Seidel sweeps (:326-352,
 * :379-416) from z = 0 (:418-427).
 */
typedef struct {
    int32_t n;
    int32_t *rp, *ci;
    double *v;
} OrcCsr;

#define ORC_AMG_MAX_LEVELS 10

typedef struct {
    int nlev;
    OrcCsr A[ORC_AMG_MAX_LEVELS], P[ORC_AMG_MAX_LEVELS], R[ORC_AMG_MAX_LEVELS];
    int32_t coarseN;
    double *lu;
} OrcAmg;

static double csr_diag(const OrcCsr *A, int32_t i)
{
    for (int32_t k = A->rp[i]; k < A->rp[i + 1]; ++k)
        if (A->ci[k] == i)
            return A->v[k];
    return 0.0;
}

static void csr_free(OrcCsr *A)
{
    free(A->rp);
    free(A->ci);
    free(A->v);
    memset(A, 0, sizeof(*A));
}

/* strong[i] as a CSR list (sp, sj) */
static void amg_strong(const OrcCsr *A, double theta, int32_t **sp, int32_t **sj)
{
    const int32_t n = A->n;
    int32_t *p = (int32_t *)xmalloc(((size_t)n + 1) * sizeof(int32_t));
    int32_t *j = (int32_t *)xmalloc(((size_t)A->rp[n] + 1) * sizeof(int32_t));
    p[0] = 0;
    for (int32_t i = 0; i < n; ++i) {
        p[i + 1] = p[i];
        double maxOff = 0.0;
        for (int32_t k = A->rp[i]; k < A->rp[i + 1]; ++k) {
            if (A->ci[k] == i)
                continue;
            maxOff = STD_MAX(maxOff, -A->v[k]);
        }
        if (maxOff <= 0.0)
            continue;
        const double thr = theta * maxOff;
        for (int32_t k = A->rp[i]; k < A->rp[i + 1]; ++k) {
            if (A->ci[k] == i)
                continue;
            if (-A->v[k] >= thr)
                j[p[i + 1]++] = A->ci[k];
        }
    }
    *sp = p;
    *sj = j;
}

/* cf[i] = 1 C point, 0 F point; returns the number of C points. */
static int32_t amg_coarsen(int32_t n, const int32_t *sp, const int32_t *sj, int32_t *cf)
{
    /* S^T, rows in ascending i as the reference appends them */
    int32_t *tp = (int32_t *)xmalloc(((size_t)n + 1) * sizeof(int32_t));
    int32_t *tj = (int32_t *)xmalloc(((size_t)sp[n] + 1) * sizeof(int32_t));
    int32_t *fill = (int32_t *)xmalloc(((size_t)n + 1) * sizeof(int32_t));
    int32_t *lambda = (int32_t *)xmalloc(((size_t)n + 1) * sizeof(int32_t));
    memset(tp, 0, ((size_t)n + 1) * sizeof(int32_t));
    for (int32_t q = 0; q < sp[n]; ++q)
        ++tp[sj[q] + 1];
    for (int32_t i = 0; i < n; ++i)
        tp[i + 1] += tp[i];
    memcpy(fill, tp, (size_t)n * sizeof(int32_t));
    for (int32_t i = 0; i < n; ++i)
        for (int32_t q = sp[i]; q < sp[i + 1]; ++q)
            tj[fill[sj[q]]++] = i;
    for (int32_t i = 0; i < n; ++i) {
        cf[i] = -1;
        lambda[i] = tp[i + 1] - tp[i];
    }
    for (;;) {
        int32_t best = -1, bestLam = -1;
        for (int32_t i = 0; i < n; ++i)
            if (cf[i] < 0 && lambda[i] > bestLam) {
                bestLam = lambda[i];
                best = i;
            }
        if (best < 0)
            break;
        cf[best] = 1;
        for (int32_t q = tp[best]; q < tp[best + 1]; ++q) {
            const int32_t j = tj[q];
            if (cf[j] < 0) {
                cf[j] = 0;
                for (int32_t r = sp[j]; r < sp[j + 1]; ++r)
                    if (cf[sj[r]] < 0)
                        ++lambda[sj[r]];
            }
        }
        lambda[best] = -1;
    }
    int32_t nc = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (cf[i] < 0)
            cf[i] = 1;
        nc += cf[i] == 1;
    }
    free(tp);
    free(tj);
    free(fill);
    free(lambda);
    return nc;
}

static void amg_prolongation(const OrcCsr *A, const int32_t *cf, OrcCsr *P)
{
    const int32_t nf = A->n;
    int32_t *cid = (int32_t *)xmalloc(((size_t)nf + 1) * sizeof(int32_t));
    int32_t nc = 0;
    for (int32_t i = 0; i < nf; ++i)
        cid[i] = cf[i] == 1 ? nc++ : -1;
    P->n = nf;
    P->rp = (int32_t *)xmalloc(((size_t)nf + 1) * sizeof(int32_t));
    P->ci = (int32_t *)xmalloc(((size_t)A->rp[nf] + (size_t)nf + 1) * sizeof(int32_t));
    P->v = (double *)xmalloc(((size_t)A->rp[nf] + (size_t)nf + 1) * sizeof(double));
    P->rp[0] = 0;
    int32_t e = 0;
    for (int32_t i = 0; i < nf; ++i) {
        if (cf[i] == 1) {
            P->ci[e] = cid[i];
            P->v[e++] = 1.0;
        } else {
            const double dii = csr_diag(A, i);
            const double inv = (fabs(dii) > 1e-30) ? 1.0 / dii : 0.0;
            for (int32_t k = A->rp[i]; k < A->rp[i + 1]; ++k) {
                const int32_t j = A->ci[k];
                if (j == i || cf[j] != 1)
                    continue;
                P->ci[e] = cid[j];
                P->v[e++] = -A->v[k] * inv;
            }
        }
        P->rp[i + 1] = e;
    }
    free(cid);
}

static void amg_transpose(const OrcCsr *M, int32_t newRows, OrcCsr *T)
{
    const int32_t nnz = M->rp[M->n];
    T->n = newRows;
    T->rp = (int32_t *)xmalloc(((size_t)newRows + 1) * sizeof(int32_t));
    T->ci = (int32_t *)xmalloc(((size_t)nnz + 1) * sizeof(int32_t));
    T->v = (double *)xmalloc(((size_t)nnz + 1) * sizeof(double));
    memset(T->rp, 0, ((size_t)newRows + 1) * sizeof(int32_t));
    for (int32_t k = 0; k < nnz; ++k)
        ++T->rp[M->ci[k] + 1];
    for (int32_t i = 0; i < newRows; ++i)
        T->rp[i + 1] += T->rp[i];
    int32_t *cur = (int32_t *)xmalloc(((size_t)newRows + 1) * sizeof(int32_t));
    memset(cur, 0, ((size_t)newRows + 1) * sizeof(int32_t));
    for (int32_t i = 0; i < M->n; ++i)
        for (int32_t k = M->rp[i]; k < M->rp[i + 1]; ++k) {
            const int32_t c = M->ci[k];
            const int32_t dst = T->rp[c] + cur[c]++;
            T->ci[dst] = i;
            T->v[dst] = M->v[k];
        }
    free(cur);
}

static int cmp_i32(const void *a, const void *b)
{
    const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* C = L * Rm, each row accumulated in the order its terms are met, columns
 * sorted; ncols columns. */
static void amg_matmul(const OrcCsr *L, const OrcCsr *Rm, int32_t ncols, OrcCsr *C)
{
    const int32_t n = L->n;
    double *acc = (double *)xmalloc(((size_t)ncols + 1) * sizeof(double));
    int32_t *mark = (int32_t *)xmalloc(((size_t)ncols + 1) * sizeof(int32_t));
    int32_t *cols = (int32_t *)xmalloc(((size_t)ncols + 1) * sizeof(int32_t));
    for (int32_t c = 0; c < ncols; ++c)
        mark[c] = -1;
    size_t cap = (size_t)L->rp[n] * 4 + 16, e = 0;
    C->n = n;
    C->rp = (int32_t *)xmalloc(((size_t)n + 1) * sizeof(int32_t));
    C->ci = (int32_t *)xmalloc(cap * sizeof(int32_t));
    C->v = (double *)xmalloc(cap * sizeof(double));
    C->rp[0] = 0;
    for (int32_t i = 0; i < n; ++i) {
        int32_t nc = 0;
        for (int32_t k = L->rp[i]; k < L->rp[i + 1]; ++k) {
            const int32_t j = L->ci[k];
            const double lij = L->v[k];
            for (int32_t kp = Rm->rp[j]; kp < Rm->rp[j + 1]; ++kp) {
                const int32_t c = Rm->ci[kp];
                const double v = lij * Rm->v[kp];
                if (mark[c] != i) {
                    mark[c] = i;
                    acc[c] = v;
                    cols[nc++] = c;
                } else {
                    acc[c] += v;
                }
            }
        }
        qsort(cols, (size_t)nc, sizeof(int32_t), cmp_i32);
        if (e + (size_t)nc > cap) {
            while (e + (size_t)nc > cap)
                cap *= 2;
            C->ci = (int32_t *)realloc(C->ci, cap * sizeof(int32_t));
            C->v = (double *)realloc(C->v, cap * sizeof(double));
        }
        for (int32_t q = 0; q < nc; ++q) {
            C->ci[e] = cols[q];
            C->v[e++] = acc[cols[q]];
        }
        C->rp[i + 1] = (int32_t)e;
    }
    free(acc);
    free(mark);
    free(cols);
}

void orc_amg_free(OrcAmg *M)
{
    for (int l = 0; l < ORC_AMG_MAX_LEVELS; ++l) {
        csr_free(&M->A[l]);
        csr_free(&M->P[l]);
        csr_free(&M->R[l]);
    }
    free(M->lu);
    M->lu = NULL;
    M->nlev = 0;
}

void orc_amg_setup(OrcAmg *M, int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values)
{
    const double theta = 0.25;
    const int maxLevels = ORC_AMG_MAX_LEVELS, coarseThreshold = 32;
    memset(M, 0, sizeof(*M));
    OrcCsr *A0 = &M->A[0];
    A0->n = (int32_t)n;
    A0->rp = (int32_t *)xmalloc(((size_t)n + 1) * sizeof(int32_t));
    A0->ci = (int32_t *)xmalloc(((size_t)rowPtr[n] + 1) * sizeof(int32_t));
    A0->v = (double *)xmalloc(((size_t)rowPtr[n] + 1) * sizeof(double));
    memcpy(A0->rp, rowPtr, ((size_t)n + 1) * sizeof(int32_t));
    memcpy(A0->ci, colIdx, (size_t)rowPtr[n] * sizeof(int32_t));
    memcpy(A0->v, values, (size_t)rowPtr[n] * sizeof(double));
    M->nlev = 1;
    for (int lvl = 0; lvl < maxLevels - 1; ++lvl) {
        OrcCsr *Af = &M->A[M->nlev - 1];
        const int32_t nf = Af->n;
        if (nf <= coarseThreshold)
            break;
        int32_t *sp, *sj;
        amg_strong(Af, theta, &sp, &sj);
        int32_t *cf = (int32_t *)xmalloc(((size_t)nf + 1) * sizeof(int32_t));
        const int32_t nc = amg_coarsen(nf, sp, sj, cf);
        free(sp);
        free(sj);
        if (nc == 0 || nc >= nf) {
            free(cf);
            break;
        }
        OrcCsr *P = &M->P[M->nlev - 1], *R = &M->R[M->nlev - 1];
        amg_prolongation(Af, cf, P);
        free(cf);
        amg_transpose(P, nc, R);
        OrcCsr AP;
        int32_t ncols = 0;
        for (int32_t q = 0; q < P->rp[P->n]; ++q)
            ncols = P->ci[q] + 1 > ncols ? P->ci[q] + 1 : ncols;
        amg_matmul(Af, P, ncols, &AP);
        amg_matmul(R, &AP, ncols, &M->A[M->nlev]);
        csr_free(&AP);
        M->nlev += 1;
    }
    const OrcCsr *Ac = &M->A[M->nlev - 1];
    const int32_t cn = Ac->n;
    M->coarseN = cn;
    M->lu = (double *)xmalloc((size_t)cn * (size_t)cn * sizeof(double) + 8);
    double *LU = M->lu;
    memset(LU, 0, (size_t)cn * (size_t)cn * sizeof(double));
    for (int32_t i = 0; i < cn; ++i)
        for (int32_t k = Ac->rp[i]; k < Ac->rp[i + 1]; ++k)
            LU[(size_t)i * cn + Ac->ci[k]] = Ac->v[k];
    for (int32_t k = 0; k < cn; ++k) {
        int32_t piv = k;
        double pivVal = fabs(LU[(size_t)k * cn + k]);
        for (int32_t i = k + 1; i < cn; ++i) {
            const double v = fabs(LU[(size_t)i * cn + k]);
            if (v > pivVal) {
                pivVal = v;
                piv = i;
            }
        }
        if (pivVal < 1e-30)
            continue;
        if (piv != k)
            for (int32_t j = 0; j < cn; ++j) {
                const double t = LU[(size_t)k * cn + j];
                LU[(size_t)k * cn + j] = LU[(size_t)piv * cn + j];
                LU[(size_t)piv * cn + j] = t;
            }
        const double dinv = 1.0 / LU[(size_t)k * cn + k];
        for (int32_t i = k + 1; i < cn; ++i) {
            const double f = LU[(size_t)i * cn + k] * dinv;
            LU[(size_t)i * cn + k] = f;
            for (int32_t j = k + 1; j < cn; ++j)
                LU[(size_t)i * cn + j] -= f * LU[(size_t)k * cn + j];
        }
    }
}

static void amg_sgs(const OrcCsr *A, double *x, const double *b)
{
    for (int32_t i = 0; i < A->n; ++i) {
        double s = b[i], aii = 0.0;
        for (int32_t k = A->rp[i]; k < A->rp[i + 1]; ++k) {
            const int32_t j = A->ci[k];
            if (j == i)
                aii = A->v[k];
            else
                s -= A->v[k] * x[j];
        }
        if (fabs(aii) > 1e-30)
            x[i] = s / aii;
    }
    for (int32_t i = A->n - 1; i >= 0; --i) {
        double s = b[i], aii = 0.0;
        for (int32_t k = A->rp[i]; k < A->rp[i + 1]; ++k) {
            const int32_t j = A->ci[k];
            if (j == i)
                aii = A->v[k];
            else
                s -= A->v[k] * x[j];
        }
        if (fabs(aii) > 1e-30)
            x[i] = s / aii;
    }
}

static void amg_direct(const OrcAmg *M, double *x, const double *b)
{
    const int32_t n = M->coarseN;
    if (n == 0)
        return;
    double *y = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    for (int32_t i = 0; i < n; ++i) {
        double s = b[i];
        for (int32_t j = 0; j < i; ++j)
            s -= M->lu[(size_t)i * n + j] * y[j];
        y[i] = s;
    }
    for (int32_t i = n - 1; i >= 0; --i) {
        double s = y[i];
        for (int32_t j = i + 1; j < n; ++j)
            s -= M->lu[(size_t)i * n + j] * x[j];
        const double d = M->lu[(size_t)i * n + i];
        x[i] = (fabs(d) > 1e-30) ? s / d : 0.0;
    }
    free(y);
}

static void csr_spmv(const OrcCsr *A, const double *x, double *y)
{
    orc_spmv(A->n, A->rp, A->ci, A->v, x, y);
}

static void amg_vcycle(const OrcAmg *M, int lvl, double *x, const double *b)
{
    if (lvl == M->nlev - 1) {
        amg_direct(M, x, b);
        return;
    }
    const OrcCsr *A = &M->A[lvl];
    const int32_t n = A->n, nc = M->R[lvl].n;
    amg_sgs(A, x, b);
    double *r = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    csr_spmv(A, x, r);
    for (int32_t i = 0; i < n; ++i)
        r[i] = b[i] - r[i];
    double *rc = (double *)xmalloc((size_t)nc * sizeof(double) + 8);
    double *ec = (double *)xmalloc((size_t)nc * sizeof(double) + 8);
    csr_spmv(&M->R[lvl], r, rc);
    for (int32_t i = 0; i < nc; ++i)
        ec[i] = 0.0;
    amg_vcycle(M, lvl + 1, ec, rc);
    csr_spmv(&M->P[lvl], ec, r);
    for (int32_t i = 0; i < n; ++i)
        x[i] += r[i];
    amg_sgs(A, x, b);
    free(r);
    free(rc);
    free(ec);
}

void orc_amg_apply(const OrcAmg *M, const double *r, double *z)
{
    const int32_t n = M->A[0].n;
    for (int32_t i = 0; i < n; ++i)
        z[i] = 0.0;
    amg_vcycle(M, 0, z, r);
}

/* Setup + one apply (test entry point); sizes[l] = rows of level l, nnzs[l]
 * its entries (up to 10 levels), *nlev and *coarseN out.  z may be NULL. */
void orc_amg_probe(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, const double *r,
                   double *z, int *nlev, int32_t *sizes, int32_t *nnzs, int32_t *coarseN)
{
    OrcAmg M;
    orc_amg_setup(&M, n, rowPtr, colIdx, values);
    *nlev = M.nlev;
    for (int l = 0; l < M.nlev; ++l) {
        sizes[l] = M.A[l].n;
        nnzs[l] = M.A[l].rp[M.A[l].n];
    }
    *coarseN = M.coarseN;
    if (z)
        orc_amg_apply(&M, r, z);
    orc_amg_free(&M);
}

/* The digest simall_amg_hierarchy_digest takes (FNV-1a over 64-bit words of
 * every level's operator, every P and R, then the dense LU), of the hierarchy
 * restated here.  Test infrastructure: it compares the library's host setup
 * with this restatement. */
static uint64_t fnv_word(uint64_t h, uint64_t w)
{
    h ^= w;
    return h * 0x100000001b3ULL;
}

static uint64_t fnv_csr(uint64_t h, const OrcCsr *m)
{
    for (int32_t i = 0; i <= m->n; ++i)
        h = fnv_word(h, (uint64_t)(uint32_t)m->rp[i]);
    for (int32_t k = 0; k < m->rp[m->n]; ++k)
        h = fnv_word(h, (uint64_t)(uint32_t)m->ci[k]);
    for (int32_t k = 0; k < m->rp[m->n]; ++k) {
        uint64_t w;
        memcpy(&w, &m->v[k], sizeof w);
        h = fnv_word(h, w);
    }
    return h;
}

uint64_t orc_amg_digest(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, int *nlev)
{
    OrcAmg M;
    orc_amg_setup(&M, n, rowPtr, colIdx, values);
    uint64_t h = 0xcbf29ce484222325ULL;
    for (int l = 0; l < M.nlev; ++l) {
        h = fnv_csr(h, &M.A[l]);
        if (l + 1 < M.nlev) {
            h = fnv_csr(h, &M.P[l]);
            h = fnv_csr(h, &M.R[l]);
        }
    }
    for (size_t q = 0; q < (size_t)M.coarseN * (size_t)M.coarseN; ++q) {
        uint64_t w;
        memcpy(&w, &M.lu[q], sizeof w);
        h = fnv_word(h, w);
    }
    *nlev = M.nlev;
    orc_amg_free(&M);
    return h;
}

/* ------------------------------------------------------------------ preconditioner objects */

/* make_preconditioner (src/solver/LinearSolvers.cpp:240-254): 1 ILU(0),
 * 2 SSOR (w = 1), 3 AMG (default parameters), anything else Jacobi (None,
 * kind 4, is the default branch's Jacobi). */
typedef struct {
    int kind; /* 0 Jacobi, 1 ILU(0), 2 SSOR, 3 AMG */
    OrcAmg amg;
    int64_t n;
    const int32_t *rowPtr, *colIdx;
    const double *values;
    double *invD, *lu, *y, *diag, *v;
    int32_t *diagPtr;
} OrcPrec;

static void prec_setup(OrcPrec *M, int kind, int64_t n, const int32_t *rowPtr, const int32_t *colIdx,
                       const double *values)
{
    memset(M, 0, sizeof(*M));
    M->kind = (kind == 1 || kind == 2 || kind == 3) ? kind : 0;
    M->n = n;
    M->rowPtr = rowPtr;
    M->colIdx = colIdx;
    M->values = values;
    if (M->kind == 3) {
        orc_amg_setup(&M->amg, n, rowPtr, colIdx, values);
    } else if (M->kind == 2) {
        M->diag = (double *)xmalloc((size_t)n * sizeof(double) + 8);
        M->invD = (double *)xmalloc((size_t)n * sizeof(double) + 8);
        M->y = (double *)xmalloc((size_t)n * sizeof(double) + 8);
        M->v = (double *)xmalloc((size_t)n * sizeof(double) + 8);
        orc_ssor_setup(n, rowPtr, colIdx, values, M->diag, M->invD);
    } else if (M->kind == 1) {
        M->lu = (double *)xmalloc((size_t)rowPtr[n] * sizeof(double) + 8);
        M->diagPtr = (int32_t *)xmalloc((size_t)n * sizeof(int32_t) + 8);
        M->y = (double *)xmalloc((size_t)n * sizeof(double) + 8);
        orc_ilu0_setup(n, rowPtr, colIdx, values, M->lu, M->diagPtr);
    } else {
        M->invD = (double *)xmalloc((size_t)n * sizeof(double) + 8);
        orc_jacobi_setup(n, rowPtr, colIdx, values, M->invD);
    }
}

static void prec_apply(const OrcPrec *M, const double *r, double *z)
{
    if (M->kind == 1)
        orc_ilu0_apply(M->n, M->rowPtr, M->colIdx, M->lu, M->diagPtr, r, z, M->y);
    else if (M->kind == 2)
        orc_ssor_apply(M->n, M->rowPtr, M->colIdx, M->values, M->diag, M->invD, 1.0, r, z, M->y, M->v);
    else if (M->kind == 3)
        orc_amg_apply(&M->amg, r, z);
    else
        for (int64_t i = 0; i < M->n; ++i)
            z[i] = M->invD[i] * r[i];
}

static void prec_free(OrcPrec *M)
{
    free(M->invD);
    free(M->lu);
    free(M->y);
    free(M->diagPtr);
    free(M->diag);
    free(M->v);
    if (M->kind == 3)
        orc_amg_free(&M->amg);
}

/* ------------------------------------------------------------------ CG */

/*
 * Preconditioned CG.  Follows CGSolver::solve (src/solver/LinearSolvers.cpp:420-451):
 * setup M; x = 0; r = b; z = M r; p = z; rz = r.z; bnorm = max(|b|,1e-30);
 * loop { Ap; pAp; if pAp == 0 -> last = sqrt(rz)/bnorm, return it;
 *        alpha = rz/pAp; x += alpha p; r -= alpha Ap; last = |r|/bnorm;
 *        if last < tol return it+1; z = M r; rzNew = r.z; beta = rzNew/rz;
 *        p = z + beta p; rz = rzNew }  return maxIt.
 * precond: 0 Jacobi, 1 ILU0, 2 SSOR, 3 AMG; any other value is Jacobi (OrcPrec).  hist (optional, maxIt long)
 * receives last after each iteration.
 */
int orc_cg(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, const double *b,
           int precond, double tol, int maxIt, double *x, double *lastRes, double *hist)
{
    OrcPrec M;
    prec_setup(&M, precond, n, rowPtr, colIdx, values);
    double *r = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    double *z = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    double *p = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    double *Ap = (double *)xmalloc((size_t)n * sizeof(double) + 8);
#define APPLY_M() prec_apply(&M, r, z)
    for (int64_t i = 0; i < n; ++i) {
        x[i] = 0.0;
        r[i] = b[i];
    }
    APPLY_M();
    memcpy(p, z, (size_t)n * sizeof(double));
    double rz = orc_dot(n, r, z);
    const double bn = norm2(n, b);
    const double bnorm = STD_MAX(bn, 1e-30);
    int ret = maxIt;
    double last = 0.0;
    for (int it = 0; it < maxIt; ++it) {
        orc_spmv(n, rowPtr, colIdx, values, p, Ap);
        const double pAp = orc_dot(n, p, Ap);
        if (pAp == 0) {
            last = sqrt(rz) / bnorm;
            ret = it;
            break;
        }
        const double alpha = rz / pAp;
        axpy(n, alpha, p, x);
        axpy(n, -alpha, Ap, r);
        const double rn = norm2(n, r);
        last = rn / bnorm;
        if (hist)
            hist[it] = last;
        if (last < tol) {
            ret = it + 1;
            break;
        }
        APPLY_M();
        const double rzNew = orc_dot(n, r, z);
        const double beta = rzNew / rz;
        for (int64_t i = 0; i < n; ++i)
            p[i] = z[i] + beta * p[i];
        rz = rzNew;
    }
#undef APPLY_M
    *lastRes = last;
    free(r);
    free(z);
    free(p);
    free(Ap);
    prec_free(&M);
    return ret;
}

/* ------------------------------------------------------------------ gpu::CgGpu */

/* gpu::ilu0_factor_inplace (src/gpu/GpuKernels.cpp:345-401): IKJ ILU(0) in
 * place; 0 when a row has no diagonal entry, a pivot U_kk is zero, or a row
 * i >= 1 ends with a zero U_ii (values are then partly factored), else 1.  On
 * success the factor equals ILU0Preconditioner::setup's (orc_ilu0_setup). */
int orc_gpu_ilu0_factor(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, double *values)
{
    int32_t *diagPos = (int32_t *)xmalloc((size_t)n * sizeof(int32_t) + 8);
    int ok = 1;
    for (int64_t i = 0; i < n && ok; ++i) {
        diagPos[i] = -1;
        for (int32_t k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                diagPos[i] = k;
                break;
            }
        if (diagPos[i] < 0)
            ok = 0;
    }
    for (int64_t i = 1; i < n && ok; ++i) {
        for (int32_t p = rowPtr[i]; p < rowPtr[i + 1] && ok; ++p) {
            const int32_t k = colIdx[p];
            if (k >= i)
                break;
            const double ukk = values[diagPos[k]];
            if (ukk == 0.0) {
                ok = 0;
                break;
            }
            const double lik = values[p] / ukk;
            values[p] = lik;
            for (int32_t q = diagPos[k] + 1; q < rowPtr[k + 1]; ++q) {
                const int32_t j = colIdx[q];
                for (int32_t r = p + 1; r < rowPtr[i + 1]; ++r)
                    if (colIdx[r] == j) {
                        values[r] -= lik * values[q];
                        break;
                    }
            }
        }
        if (ok && values[diagPos[i]] == 0.0)
            ok = 0;
    }
    free(diagPos);
    return ok;
}

/* gpu::CgGpu::set_matrix + solve (src/gpu/CgGpu.cpp:35-238) on the GPU
 * facade's host path (src/gpu/GpuKernels.cpp: spmv_csr :196-283, dot :125-145,
 * nrm2 :147-165, axpy/scal/xpby, jacobi_apply :286-334 z_i = r_i / d_i,
 * ilu0_apply :403-481).  precond: 0 None (z = r), 1 Jacobi (d_i = the row's
 * first diagonal entry, 1.0 when missing; divides by 1.0 where d_i = 0), 2
 * ILU0 (falls back to Jacobi for good when the factor fails: *precondAfter).
 * x is the initial guess and the solution.  out[0..3]: iterations,
 * finalResidual ||r||_2 (absolute), initialResidual, converged.  Stop test
 * ||r|| / bRef <= tol (bRef = ||b||, 1 when b = 0) or, with relativeOrders > 0,
 * ||r|| <= ||r_0|| 10^-relativeOrders -- first trigger wins; |p.q| < 1e-300
 * ends the loop leaving iterations and finalResidual at 0 (as the reference
 * does).  *lastResidual: CgGpu::last_residual(). */
void orc_cggpu_solve(int precond, double tol, int maxIt, double relativeOrders, int64_t n, const int32_t *rowPtr,
                     const int32_t *colIdx, const double *values, const double *b, double *x, double *out,
                     int *precondAfter, double *lastResidual)
{
    const int64_t nnz = rowPtr[n];
    double *d = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    double *lu = NULL;
    if (precond == 2) {
        lu = (double *)xmalloc((size_t)nnz * sizeof(double) + 8);
        memcpy(lu, values, (size_t)nnz * sizeof(double));
        if (!orc_gpu_ilu0_factor(n, rowPtr, colIdx, lu)) {
            precond = 1;
            free(lu);
            lu = NULL;
        }
    }
    if (precond == 1)
        for (int64_t i = 0; i < n; ++i) {
            d[i] = 1.0;
            for (int32_t k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
                if (colIdx[k] == i) {
                    d[i] = values[k];
                    break;
                }
        }
    *precondAfter = precond;
    double *r = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    double *z = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    double *p = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    double *q = (double *)xmalloc((size_t)n * sizeof(double) + 8);
    out[0] = 0.0;
    out[1] = 0.0;
    out[3] = 0.0;
#define APPLY_M()                                                                                        \
    do {                                                                                                 \
        if (precond == 0) {                                                                              \
            memcpy(z, r, (size_t)n * sizeof(double));                                                   \
        } else if (precond == 1) {                                                                       \
            for (int64_t i = 0; i < n; ++i)                                                              \
                z[i] = r[i] / (d[i] != 0.0 ? d[i] : 1.0);                                                \
        } else {                                                                                         \
            for (int64_t i = 0; i < n; ++i) {                                                            \
                double s = r[i];                                                                         \
                for (int32_t k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {                                    \
                    if (colIdx[k] < i)                                                                   \
                        s -= lu[k] * z[colIdx[k]];                                                       \
                    else                                                                                 \
                        break;                                                                           \
                }                                                                                        \
                z[i] = s;                                                                                \
            }                                                                                            \
            for (int64_t ii = n - 1; ii >= 0; --ii) {                                                    \
                double s = z[ii], dg = 1.0;                                                              \
                for (int32_t k = rowPtr[ii]; k < rowPtr[ii + 1]; ++k) {                                  \
                    if (colIdx[k] > ii)                                                                  \
                        s -= lu[k] * z[colIdx[k]];                                                       \
                    else if (colIdx[k] == ii)                                                            \
                        dg = lu[k];                                                                      \
                }                                                                                        \
                z[ii] = s / (dg != 0.0 ? dg : 1.0);                                                      \
            }                                                                                            \
        }                                                                                                \
    } while (0)
    /* r = b - A x0: spmv, scal(-1), axpy(1, b) */
    orc_spmv(n, rowPtr, colIdx, values, x, r);
    for (int64_t i = 0; i < n; ++i)
        r[i] = -1.0 * r[i];
    axpy(n, 1.0, b, r);
    const double bNorm = norm2(n, b);
    const double bRef = bNorm > 0.0 ? bNorm : 1.0;
    double rNorm = norm2(n, r);
    out[2] = rNorm;
    if (rNorm / bRef <= tol) {
        out[0] = 0.0;
        out[1] = rNorm;
        out[3] = 1.0;
        *lastResidual = rNorm;
    } else {
        APPLY_M();
        memcpy(p, z, (size_t)n * sizeof(double));
        double rhoOld = orc_dot(n, r, z);
        const double dropTol = relativeOrders > 0.0 ? rNorm * pow(10.0, -relativeOrders) : 0.0;
        for (int it = 1; it <= maxIt; ++it) {
            orc_spmv(n, rowPtr, colIdx, values, p, q);
            const double pq = orc_dot(n, p, q);
            if (fabs(pq) < 1e-300)
                break;
            const double alpha = rhoOld / pq;
            axpy(n, alpha, p, x);
            axpy(n, -alpha, q, r);
            rNorm = norm2(n, r);
            if (rNorm / bRef <= tol || (dropTol > 0.0 && rNorm <= dropTol)) {
                out[0] = it;
                out[1] = rNorm;
                out[3] = 1.0;
                break;
            }
            APPLY_M();
            const double rhoNew = orc_dot(n, r, z);
            const double beta = rhoNew / rhoOld;
            for (int64_t i = 0; i < n; ++i)
                p[i] = 1.0 * z[i] + beta * p[i];
            rhoOld = rhoNew;
            if (it == maxIt) {
                out[0] = it;
                out[1] = rNorm;
                out[3] = 0.0;
            }
        }
        *lastResidual = out[1];
    }
#undef APPLY_M
    free(r);
    free(z);
    free(p);
    free(q);
    free(d);
    free(lu);
}

/* ------------------------------------------------------------------ face-conductance extension */

/*
 * Face-conductance Poisson operator (an extension; the reference cannot
 * express per-face k or non-zero Dirichlet values).  It restates the
 * reference face coefficient (src/solver/SimpleAlgorithm.cpp:391-393, :417,
 * :427) with k_f in place of 1/aP_f:
 *   g_f    = rho*|A|^2 / max(|d.A|, 1e-30)   (d as in orc_assemble)
 *   coef_f = k_f * g_f
 * interior faces add +oo,-on,+nn,-no; a Dirichlet face (isDirichlet[f])
 * adds +oo and rhs_o += coef_f * pb_f.  rhs starts from src (cell source).
 * No pin is applied.  g receives g_f (0 for Neumann boundary faces).
 */
void orc_assemble_face_k(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor,
                         const double *ax, const double *ay, const double *az, const double *fcx,
                         const double *fcy, const double *fcz, const double *ccx, const double *ccy,
                         const double *ccz, const uint8_t *isDirichlet, double rho, const double *k,
                         const double *pb, const double *src, const int32_t *rowPtr, const int32_t *colIdx,
                         double *values, double *rhs, double *g)
{
    const int64_t nnz = rowPtr[nC];
    for (int64_t q = 0; q < nnz; ++q)
        values[q] = 0.0;
    for (int64_t c = 0; c < nC; ++c)
        rhs[c] = src[c];
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        const double Ax = ax[f], Ay = ay[f], Az = az[f];
        const double Amag2 = Ax * Ax + Ay * Ay + Az * Az;
        double dx, dy, dz;
        g[f] = 0.0;
        if (n != ORC_BOUNDARY) {
            dx = ccx[n] - ccx[o];
            dy = ccy[n] - ccy[o];
            dz = ccz[n] - ccz[o];
        } else if (isDirichlet[f]) {
            dx = fcx[f] - ccx[o];
            dy = fcy[f] - ccy[o];
            dz = fcz[f] - ccz[o];
        } else {
            continue;
        }
        const double ddotA = fabs(dx * Ax + dy * Ay + dz * Az);
        const double gf = rho * Amag2 / STD_MAX(ddotA, 1e-30);
        const double coef = k[f] * gf;
        g[f] = gf;
        if (n != ORC_BOUNDARY) {
            add_at(rowPtr, colIdx, values, o, o, coef);
            add_at(rowPtr, colIdx, values, o, n, -coef);
            add_at(rowPtr, colIdx, values, n, n, coef);
            add_at(rowPtr, colIdx, values, n, o, -coef);
        } else {
            add_at(rowPtr, colIdx, values, o, o, coef);
            rhs[o] += coef * pb[f];
        }
    }
}

/*
 * Adjoint gradient of L(x) with A(k) x = b(k, pb), given x and the adjoint
 * lambda = A^-T dL/dx:
 *   interior f:  dL/dk_f  = -g_f (lambda_o - lambda_n)(x_o - x_n)
 *   Dirichlet f: dL/dk_f  = -g_f lambda_o (x_o - pb_f)
 *                dL/dpb_f =  k_f g_f lambda_o
 * Neumann boundary faces get 0.  This is -(dR/dalpha)^T lambda of
 * solve_discrete_adjoint (src/adjoint/DiscreteAdjoint.cpp:170-182) for
 * R = A(k) x - b(k, pb).
 */
void orc_face_k_gradient(int64_t nF, const int64_t *owner, const int64_t *neighbor, const uint8_t *isDirichlet,
                         const double *g, const double *k, const double *pb, const double *x,
                         const double *lambda, double *dk, double *dpb)
{
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        dk[f] = 0.0;
        dpb[f] = 0.0;
        if (n != ORC_BOUNDARY) {
            dk[f] = -g[f] * (lambda[o] - lambda[n]) * (x[o] - x[n]);
        } else if (isDirichlet[f]) {
            dk[f] = -g[f] * lambda[o] * (x[o] - pb[f]);
            dpb[f] = k[f] * g[f] * lambda[o];
        }
    }
}

/* ------------------------------------------------------------------ the face loops around the solve */

/* BCType ordinals (src/solver/Solver.hpp:105-121) used by the face loops. */
enum { ORC_BC_WALL = 0, ORC_BC_NOSLIP = 1, ORC_BC_MOVING = 2, ORC_BC_VELIN = 4, ORC_BC_SYMMETRY = 9 };

/* compute_face_fluxes (src/solver/SimpleAlgorithm.cpp:201-237).  A periodic
 * face (twin[f] >= 0; twin may be NULL) takes 0.5 (U_o + U_t) with t the twin
 * face's owner (:214-219).  zoneType[z] = the BCType ordinal of the first boundary spec
 * with zone z (find_bc), -1 when there is none; zoneVec[3 z .. 3 z + 2] its
 * vectorValue.  Face velocity: interior 0.5 (U_o + U_n); VelocityInlet and
 * MovingWall the zone's vector; NoSlipWall, Wall and Symmetry zero; any other
 * boundary (or none) the owner's velocity. */
void orc_face_fluxes(int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *ax, const double *ay,
                     const double *az, const uint32_t *zone, const int *zoneType, const double *zoneVec, int nZones,
                     double rho, const double *Ux, const double *Uy, const double *Uz, double *phi,
                     const int32_t *twin)
{
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        double ux, uy, uz;
        if (n != ORC_BOUNDARY) {
            ux = 0.5 * (Ux[o] + Ux[n]);
            uy = 0.5 * (Uy[o] + Uy[n]);
            uz = 0.5 * (Uz[o] + Uz[n]);
        } else if (twin && twin[f] >= 0) {
            const int64_t tw = owner[twin[f]];
            ux = 0.5 * (Ux[o] + Ux[tw]);
            uy = 0.5 * (Uy[o] + Uy[tw]);
            uz = 0.5 * (Uz[o] + Uz[tw]);
        } else {
            const uint32_t z = zone[f];
            const int t = (int)z < nZones ? zoneType[z] : -1;
            if (t == ORC_BC_VELIN || t == ORC_BC_MOVING) {
                ux = zoneVec[3 * z];
                uy = zoneVec[3 * z + 1];
                uz = zoneVec[3 * z + 2];
            } else if (t == ORC_BC_NOSLIP || t == ORC_BC_WALL || t == ORC_BC_SYMMETRY) {
                ux = uy = uz = 0.0;
            } else {
                ux = Ux[o];
                uy = Uy[o];
                uz = Uz[o];
            }
        }
        phi[f] = rho * (ux * ax[f] + uy * ay[f] + uz * az[f]);
    }
}

/* LeastSquaresGradient (src/solver/Gradient.cpp:17-133): the inverse of the
 * weighted normal matrix per cell (precompute, invert3x3_sym), then the
 * gradient of phi with the boundary faces' difference taken as zero. */
static void orc_inv3_sym(double xx, double xy, double xz, double yy, double yz, double zz, double out[6])
{
    const double det = xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz);
    if (fabs(det) < 1e-30) {
        out[0] = out[1] = out[2] = out[3] = out[4] = out[5] = 0.0;
        return;
    }
    const double inv = 1.0 / det;
    out[0] = (yy * zz - yz * yz) * inv;
    out[1] = -(xy * zz - yz * xz) * inv;
    out[2] = (xy * yz - yy * xz) * inv;
    out[3] = (xx * zz - xz * xz) * inv;
    out[4] = -(xx * yz - xy * xz) * inv;
    out[5] = (xx * yy - xy * xy) * inv;
}

void orc_lsq_inverse(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *fcx,
                     const double *fcy, const double *fcz, const double *ccx, const double *ccy, const double *ccz,
                     double *mInv /* [6 nC] */)
{
    double *A = (double *)calloc((size_t)(6 * nC), sizeof(double));
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        if (o == ORC_BOUNDARY)
            continue;
        double d[2][3];
        int64_t cells[2];
        int cnt;
        if (n == ORC_BOUNDARY) {
            d[0][0] = fcx[f] - ccx[o];
            d[0][1] = fcy[f] - ccy[o];
            d[0][2] = fcz[f] - ccz[o];
            cells[0] = o;
            cnt = 1;
        } else {
            const double dx = ccx[n] - ccx[o], dy = ccy[n] - ccy[o], dz = ccz[n] - ccz[o];
            d[0][0] = dx;
            d[0][1] = dy;
            d[0][2] = dz;
            d[1][0] = -dx;
            d[1][1] = -dy;
            d[1][2] = -dz;
            cells[0] = o;
            cells[1] = n;
            cnt = 2;
        }
        for (int k = 0; k < cnt; ++k) {
            const double dx = d[k][0], dy = d[k][1], dz = d[k][2];
            const double w2 = 1.0 / (dx * dx + dy * dy + dz * dz + 1e-30);
            double *a = A + 6 * cells[k];
            a[0] += w2 * dx * dx;
            a[1] += w2 * dx * dy;
            a[2] += w2 * dx * dz;
            a[3] += w2 * dy * dy;
            a[4] += w2 * dy * dz;
            a[5] += w2 * dz * dz;
        }
    }
    for (int64_t c = 0; c < nC; ++c) {
        const double *a = A + 6 * c;
        orc_inv3_sym(a[0], a[1], a[2], a[3], a[4], a[5], mInv + 6 * c);
    }
    free(A);
}

void orc_lsq_gradient(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *fcx,
                      const double *fcy, const double *fcz, const double *ccx, const double *ccy, const double *ccz,
                      const double *mInv, const double *phi, double *gx, double *gy, double *gz)
{
    double *b = (double *)calloc((size_t)(3 * nC), sizeof(double));
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        if (o == ORC_BOUNDARY)
            continue;
        if (n == ORC_BOUNDARY) {
            const double dx = fcx[f] - ccx[o], dy = fcy[f] - ccy[o], dz = fcz[f] - ccz[o];
            const double w2 = 1.0 / (dx * dx + dy * dy + dz * dz + 1e-30);
            const double dphi = 0.0;
            b[3 * o] += w2 * dx * dphi;
            b[3 * o + 1] += w2 * dy * dphi;
            b[3 * o + 2] += w2 * dz * dphi;
        } else {
            const double dx = ccx[n] - ccx[o], dy = ccy[n] - ccy[o], dz = ccz[n] - ccz[o];
            const double w2 = 1.0 / (dx * dx + dy * dy + dz * dz + 1e-30);
            const double dphi = phi[n] - phi[o];
            b[3 * o] += w2 * dx * dphi;
            b[3 * o + 1] += w2 * dy * dphi;
            b[3 * o + 2] += w2 * dz * dphi;
            b[3 * n] += w2 * dx * -dphi;
            b[3 * n + 1] += w2 * dy * -dphi;
            b[3 * n + 2] += w2 * dz * -dphi;
        }
    }
    for (int64_t c = 0; c < nC; ++c) {
        const double *m = mInv + 6 * c, bx = b[3 * c], by = b[3 * c + 1], bz = b[3 * c + 2];
        gx[c] = m[0] * bx + m[1] * by + m[2] * bz;
        gy[c] = m[1] * bx + m[3] * by + m[4] * bz;
        gz[c] = m[2] * bx + m[4] * by + m[5] * bz;
    }
    free(b);
}

/* correct_fields (src/solver/SimpleAlgorithm.cpp:450-487): p += urfP p';
 * U -= V / max(aP, 1e-30) grad p' (least-squares gradient); interior faces
 * phi += rho |A|^2 / max(0.5 (aP_o + aP_n) |d.A|, 1e-30) (p'_o - p'_n). */
void orc_correct_fields(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *ax,
                        const double *ay, const double *az, const double *fcx, const double *fcy, const double *fcz,
                        const double *ccx, const double *ccy, const double *ccz, const double *vol, double rho,
                        double urfP, const double *aP, const double *pPrime, double *p, double *Ux, double *Uy,
                        double *Uz, double *phi)
{
    for (int64_t c = 0; c < nC; ++c)
        p[c] += urfP * pPrime[c];
    double *mInv = (double *)malloc((size_t)(6 * nC) * sizeof(double));
    double *g = (double *)malloc((size_t)(3 * nC) * sizeof(double));
    orc_lsq_inverse(nC, nF, owner, neighbor, fcx, fcy, fcz, ccx, ccy, ccz, mInv);
    orc_lsq_gradient(nC, nF, owner, neighbor, fcx, fcy, fcz, ccx, ccy, ccz, mInv, pPrime, g, g + nC, g + 2 * nC);
    for (int64_t c = 0; c < nC; ++c) {
        const double w = vol[c] / STD_MAX(aP[c], 1e-30);
        Ux[c] -= w * g[c];
        Uy[c] -= w * g[nC + c];
        Uz[c] -= w * g[2 * nC + c];
    }
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        const double Ax = ax[f], Ay = ay[f], Az = az[f];
        const double Amag2 = Ax * Ax + Ay * Ay + Az * Az;
        if (n != ORC_BOUNDARY) {
            const double dx = ccx[n] - ccx[o], dy = ccy[n] - ccy[o], dz = ccz[n] - ccz[o];
            const double ddotA = fabs(dx * Ax + dy * Ay + dz * Az);
            const double aPf = 0.5 * (aP[o] + aP[n]);
            const double coef = rho * Amag2 / STD_MAX(aPf * ddotA, 1e-30);
            phi[f] += coef * (pPrime[o] - pPrime[n]);
        }
    }
    free(mInv);
    free(g);
}

/* ------------------------------------------------------------------ momentum */

/*
 * assemble_momentum (src/solver/SimpleAlgorithm.cpp:240-355) for one velocity
 * component, first-order upwind, no periodic faces.  values (on the shared
 * pattern) and rhs are overwritten.  Face loop in face order with the
 * reference's add_at scatter:
 *   F = phi_f, ConvO = max(F, 0), ConvN = max(-F, 0), D = mu |A|^2 / max(|d.A|, 1e-30)
 *   (d: neighbour centroid - owner centroid, or face centroid - owner
 *   centroid on a boundary face);
 *   interior: oo += ConvO + D, on -= ConvN + D, nn += ConvN + D, no -= ConvO + D;
 *   boundary by the zone's first spec (zoneType[z], -1 when none):
 *     NoSlipWall / Wall / VelocityInlet / MovingWall: oo += ConvO + D,
 *       rhs_o += (ConvN + D) Ub, Ub = 0 for the walls, the zone vector's
 *       component otherwise;  Symmetry: nothing;  any other: oo += ConvO.
 * Then rhs_c -= gp_c vol_c (gp = the component of the pressure gradient);
 * transient (dt > 0): Vrho_dt = rho vol_c / dt, BDF2 (useBDF2) adds
 * 1.5 Vrho_dt to the diagonal and (2 Un - 0.5 Unm1) Vrho_dt to rhs, implicit
 * Euler Vrho_dt and Un Vrho_dt; then Patankar under-relaxation:
 * a = diag / urfU, rhs_c += (a - diag) Ucomp_c.  aPout (optional) receives the
 * relaxed diagonal (the reference captures it for component 0).
 * opt = {rho, mu, urfU, dt}.
 */
void orc_assemble_momentum(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *ax,
                           const double *ay, const double *az, const double *fcx, const double *fcy,
                           const double *fcz, const double *ccx, const double *ccy, const double *ccz,
                           const double *vol, const uint32_t *zone, const int *zoneType, const double *zoneVec,
                           int nZones, const int32_t *rowPtr, const int32_t *colIdx, const double *opt, int useBDF2,
                           int comp, const double *phi, const double *gp, const double *Ucomp, const double *Un,
                           const double *Unm1, double *values, double *rhs, double *aPout, const int32_t *twin)
{
    const double rho = opt[0], mu = opt[1], urfU = opt[2], dt = opt[3];
    const int64_t nnz = rowPtr[nC];
    for (int64_t k = 0; k < nnz; ++k)
        values[k] = 0.0;
    for (int64_t c = 0; c < nC; ++c)
        rhs[c] = 0.0;
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        const double Ax = ax[f], Ay = ay[f], Az = az[f];
        const double Amag2 = Ax * Ax + Ay * Ay + Az * Az;
        const double Ff = phi[f];
        const double ConvO = STD_MAX(Ff, 0.0);
        const double ConvN = STD_MAX(-Ff, 0.0);
        if (n != ORC_BOUNDARY) {
            const double dx = ccx[n] - ccx[o], dy = ccy[n] - ccy[o], dz = ccz[n] - ccz[o];
            const double ddotA = fabs(dx * Ax + dy * Ay + dz * Az);
            const double D = mu * Amag2 / STD_MAX(ddotA, 1e-30);
            add_at(rowPtr, colIdx, values, o, o, ConvO + D);
            add_at(rowPtr, colIdx, values, o, n, -(ConvN + D));
            add_at(rowPtr, colIdx, values, n, n, ConvN + D);
            add_at(rowPtr, colIdx, values, n, o, -(ConvO + D));
        } else {
            const uint32_t z = zone[f];
            const int t = (int)z < nZones ? zoneType[z] : -1;
            const double dx = fcx[f] - ccx[o], dy = fcy[f] - ccy[o], dz = fcz[f] - ccz[o];
            const double ddotA = fabs(dx * Ax + dy * Ay + dz * Az);
            const double D = mu * Amag2 / STD_MAX(ddotA, 1e-30);
            if (twin && twin[f] >= 0) {  /* periodic (:275-282): half an interior face's coupling */
                const int64_t tw = owner[twin[f]];
                add_at(rowPtr, colIdx, values, o, o, ConvO + D);
                add_at(rowPtr, colIdx, values, o, tw, -(ConvN + D));
            } else if (t == ORC_BC_NOSLIP || t == ORC_BC_WALL || t == ORC_BC_VELIN || t == ORC_BC_MOVING) {
                const double Ub = (t == ORC_BC_NOSLIP || t == ORC_BC_WALL) ? 0.0 : zoneVec[3 * z + comp];
                add_at(rowPtr, colIdx, values, o, o, ConvO + D);
                rhs[o] += (ConvN + D) * Ub;
            } else if (t == ORC_BC_SYMMETRY) {
                /* zero normal gradient: no contribution */
            } else {
                add_at(rowPtr, colIdx, values, o, o, ConvO);
            }
        }
    }
    for (int64_t c = 0; c < nC; ++c)
        rhs[c] -= gp[c] * vol[c];
    if (dt > 0.0) {
        for (int64_t c = 0; c < nC; ++c) {
            const double Vrho_dt = rho * vol[c] / dt;
            const int32_t kd = find_col(rowPtr, colIdx, c, c);
            if (kd < 0)
                continue;
            if (useBDF2) {
                values[kd] += 1.5 * Vrho_dt;
                rhs[c] += (2.0 * Un[c] - 0.5 * Unm1[c]) * Vrho_dt;
            } else {
                values[kd] += Vrho_dt;
                rhs[c] += Un[c] * Vrho_dt;
            }
        }
    }
    for (int64_t c = 0; c < nC; ++c) {
        const int32_t kd = find_col(rowPtr, colIdx, c, c);
        if (kd < 0)
            continue;
        const double aDiag = values[kd];
        const double scaled = aDiag / urfU;
        values[kd] = scaled;
        rhs[c] += (scaled - aDiag) * Ucomp[c];
    }
    if (aPout)
        for (int64_t c = 0; c < nC; ++c) {
            const int32_t kd = find_col(rowPtr, colIdx, c, c);
            aPout[c] = kd >= 0 ? values[kd] : 0.0;
        }
}

/* ------------------------------------------------------------------ non-symmetric Krylov */

/*
 * BiCGSTAB (BiCGSTABSolver::solve, src/solver/LinearSolvers.cpp:363-405), x
 * from 0: r = b - A x, rh = r, rho = alpha = omega = 1, v = 0;
 * loop { rhoNew = rh.r; if 0 -> last = |r|/bnorm, return it;
 *        beta = (rhoNew/rho)(alpha/omega); p = r + beta (p - omega v);
 *        y = M p; v = A y; alpha = rhoNew / rh.v; s = r - alpha v;
 *        if |s| < tol bnorm -> x += alpha y, last = |s|/bnorm, return it+1;
 *        z = M s; t = A z; omega = t.s / max(t.t, 1e-30);
 *        x += alpha y + omega z; r = s - omega t; rho = rhoNew;
 *        last = |r|/bnorm; if last < tol return it+1 }  return maxIt.
 */
int orc_bicgstab(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, const double *b,
                 int precond, double tol, int maxIt, double *x, double *lastRes)
{
    OrcPrec M;
    prec_setup(&M, precond, n, rowPtr, colIdx, values);
    const size_t bytes = (size_t)n * sizeof(double) + 8;
    double *r = (double *)xmalloc(bytes), *rh = (double *)xmalloc(bytes), *p = (double *)xmalloc(bytes);
    double *v = (double *)xmalloc(bytes), *s = (double *)xmalloc(bytes), *t = (double *)xmalloc(bytes);
    double *y = (double *)xmalloc(bytes), *z = (double *)xmalloc(bytes);
    for (int64_t i = 0; i < n; ++i) {
        x[i] = 0.0;
        p[i] = 0.0;
    }
    orc_spmv(n, rowPtr, colIdx, values, x, v);
    for (int64_t i = 0; i < n; ++i)
        r[i] = b[i] - v[i];
    memcpy(rh, r, (size_t)n * sizeof(double));
    double rho = 1.0, alpha = 1.0, omega = 1.0, last = 0.0;
    const double bn = norm2(n, b);
    const double bnorm = STD_MAX(bn, 1e-30);
    for (int64_t i = 0; i < n; ++i)
        v[i] = 0.0;
    int ret = maxIt;
    for (int it = 0; it < maxIt; ++it) {
        const double rhoNew = orc_dot(n, rh, r);
        if (rhoNew == 0.0) {
            last = norm2(n, r) / bnorm;
            ret = it;
            goto out;
        }
        const double beta = (rhoNew / rho) * (alpha / omega);
        for (int64_t i = 0; i < n; ++i)
            p[i] = r[i] + beta * (p[i] - omega * v[i]);
        prec_apply(&M, p, y);
        orc_spmv(n, rowPtr, colIdx, values, y, v);
        alpha = rhoNew / orc_dot(n, rh, v);
        for (int64_t i = 0; i < n; ++i)
            s[i] = r[i] - alpha * v[i];
        if (norm2(n, s) < tol * bnorm) {
            axpy(n, alpha, y, x);
            last = norm2(n, s) / bnorm;
            ret = it + 1;
            goto out;
        }
        prec_apply(&M, s, z);
        orc_spmv(n, rowPtr, colIdx, values, z, t);
        {
            const double tt = orc_dot(n, t, t);
            omega = orc_dot(n, t, s) / STD_MAX(tt, 1e-30);
        }
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * y[i] + omega * z[i];
            r[i] = s[i] - omega * t[i];
        }
        rho = rhoNew;
        last = norm2(n, r) / bnorm;
        if (last < tol) {
            ret = it + 1;
            goto out;
        }
    }
out:
    *lastRes = last;
    free(r);
    free(rh);
    free(p);
    free(v);
    free(s);
    free(t);
    free(y);
    free(z);
    prec_free(&M);
    return ret;
}

/*
 * GMRES(m), left-preconditioned, modified Gram-Schmidt and Givens rotations
 * (GMRESmSolver::solve, src/solver/LinearSolvers.cpp:268-343), x from 0.
 * Each cycle: r = b - A x, z = M r, beta = |z|; beta < tol bnorm -> last =
 * beta/bnorm, return iter.  V0 = z/beta, s = (beta, 0, ...); Arnoldi steps
 * j = 0.. while j < m and iter < maxIt: z = M A v_j; H_ij = v_i.z, z -= H_ij v_i
 * (i = 0..j); H_{j+1,j} = |z|; v_{j+1} = z / H_{j+1,j} unless it is 0; apply
 * the previous rotations to column j, form the new one with hypot, rotate s;
 * last = |s_{j+1}|/bnorm, stop the cycle when last < tol (j counts the step,
 * iter does not).  Back-substitute H y = s over the j steps, x += V y; return
 * iter when last < tol.  The outer loop runs at most maxIt cycles.
 */
int orc_gmres(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, const double *b,
              int precond, double tol, int maxIt, int restart, double *x, double *lastRes)
{
    OrcPrec M;
    prec_setup(&M, precond, n, rowPtr, colIdx, values);
    const int m = restart > 1 ? restart : 1;
    const size_t bytes = (size_t)n * sizeof(double) + 8;
    double *r = (double *)xmalloc(bytes), *w = (double *)xmalloc(bytes), *z = (double *)xmalloc(bytes);
    double *V = (double *)xmalloc((size_t)(m + 1) * bytes);
    double *H = (double *)xmalloc((size_t)(m + 1) * (size_t)m * sizeof(double));
    double *cs = (double *)xmalloc((size_t)m * sizeof(double)), *sn = (double *)xmalloc((size_t)m * sizeof(double));
    double *sv = (double *)xmalloc((size_t)(m + 1) * sizeof(double)), *yv = (double *)xmalloc((size_t)m * sizeof(double) + 8);
#define VV(i) (V + (size_t)(i) * ((size_t)n + 1))
#define HH(i, j) H[(size_t)(i) * (size_t)m + (size_t)(j)]
    memset(V, 0, (size_t)(m + 1) * bytes);
    memset(H, 0, (size_t)(m + 1) * (size_t)m * sizeof(double));
    memset(cs, 0, (size_t)m * sizeof(double));
    memset(sn, 0, (size_t)m * sizeof(double));
    for (int64_t i = 0; i < n; ++i)
        x[i] = 0.0;
    const double bn = norm2(n, b);
    const double bnorm = STD_MAX(bn, 1e-30);
    double last = 0.0;
    int iter = 0;
    int ret = -1;
    for (int outer = 0; outer < maxIt && ret < 0; ++outer) {
        orc_spmv(n, rowPtr, colIdx, values, x, w);
        for (int64_t i = 0; i < n; ++i)
            r[i] = b[i] - w[i];
        prec_apply(&M, r, z);
        const double beta = norm2(n, z);
        if (beta < tol * bnorm) {
            last = beta / bnorm;
            ret = iter;
            break;
        }
        memcpy(VV(0), z, (size_t)n * sizeof(double));
        {
            const double sc = 1.0 / beta;
            for (int64_t i = 0; i < n; ++i)
                VV(0)[i] *= sc;
        }
        for (int i = 0; i <= m; ++i)
            sv[i] = 0.0;
        sv[0] = beta;
        int j;
        for (j = 0; j < m && iter < maxIt; ++j, ++iter) {
            orc_spmv(n, rowPtr, colIdx, values, VV(j), w);
            prec_apply(&M, w, z);
            for (int i = 0; i <= j; ++i) {
                HH(i, j) = orc_dot(n, VV(i), z);
                axpy(n, -HH(i, j), VV(i), z);
            }
            HH(j + 1, j) = norm2(n, z);
            if (HH(j + 1, j) != 0.0) {
                memcpy(VV(j + 1), z, (size_t)n * sizeof(double));
                const double sc = 1.0 / HH(j + 1, j);
                for (int64_t i = 0; i < n; ++i)
                    VV(j + 1)[i] *= sc;
            }
            for (int i = 0; i < j; ++i) {
                const double t = cs[i] * HH(i, j) + sn[i] * HH(i + 1, j);
                HH(i + 1, j) = -sn[i] * HH(i, j) + cs[i] * HH(i + 1, j);
                HH(i, j) = t;
            }
            const double dd = hypot(HH(j, j), HH(j + 1, j));
            cs[j] = HH(j, j) / dd;
            sn[j] = HH(j + 1, j) / dd;
            HH(j, j) = dd;
            HH(j + 1, j) = 0.0;
            const double t = cs[j] * sv[j];
            sv[j + 1] = -sn[j] * sv[j];
            sv[j] = t;
            last = fabs(sv[j + 1]) / bnorm;
            if (last < tol) {
                ++j;
                break;
            }
        }
        for (int i = j - 1; i >= 0; --i) {
            double sum = sv[i];
            for (int k = i + 1; k < j; ++k)
                sum -= HH(i, k) * yv[k];
            yv[i] = sum / HH(i, i);
        }
        for (int i = 0; i < j; ++i)
            axpy(n, yv[i], VV(i), x);
        if (last < tol)
            ret = iter;
    }
#undef VV
#undef HH
    if (ret < 0)
        ret = iter;
    *lastRes = last;
    free(r);
    free(w);
    free(z);
    free(V);
    free(H);
    free(cs);
    free(sn);
    free(sv);
    free(yv);
    prec_free(&M);
    return ret;
}

/*
 * TFQMR (TfqmrSolver::solve, src/solver/LinearSolvers.cpp:497-609), x from 0:
 * r = rh = w = b; u1 = M r; v = Au1 = A u1; tau = |r|; bnorm = max(|b|, 1e-30);
 * tau/bnorm < tol -> last = tau/bnorm, return 0.  rho = rh.r, theta = eta =
 * alpha = 0, d = 0.  Each iteration:
 *   sigma = rh.v; |sigma| < 1e-30 -> last = tau/bnorm, return it;
 *   alpha = rho/sigma; u2 = u1 - alpha M v; Au2 = A u2;
 *   two half steps (u = u1, Au1 then u = u2, Au2):
 *     w -= alpha Au; theta' = |w|/max(tau, 1e-30); c = 1/sqrt(1 + theta'^2);
 *     tau' = tau theta' c; eta' = c c alpha;
 *     d = u + (theta theta eta / max(alpha, 1e-30)) d; x += eta' d;
 *     (tau, theta, eta) = (tau', theta', eta');
 *   last = tau sqrt(2(it+1) + 1) / bnorm; if last < tol: last = |b - A x|/bnorm
 *     and return it+1 when that is < tol;
 *   r -= alpha (Au1 + Au2); rhoNew = rh.r; |rho| < 1e-30 -> last = tau/bnorm,
 *   return it; beta = rhoNew/rho; u1 = M r + beta (u2 + beta u1); Au1 = A u1;
 *   v = Au1 + beta (Au2 + beta v); rho = rhoNew.
 * Returns maxIt when the loop ends; *lastRes is left as it was when nothing
 * sets it (maxIt <= 0), as the reference leaves its member.
 */
int orc_tfqmr(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, const double *b,
              int precond, double tol, int maxIt, double *x, double *lastRes)
{
    OrcPrec M;
    prec_setup(&M, precond, n, rowPtr, colIdx, values);
    const size_t bytes = (size_t)n * sizeof(double) + 8;
    double *r = (double *)xmalloc(bytes), *rh = (double *)xmalloc(bytes), *w = (double *)xmalloc(bytes);
    double *d = (double *)xmalloc(bytes), *u1 = (double *)xmalloc(bytes), *u2 = (double *)xmalloc(bytes);
    double *v = (double *)xmalloc(bytes), *Au1 = (double *)xmalloc(bytes), *Au2 = (double *)xmalloc(bytes);
    double *z = (double *)xmalloc(bytes);
    int ret = maxIt;
    for (int64_t i = 0; i < n; ++i) {
        x[i] = 0.0;
        d[i] = 0.0;
        r[i] = b[i];
    }
    memcpy(rh, r, (size_t)n * sizeof(double));
    memcpy(w, r, (size_t)n * sizeof(double));
    prec_apply(&M, r, u1);
    orc_spmv(n, rowPtr, colIdx, values, u1, v);
    memcpy(Au1, v, (size_t)n * sizeof(double));
    double tau = norm2(n, r);
    const double bn = norm2(n, b);
    const double bnorm = STD_MAX(bn, 1e-30);
    if (tau / bnorm < tol) {
        *lastRes = tau / bnorm;
        ret = 0;
        goto out;
    }
    {
        double rho = orc_dot(n, rh, r);
        double theta = 0.0, eta = 0.0, alpha = 0.0;
        for (int it = 0; it < maxIt; ++it) {
            const double sigma = orc_dot(n, rh, v);
            if (fabs(sigma) < 1.0e-30) {
                *lastRes = tau / bnorm;
                ret = it;
                goto out;
            }
            alpha = rho / sigma;
            prec_apply(&M, v, z);
            for (int64_t i = 0; i < n; ++i)
                u2[i] = u1[i] - alpha * z[i];
            orc_spmv(n, rowPtr, colIdx, values, u2, Au2);
            for (int half = 0; half < 2; ++half) {
                const double *u = half ? u2 : u1;
                const double *Au = half ? Au2 : Au1;
                for (int64_t i = 0; i < n; ++i)
                    w[i] -= alpha * Au[i];
                const double theta_new = norm2(n, w) / STD_MAX(tau, 1.0e-30);
                const double c = 1.0 / sqrt(1.0 + theta_new * theta_new);
                const double tau_new = tau * theta_new * c;
                const double eta_new = c * c * alpha;
                for (int64_t i = 0; i < n; ++i) {
                    d[i] = u[i] + (theta * theta * eta / STD_MAX(alpha, 1.0e-30)) * d[i];
                    x[i] += eta_new * d[i];
                }
                tau = tau_new;
                theta = theta_new;
                eta = eta_new;
            }
            const double resBound = tau * sqrt(2.0 * (it + 1) + 1.0);
            *lastRes = resBound / bnorm;
            if (*lastRes < tol) {
                orc_spmv(n, rowPtr, colIdx, values, x, z);
                for (int64_t i = 0; i < n; ++i)
                    z[i] = b[i] - z[i];
                *lastRes = norm2(n, z) / bnorm;
                if (*lastRes < tol) {
                    ret = it + 1;
                    goto out;
                }
            }
            for (int64_t i = 0; i < n; ++i)
                r[i] -= alpha * (Au1[i] + Au2[i]);
            const double rhoNew = orc_dot(n, rh, r);
            if (fabs(rho) < 1.0e-30) {
                *lastRes = tau / bnorm;
                ret = it;
                goto out;
            }
            const double beta = rhoNew / rho;
            prec_apply(&M, r, z);
            for (int64_t i = 0; i < n; ++i)
                u1[i] = z[i] + beta * (u2[i] + beta * u1[i]);
            orc_spmv(n, rowPtr, colIdx, values, u1, Au1);
            for (int64_t i = 0; i < n; ++i)
                v[i] = Au1[i] + beta * (Au2[i] + beta * v[i]);
            rho = rhoNew;
        }
    }
out:
    free(r);
    free(rh);
    free(w);
    free(d);
    free(u1);
    free(u2);
    free(v);
    free(Au1);
    free(Au2);
    free(z);
    prec_free(&M);
    return ret;
}

/* ------------------------------------------------------------------ one SIMPLE outer iteration */

/* make_linear_solver (src/solver/Solver.cpp:25-39) for cfg = {kind, precond,
 * maxIt, restart}: 0 GMRES, 1 BiCGSTAB, 2 CG, 3 TFQMR. */
static int orc_linear_solve(const int *cfg, double tol, int64_t n, const int32_t *rowPtr, const int32_t *colIdx,
                            const double *values, const double *b, double *x, double *last)
{
    switch (cfg[0]) {
    case 1:
        return orc_bicgstab(n, rowPtr, colIdx, values, b, cfg[1], tol, cfg[2], x, last);
    case 2:
        return orc_cg(n, rowPtr, colIdx, values, b, cfg[1], tol, cfg[2], x, last, NULL);
    case 3:
        return orc_tfqmr(n, rowPtr, colIdx, values, b, cfg[1], tol, cfg[2], x, last);
    default:
        return orc_gmres(n, rowPtr, colIdx, values, b, cfg[1], tol, cfg[2], cfg[3], x, last);
    }
}

/*
 * SimpleAlgorithm::iterate (src/solver/SimpleAlgorithm.cpp:522-547) and the
 * iterate() overrides of PisoAlgorithm (src/solver/PisoAlgorithm.cpp:27-70)
 * and PimpleAlgorithm (src/solver/PimpleAlgorithm.cpp:48-96), no periodic
 * faces, no halo exchange.  loops = {nOuterCorrectors, nCorrectors,
 * nNonOrthCorr, momentumPredictor} (SIMPLE: {1, 1, 0, 1}); tolUP = {tolU,
 * tolP} (PIMPLE's early exit, 0 disables).  Per outer corrector:
 *   compute_face_fluxes; if momentumPredictor: for k in x, y, z:
 *   assemble_momentum(k), solve it from x = 0 into U_k, res.mom[k] = |A U_k - b|;
 *   nCorrectors times { compute_face_fluxes; nNonOrthCorr + 1 times {
 *   assemble_pressure_correction (SIMPLEC: the denominator from the momentum
 *   matrix); solve p' from 0; correct_fields; the last pass's |rhs| is
 *   res.cont } }; then stop when both tolerances that are set hold.
 * opt = {rho, mu, urfU, urfP, dt}; flags bit 0 BDF2 (the transient term uses
 * Un and Unm1), bit 1 SIMPLEC.  momCfg / pCfg = {kind, precond, maxIt,
 * restart}.  U [3][nC], p [nC] in/out; phi [nF], aP [nC] (in/out: kept from
 * the last predictor), pPrime [nC] out; res [4] = mom x, y, z and cont;
 * iters [4] the last momentum solves' and the last pressure solve's counts.
 * Returns the index of the last outer corrector run.
 * isPressure[z] marks zones with a PressureOutlet / PressureInlet spec.
 */
int orc_simple_iterate(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *ax,
                       const double *ay, const double *az, const double *fcx, const double *fcy, const double *fcz,
                       const double *ccx, const double *ccy, const double *ccz, const double *vol,
                       const uint32_t *zone, const int *zoneType, const double *zoneVec, const uint8_t *isPressure,
                       int nZones, const int32_t *rowPtr, const int32_t *colIdx, const double *opt, int flags,
                       const int *momCfg, double momTol, const int *pCfg, double pTol, const int *loops,
                       const double *tolUP, double *U, double *p, const double *Un, const double *Unm1, double *phi,
                       double *aP, double *pPrime, double *res, int *iters, const int32_t *twin)
{
    const double rho = opt[0], mu = opt[1], urfU = opt[2], urfP = opt[3], dt = opt[4];
    const int bdf2 = flags & 1, simplec = (flags >> 1) & 1;
    const int nOuter = loops[0] < 1 ? 1 : loops[0], nCorr = loops[1] < 1 ? 1 : loops[1];
    const int nNonOrth = loops[2] < 0 ? 0 : loops[2], predictor = loops[3];
    const int64_t nnz = rowPtr[nC];
    double *values = (double *)xmalloc((size_t)nnz * sizeof(double) + 8);
    double *rhs = (double *)xmalloc((size_t)nC * sizeof(double) + 8);
    double *Ax = (double *)xmalloc((size_t)nC * sizeof(double) + 8);
    double *g = (double *)xmalloc((size_t)(3 * nC) * sizeof(double) + 8);
    double *mInv = (double *)xmalloc((size_t)(6 * nC) * sizeof(double) + 8);
    double *den = (double *)xmalloc((size_t)nC * sizeof(double) + 8);
    double *pvals = (double *)xmalloc((size_t)nnz * sizeof(double) + 8);
    const double momOpt[4] = {rho, mu, urfU, dt};
    orc_lsq_inverse(nC, nF, owner, neighbor, fcx, fcy, fcz, ccx, ccy, ccz, mInv);
    for (int k = 0; k < 4; ++k)
        res[k] = 0.0;
    int outer;
    for (outer = 0; outer < nOuter; ++outer) {
        orc_face_fluxes(nF, owner, neighbor, ax, ay, az, zone, zoneType, zoneVec, nZones, rho, U, U + nC, U + 2 * nC,
                        phi, twin);
        if (predictor) {
            orc_lsq_gradient(nC, nF, owner, neighbor, fcx, fcy, fcz, ccx, ccy, ccz, mInv, p, g, g + nC, g + 2 * nC);
            for (int k = 0; k < 3; ++k) {
                orc_assemble_momentum(nC, nF, owner, neighbor, ax, ay, az, fcx, fcy, fcz, ccx, ccy, ccz, vol, zone,
                                      zoneType, zoneVec, nZones, rowPtr, colIdx, momOpt, bdf2, k, phi, g + k * nC,
                                      U + k * nC, Un ? Un + k * nC : NULL, Unm1 ? Unm1 + k * nC : NULL, values, rhs,
                                      k == 0 ? aP : NULL, twin);
                double last = 0.0;
                iters[k] = orc_linear_solve(momCfg, momTol, nC, rowPtr, colIdx, values, rhs, U + k * nC, &last);
                orc_spmv(nC, rowPtr, colIdx, values, U + k * nC, Ax);
                double s = 0.0;
                for (int64_t i = 0; i < nC; ++i) {
                    const double d = Ax[i] - rhs[i];
                    s += d * d;
                }
                res[k] = sqrt(s);
            }
        }
        for (int corr = 0; corr < nCorr; ++corr) {
            orc_face_fluxes(nF, owner, neighbor, ax, ay, az, zone, zoneType, zoneVec, nZones, rho, U, U + nC,
                            U + 2 * nC, phi, twin);
            for (int no = 0; no <= nNonOrth; ++no) {
                if (simplec)
                    orc_simplec_denominator(nC, rowPtr, colIdx, values, aP, den);
                orc_assemble(nC, nF, owner, neighbor, ax, ay, az, fcx, fcy, fcz, zone, ccx, ccy, ccz, isPressure,
                             nZones, rho, simplec ? den : aP, phi, rowPtr, colIdx, pvals, rhs, twin);
                double last = 0.0;
                iters[3] = orc_linear_solve(pCfg, pTol, nC, rowPtr, colIdx, pvals, rhs, pPrime, &last);
                double cs = 0.0;
                for (int64_t i = 0; i < nC; ++i)
                    cs += rhs[i] * rhs[i];
                res[3] = sqrt(cs);
                orc_correct_fields(nC, nF, owner, neighbor, ax, ay, az, fcx, fcy, fcz, ccx, ccy, ccz, vol, rho, urfP,
                                   aP, pPrime, p, U, U + nC, U + 2 * nC, phi);
            }
        }
        /* PimpleAlgorithm's converged(): every set tolerance holds */
        const double tolU = tolUP[0], tolP = tolUP[1];
        int conv = (tolU > 0.0) || (tolP > 0.0);
        if (tolU > 0.0) {
            double mm = fabs(res[0]);
            mm = STD_MAX(mm, fabs(res[1]));
            mm = STD_MAX(mm, fabs(res[2]));
            if (mm > tolU)
                conv = 0;
        }
        if (tolP > 0.0 && fabs(res[3]) > tolP)
            conv = 0;
        if (conv)
            break;
    }
    free(values);
    free(rhs);
    free(Ax);
    free(g);
    free(mInv);
    free(den);
    free(pvals);
    return outer < nOuter ? outer : nOuter - 1;
}

/* ------------------------------------------------------------------ SIMP topology optimisation */

/*
 * SimpTopology::apply_helmholtz_filter (src/optimization/SimpTopology.cpp:48-130)
 * restated on the mesh's CSR pattern (diagonal + interior-face neighbours,
 * the pattern build_sparsity makes): row c starts with its volume on the
 * diagonal; every interior face with a = |A| > 0 and d = |C_n - C_o| > 0 adds
 * coeff = r^2 a / d to both diagonals (face order) and -coeff to both
 * off-diagonal slots; CG + Jacobi (tol 1e-9, 400 iterations) on b = rho vol;
 * rhoT = clamp(x, 0, 1).  r == 0 copies rho.
 */
static void orc_helmholtz(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *ax,
                          const double *ay, const double *az, const double *ccx, const double *ccy, const double *ccz,
                          const double *vol, const int32_t *rowPtr, const int32_t *colIdx, double r, const double *rho,
                          double *rhoT)
{
    if (r <= 0.0) {
        memcpy(rhoT, rho, (size_t)nC * sizeof(double));
        return;
    }
    const double r2 = r * r;
    const int64_t nnz = rowPtr[nC];
    double *values = (double *)xmalloc((size_t)nnz * sizeof(double) + 8);
    for (int64_t k = 0; k < nnz; ++k)
        values[k] = 0.0;
    for (int64_t c = 0; c < nC; ++c)
        values[find_col(rowPtr, colIdx, c, c)] = vol[c];
    for (int64_t f = 0; f < nF; ++f) {
        const int64_t o = owner[f], n = neighbor[f];
        if (n == ORC_BOUNDARY)
            continue;
        const double a = sqrt(ax[f] * ax[f] + ay[f] * ay[f] + az[f] * az[f]);
        const double dx = ccx[n] - ccx[o], dy = ccy[n] - ccy[o], dz = ccz[n] - ccz[o];
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        if (d <= 0 || a <= 0)
            continue;
        const double coeff = r2 * a / d;
        add_at(rowPtr, colIdx, values, o, o, coeff);
        add_at(rowPtr, colIdx, values, o, n, -coeff);
        add_at(rowPtr, colIdx, values, n, n, coeff);
        add_at(rowPtr, colIdx, values, n, o, -coeff);
    }
    double *b = (double *)xmalloc((size_t)nC * sizeof(double) + 8);
    double *x = (double *)xmalloc((size_t)nC * sizeof(double) + 8);
    memset(b, 0, (size_t)nC * sizeof(double) + 8);
    for (int64_t i = 0; i < nC; ++i)
        b[i] = rho[i] * vol[i];
    double last = 0.0;
    orc_cg(nC, rowPtr, colIdx, values, b, 0, 1e-9, 400, x, &last, NULL);
    for (int64_t i = 0; i < nC; ++i)
        rhoT[i] = x[i] < 0.0 ? 0.0 : (1.0 < x[i] ? 1.0 : x[i]);
    free(values);
    free(b);
    free(x);
}

/*
 * SimpTopology::step (SimpTopology.cpp:132-227): filter rho -> rhoT;
 * K = Kmin + (Kmax - Kmin) rhoT^p; the sensitivity through the filter (r > 0:
 * rho is overwritten with dC and filtered into dCt, as the reference does) or
 * copied; optimality-criteria update with bisection on the volume
 * multiplier (at most 64 halvings while (l2 - l1) > 1e-9 (l1 + l2 + 1e-30);
 * the last halving's candidate is kept).  cfg = {penalty, Kmin, Kmax,
 * filterRadius, volumeFraction, move, damping, rhoMin}.  Returns
 * sum |rho_new - rho| / nC (rho as it stands before the update).
 */
double orc_simp_step(int64_t nC, int64_t nF, const int64_t *owner, const int64_t *neighbor, const double *ax,
                     const double *ay, const double *az, const double *ccx, const double *ccy, const double *ccz,
                     const double *vol, const int32_t *rowPtr, const int32_t *colIdx, const double *cfg, double *rho,
                     double *rhoT, double *kSimp, double *dC, double *dCt)
{
    const double p = cfg[0], Kmin = cfg[1], Kmax = cfg[2], r = cfg[3], vf = cfg[4], move = cfg[5], damping = cfg[6],
                 rhoMin = cfg[7];
    orc_helmholtz(nC, nF, owner, neighbor, ax, ay, az, ccx, ccy, ccz, vol, rowPtr, colIdx, r, rho, rhoT);
    const double dK = Kmax - Kmin;
    for (int64_t c = 0; c < nC; ++c)
        kSimp[c] = Kmin + dK * pow(rhoT[c], p);
    if (r > 0.0) {
        for (int64_t c = 0; c < nC; ++c)
            rho[c] = dC[c];
        orc_helmholtz(nC, nF, owner, neighbor, ax, ay, az, ccx, ccy, ccz, vol, rowPtr, colIdx, r, rho, rhoT);
        for (int64_t c = 0; c < nC; ++c)
            dCt[c] = rhoT[c];
    } else {
        for (int64_t c = 0; c < nC; ++c)
            dCt[c] = dC[c];
    }
    double Vtot = 0.0;
    for (int64_t c = 0; c < nC; ++c)
        Vtot += vol[c];
    const double Vtarget = vf * Vtot;
    double *rhoNew = (double *)xmalloc((size_t)nC * sizeof(double) + 8);
    for (int64_t c = 0; c < nC; ++c)
        rhoNew[c] = 0.0;
    double l1 = 0.0, l2 = 1e9;
    for (int it = 0; it < 64 && (l2 - l1) > 1e-9 * (l1 + l2 + 1e-30); ++it) {
        const double lmid = 0.5 * (l1 + l2);
        double V = 0.0;
        for (int64_t c = 0; c < nC; ++c) {
            const double s = -dCt[c] / STD_MAX(1e-12, lmid);
            const double bf = pow(STD_MAX(0.0, s), damping);
            const double old = rho[c];
            const double lo = STD_MAX(rhoMin, old - move);
            const double hi = (old + move < 1.0) ? old + move : 1.0; /* std::min(1.0, old + move) */
            const double t = old * bf;
            /* std::clamp(t, lo, hi) as the reference's library evaluates it,
             * min(max(t, lo), hi) -- which also fixes its result when the
             * move limits cross (lo > hi: hi) */
            const double mx = t < lo ? lo : t;
            const double v = hi < mx ? hi : mx;
            rhoNew[c] = v;
            V += v * vol[c];
        }
        if (V > Vtarget)
            l1 = lmid;
        else
            l2 = lmid;
    }
    double change = 0.0;
    for (int64_t c = 0; c < nC; ++c) {
        change += fabs(rhoNew[c] - rho[c]);
        rho[c] = rhoNew[c];
    }
    free(rhoNew);
    return change / (double)nC;
}
