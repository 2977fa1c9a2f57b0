// clusters.cpp -- cluster enumeration and NV-centre states (host C++).
//
// Enumeration restates the reference's graph growth bit for bit:
//   cSpinCollection::getConnectionMatrix (src/source/spin/SpinCollection/
//   SpinCollection.cpp:31-57): connected iff Euclidean distance <= cutoff, no
//   self connection;
//   cDepthFirstPathTracing::generate / subgraph_growth (src/source/spin/
//   SpinCluster/SpinClusterAlgorithm.cpp:98-148): order o clusters grow from
//   every order o-1 cluster (in set order) by every spin connected to any
//   member, recording the parent's position;
//   cClusterIndex::operator< (SpinClusterIndex.cpp:55-64): size, then
//   lexicographic on sorted indices (std::set order);
//   cSpinCluster::getSubClusters (SpinCluster.cpp:82-98): transitive closure
//   of parent positions, as a std::set of (order, position) pairs.
// The reference keeps dense (#candidates x nspin) matrices and walks std::set
// with std::advance; here clusters are sorted uint32 tuples deduplicated by a
// hash table, so enumeration is O(#clusters * order * degree).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oops_cce.h"
#include "oops_expv.h"

int oops_set_status(int code, const char *msg);

struct oops_clusters {
    int max_order = 0;
    std::vector<std::vector<uint32_t>> idx;      // per order: count*(order+1)
    std::vector<std::vector<uint64_t>> sub_off;  // per order: count+1
    std::vector<std::vector<uint32_t>> sub;      // per order: pairs (order, pos)
    size_t count(int o) const { return idx[o].size() / (size_t)(o + 1); }
};

namespace {

uint64_t hash_tuple(const uint32_t *t, size_t w)
{
    uint64_t h = 1469598103934665603ULL;
    for (size_t a = 0; a < w; ++a) {
        h ^= t[a];
        h *= 1099511628211ULL;
    }
    return h ^ (h >> 29);
}

}  // namespace

// Graph growth and sub-cluster closures from ascending neighbour lists (CSR):
// cDepthFirstPathTracing::generate and cSpinCluster::getSubClusters.
// Flat arrays throughout: per order the tuples (w = order+1 sorted spin
// indices each) in one vector, an open-addressing table of tuple numbers for
// deduplication, parent lists in CSR form (a tuple's parents arrive in
// increasing order because parents are visited in order, each at most once
// per tuple), closures collected with per-order stamp marks and sorted once.
static void grow_clusters(oops_clusters *c, size_t nspin, const std::vector<size_t> &nb_off,
                          const std::vector<uint32_t> &nb, int max_order)
{
    // order 0
    c->idx[0].resize(nspin);
    for (size_t i = 0; i < nspin; ++i) c->idx[0][i] = (uint32_t)i;
    // parents of every cluster, CSR per order (positions in set order)
    std::vector<std::vector<uint64_t>> par_off(max_order);
    std::vector<std::vector<uint32_t>> par(max_order);
    par_off[0].assign(nspin + 1, 0);
    std::vector<char> mark(nspin, 0);
    std::vector<uint32_t> cand;
    for (int o = 1; o < max_order; ++o) {
        const size_t pw = (size_t)o, w = (size_t)o + 1;
        const size_t np = c->count(o - 1);
        const uint32_t *P = c->idx[o - 1].data();
        std::vector<uint32_t> tup;                 // tuples in discovery order, w each
        std::vector<uint32_t> link_t, link_p;      // (tuple, parent) in discovery order
        // the table starts at ~4x the parents (each grows a few new tuples)
        size_t cap = 1024;
        while (cap < 4 * np) cap *= 2;
        std::vector<uint32_t> table(cap, 0xffffffffu);
        tup.reserve(2 * np * w);
        link_t.reserve(8 * np);
        link_p.reserve(8 * np);
        uint32_t child[16];
        size_t ntup = 0;
        for (size_t p = 0; p < np; ++p) {
            const uint32_t *ps = P + p * pw;
            cand.clear();
            for (size_t a = 0; a < pw; ++a)
                for (size_t e = nb_off[ps[a]]; e < nb_off[ps[a] + 1]; ++e)
                    if (!mark[nb[e]]) {
                        mark[nb[e]] = 1;
                        cand.push_back(nb[e]);
                    }
            for (uint32_t j : cand) mark[j] = 0;
            std::sort(cand.begin(), cand.end());
            for (uint32_t j : cand) {
                if (std::binary_search(ps, ps + pw, j)) continue;
                size_t q = 0, a = 0;
                bool put = false;
                while (q < w) {
                    if (!put && (a == pw || j < ps[a])) { child[q++] = j; put = true; }
                    else child[q++] = ps[a++];
                }
                if (2 * (ntup + 1) > cap) {  // grow and rehash
                    cap *= 2;
                    table.assign(cap, 0xffffffffu);
                    for (size_t t = 0; t < ntup; ++t) {
                        size_t h = (size_t)hash_tuple(&tup[t * w], w) & (cap - 1);
                        while (table[h] != 0xffffffffu) h = (h + 1) & (cap - 1);
                        table[h] = (uint32_t)t;
                    }
                }
                size_t h = (size_t)hash_tuple(child, w) & (cap - 1);
                uint32_t found = 0xffffffffu;
                while (table[h] != 0xffffffffu) {
                    if (std::memcmp(&tup[(size_t)table[h] * w], child, w * sizeof(uint32_t)) == 0) {
                        found = table[h];
                        break;
                    }
                    h = (h + 1) & (cap - 1);
                }
                if (found == 0xffffffffu) {
                    found = (uint32_t)ntup++;
                    table[h] = found;
                    tup.insert(tup.end(), child, child + w);
                }
                link_t.push_back(found);
                link_p.push_back((uint32_t)p);
            }
        }
        // set order (lexicographic on the sorted indices)
        std::vector<uint32_t> ord(ntup), pos(ntup);
        for (size_t q = 0; q < ntup; ++q) ord[q] = (uint32_t)q;
        std::sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) {
            return std::lexicographical_compare(&tup[(size_t)a * w], &tup[(size_t)a * w + w],
                                                &tup[(size_t)b * w], &tup[(size_t)b * w + w]);
        });
        for (size_t q = 0; q < ntup; ++q) pos[ord[q]] = (uint32_t)q;
        c->idx[o].resize(ntup * w);
        for (size_t q = 0; q < ntup; ++q)
            std::copy(&tup[(size_t)ord[q] * w], &tup[(size_t)ord[q] * w + w], c->idx[o].begin() + q * w);
        // parents, CSR in set order; a stable counting sort keeps each
        // tuple's parents in discovery (increasing) order
        par_off[o].assign(ntup + 1, 0);
        for (uint32_t t : link_t) par_off[o][pos[t] + 1]++;
        for (size_t q = 0; q < ntup; ++q) par_off[o][q + 1] += par_off[o][q];
        par[o].resize(link_t.size());
        std::vector<uint64_t> fill(par_off[o].begin(), par_off[o].end() - 1);
        for (size_t e = 0; e < link_t.size(); ++e) par[o][fill[pos[link_t[e]]]++] = link_p[e];
        if (ntup == 0) break;
    }
    // closures, bottom-up: union of every parent and its closure, as sorted
    // (order, position) pairs
    std::vector<std::vector<uint32_t>> stamp(max_order);
    for (int o = 0; o < max_order; ++o) stamp[o].assign(c->count(o), 0);
    uint32_t gen = 0;
    std::vector<uint64_t> acc;
    for (int o = 0; o < max_order; ++o) {
        const size_t n = c->count(o);
        c->sub_off[o].assign(n + 1, 0);
        std::vector<uint32_t> &S = c->sub[o];
        S.clear();
        for (size_t q = 0; q < n; ++q) {
            acc.clear();
            if (o > 0) {
                ++gen;
                for (uint64_t e = par_off[o][q]; e < par_off[o][q + 1]; ++e) {
                    const uint32_t p = par[o][e];
                    if (stamp[o - 1][p] != gen) {
                        stamp[o - 1][p] = gen;
                        acc.push_back(((uint64_t)(o - 1) << 32) | p);
                    }
                    const std::vector<uint32_t> &sp = c->sub[o - 1];
                    for (uint64_t r = c->sub_off[o - 1][p]; r < c->sub_off[o - 1][p + 1]; ++r) {
                        const uint32_t so = sp[2 * r], spos = sp[2 * r + 1];
                        if (stamp[so][spos] != gen) {
                            stamp[so][spos] = gen;
                            acc.push_back(((uint64_t)so << 32) | spos);
                        }
                    }
                }
                std::sort(acc.begin(), acc.end());
            }
            c->sub_off[o][q + 1] = c->sub_off[o][q] + acc.size();
            for (uint64_t x : acc) {
                S.push_back((uint32_t)(x >> 32));
                S.push_back((uint32_t)(x & 0xffffffffu));
            }
        }
    }
}

// Enumeration from coordinates: neighbours within the cutoff, then growth.
extern "C" int oops_clusters_enumerate(size_t nspin, const double *coords, double cutoff,
                                       int max_order, oops_clusters **out)
{
    if (!out || (nspin && !coords)) return oops_set_status(OOPS_ERR_ARG, "null pointer");
    if (max_order < 1 || max_order > 16) return oops_set_status(OOPS_ERR_SIZE, "max_order must be 1..16");
    if (nspin >= 0xffffffffu) return oops_set_status(OOPS_ERR_SIZE, "too many spins");
    oops_clusters *c = new oops_clusters();
    c->max_order = max_order;
    c->idx.resize(max_order);
    c->sub_off.resize(max_order);
    c->sub.resize(max_order);
    // neighbour lists (CSR, ascending): sqrt(dist^2) <= cutoff, i != j; the
    // square root is taken only near the cutoff, so the decision is the
    // reference's bit for bit.  The connected pairs are listed in (i, j)
    // order, then scattered into both rows: row r receives its i < r
    // neighbours (from earlier rows, increasing) before its j > r ones, so
    // every row comes out ascending without a sort.
    const double c2 = cutoff * cutoff, lo2 = c2 * (1.0 - 1e-12), hi2 = c2 * (1.0 + 1e-12);
    std::vector<uint32_t> pairs_ij;
    pairs_ij.reserve(16 * nspin);
    std::vector<size_t> nb_off(nspin + 1, 0);
    auto test_pair = [&](size_t i, size_t j) {  // i < j, the reference's arithmetic
        const double dx = coords[3 * i] - coords[3 * j];
        const double dy = coords[3 * i + 1] - coords[3 * j + 1];
        const double dz = coords[3 * i + 2] - coords[3 * j + 2];
        const double d2 = dx * dx + dy * dy + dz * dz;
        const bool conn = d2 < lo2 ? true : (d2 > hi2 ? false : std::sqrt(d2) <= cutoff);
        if (conn) {
            pairs_ij.push_back((uint32_t)i);
            pairs_ij.push_back((uint32_t)j);
            nb_off[i + 1]++;
            nb_off[j + 1]++;
        }
    };
    for (size_t i = 0; i < nspin; ++i)
        for (size_t j = i + 1; j < nspin; ++j) test_pair(i, j);
    for (size_t i = 0; i < nspin; ++i) nb_off[i + 1] += nb_off[i];
    std::vector<uint32_t> nb(nb_off[nspin]);
    {
        std::vector<size_t> fill(nb_off.begin(), nb_off.end() - 1);
        for (size_t e = 0; e < pairs_ij.size(); e += 2) {
            const uint32_t i = pairs_ij[e], j = pairs_ij[e + 1];
            nb[fill[i]++] = j;
            nb[fill[j]++] = i;
        }
    }
    grow_clusters(c, nspin, nb_off, nb, max_order);
    *out = c;
    return OOPS_OK;
}

// The same enumeration from a connection matrix instead of coordinates (the
// reference's cDepthFirstPathTracing takes the sp_mat that
// cSpinCollection::getConnectionMatrix builds): row_off (nspin+1 entries)
// and cols give every spin's connected spins; the diagonal is ignored (the
// reference zeroes it) and the matrix must be symmetric.
extern "C" int oops_clusters_enumerate_graph(size_t nspin, const size_t *row_off,
                                             const unsigned *cols, int max_order,
                                             oops_clusters **out)
{
    if (!out || !row_off || (row_off[nspin] && !cols)) return oops_set_status(OOPS_ERR_ARG, "null pointer");
    if (max_order < 1 || max_order > 16) return oops_set_status(OOPS_ERR_SIZE, "max_order must be 1..16");
    if (nspin >= 0xffffffffu) return oops_set_status(OOPS_ERR_SIZE, "too many spins");
    std::vector<size_t> nb_off(nspin + 1, 0);
    std::vector<uint32_t> nb;
    nb.reserve(row_off[nspin]);
    for (size_t i = 0; i < nspin; ++i) {
        if (row_off[i + 1] < row_off[i]) return oops_set_status(OOPS_ERR_ARG, "row offsets must not decrease");
        const size_t start = nb.size();
        for (size_t e = row_off[i]; e < row_off[i + 1]; ++e) {
            if (cols[e] >= nspin) return oops_set_status(OOPS_ERR_ARG, "column index out of range");
            if (cols[e] != i) nb.push_back(cols[e]);
        }
        std::sort(nb.begin() + start, nb.end());
        nb.erase(std::unique(nb.begin() + start, nb.end()), nb.end());
        nb_off[i + 1] = nb.size();
    }
    for (size_t i = 0; i < nspin; ++i)
        for (size_t e = nb_off[i]; e < nb_off[i + 1]; ++e) {
            const uint32_t j = nb[e];
            if (!std::binary_search(nb.begin() + nb_off[j], nb.begin() + nb_off[j + 1], (uint32_t)i))
                return oops_set_status(OOPS_ERR_ARG, "connection matrix is not symmetric");
        }
    oops_clusters *c = new oops_clusters();
    c->max_order = max_order;
    c->idx.resize(max_order);
    c->sub_off.resize(max_order);
    c->sub.resize(max_order);
    grow_clusters(c, nspin, nb_off, nb, max_order);
    *out = c;
    return OOPS_OK;
}

extern "C" int oops_clusters_destroy(oops_clusters *c)
{
    delete c;
    return OOPS_OK;
}

extern "C" size_t oops_clusters_count(const oops_clusters *c, int order)
{
    if (!c || order < 0 || order >= c->max_order) return 0;
    return c->count(order);
}

extern "C" int oops_clusters_indices(const oops_clusters *c, int order, unsigned *out)
{
    if (!c || !out || order < 0 || order >= c->max_order) return oops_set_status(OOPS_ERR_ARG, "bad arguments");
    std::memcpy(out, c->idx[order].data(), c->idx[order].size() * sizeof(uint32_t));
    return OOPS_OK;
}

extern "C" size_t oops_clusters_subcluster_total(const oops_clusters *c, int order)
{
    if (!c || order < 0 || order >= c->max_order) return 0;
    return c->sub_off[order].empty() ? 0 : (size_t)c->sub_off[order].back();
}

extern "C" int oops_clusters_subclusters(const oops_clusters *c, int order, size_t *offsets,
                                         unsigned *pairs)
{
    if (!c || !offsets || !pairs || order < 0 || order >= c->max_order)
        return oops_set_status(OOPS_ERR_ARG, "bad arguments");
    for (size_t q = 0; q < c->sub_off[order].size(); ++q) offsets[q] = (size_t)c->sub_off[order][q];
    std::memcpy(pairs, c->sub[order].data(), c->sub[order].size() * sizeof(uint32_t));
    return OOPS_OK;
}

// ---------------------------------------------------------------------------
// NV electron states (NVCenter::make_espin_hamiltonian, DefectCenter.cpp:32-45;
// cSPIN::get_spin_vector, Spin.cpp:88-95): H = D (S.n111)^2 + gamma_e B.S for
// the spin-1 NV electron, eigenvalues ascending, <S> of each eigenstate.
// ---------------------------------------------------------------------------
extern "C" int oops_nv_states(const double *B, double *evals, double *svec)
{
    if (!B || !evals || !svec) return oops_set_status(OOPS_ERR_ARG, "null pointer");
    typedef std::complex<double> cd;
    const double PI = 3.14159265358979323846;
    const double Dzf = 2.87e3 * 2.0 * PI * 1e6;
    const double ge = -1.760859708e11;
    const double r2 = 1.0 / std::sqrt(2.0);
    cd sx[3][3] = {{0, r2, 0}, {r2, 0, r2}, {0, r2, 0}};
    cd sy[3][3] = {{0, cd(0, -r2), 0}, {cd(0, r2), 0, cd(0, -r2)}, {0, cd(0, r2), 0}};
    cd sz[3][3] = {{1, 0, 0}, {0, 0, 0}, {0, 0, -1}};
    cd s111[3][3], H[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) s111[r][c] = (sx[r][c] + sy[r][c] + sz[r][c]) / std::sqrt(3.0);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            cd acc = 0;
            for (int k = 0; k < 3; ++k) acc += s111[r][k] * s111[k][c];
            H[r][c] = Dzf * acc + ge * (B[0] * sx[r][c] + B[1] * sy[r][c] + B[2] * sz[r][c]);
        }
    // complex Jacobi (A <- G^H A G), V accumulates G
    cd V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = std::abs(H[0][1]) + std::abs(H[0][2]) + std::abs(H[1][2]);
        if (off == 0.0) break;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 3; ++q) {
                cd apq = H[p][q];
                double mag = std::abs(apq);
                if (mag == 0.0) continue;
                double zeta = (H[q][q].real() - H[p][p].real()) / (2.0 * mag);
                double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                double cc = 1.0 / std::sqrt(1.0 + t * t), ss = t * cc;
                cd e = std::conj(apq) / mag;  // e^{-i phi}
                // G: col p = (c, -s e)^T at rows (p, q); col q = (s, c e)
                for (int k = 0; k < 3; ++k) {
                    cd ap = H[k][p], aq = H[k][q];
                    H[k][p] = cc * ap - ss * aq * e;
                    H[k][q] = ss * ap + cc * aq * e;
                    cd vp = V[k][p], vq = V[k][q];
                    V[k][p] = cc * vp - ss * vq * e;
                    V[k][q] = ss * vp + cc * vq * e;
                }
                for (int k = 0; k < 3; ++k) {
                    cd ap = H[p][k], aq = H[q][k];
                    H[p][k] = cc * ap - ss * aq * std::conj(e);
                    H[q][k] = ss * ap + cc * aq * std::conj(e);
                }
            }
    }
    int ord[3] = {0, 1, 2};
    std::sort(ord, ord + 3, [&](int a, int b) { return H[a][a].real() < H[b][b].real(); });
    const cd(*ops[3])[3] = {sx, sy, sz};
    for (int s = 0; s < 3; ++s) {
        int col = ord[s];
        evals[s] = H[col][col].real();
        for (int a = 0; a < 3; ++a) {
            cd acc = 0;
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) acc += std::conj(V[r][col]) * ops[a][r][c] * V[c][col];
            svec[3 * s + a] = acc.real();
        }
    }
    return OOPS_OK;
}

// The bath state SingleSampleCCE::prepare_bath_state draws
// (src/source/app/single_sample_cce.cpp:35-46): srand(seed), then
// rand() % 2 per bath spin.  The reference takes rand() from the C library;
// on glibc (the reference's Linux target) that is random_r's TYPE_3
// generator, restated here so that the states do not depend on the host's
// library: a 31-word state seeded by the Park-Miller recurrence
// x_i = 16807 x_{i-1} mod (2^31 - 1) (Schrage's factorisation, x_0 = seed,
// or 1 for seed 0), x_31..x_33 = x_0..x_2, then the additive lagged
// Fibonacci recurrence x_i = x_{i-31} + x_{i-3} mod 2^32, whose outputs from
// i = 344 on are rand() = x_i >> 1 (the first 310 are discarded by srand).
extern "C" int oops_bath_state_from_seed(unsigned seed, size_t nbath, unsigned char *state)
{
    if (!state && nbath) return oops_set_status(OOPS_ERR_ARG, "null state buffer");
    std::vector<uint32_t> r(344 + nbath);
    int32_t x = (int32_t)seed;
    if (x == 0) x = 1;
    r[0] = (uint32_t)x;
    for (int i = 1; i < 31; ++i) {
        const int32_t hi = x / 127773, lo = x % 127773;
        x = 16807 * lo - 2836 * hi;
        if (x < 0) x += 2147483647;
        r[i] = (uint32_t)x;
    }
    for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
    for (size_t i = 34; i < r.size(); ++i) r[i] = r[i - 31] + r[i - 3];
    for (size_t j = 0; j < nbath; ++j) state[j] = (unsigned char)((r[344 + j] >> 1) & 1u);
    return OOPS_OK;
}
