// host_build.cpp -- preprocessing of FFEA blobs into the packed GPU layout.
//
// Replaces the set-up half of the reference path:
//   Blob::calculate_node_element_connectivity (src/Blob.cpp:3974-4019)
//     -> per-node (element, corner) gather lists in element order;
//   NoMassCGSolver::init's sparsity pattern (src/NoMassCGSolver.cpp:63-162)
//     -> one 3x3 block per mesh edge, stored once (the transpose serves the
//        other direction), with the list of (element, a, b) terms that sum to it;
//   Blob::linearise_force's "first element wins" rule (src/Blob.cpp:1066-1085)
//     -> for every secondary node with a Stokes drag, the two linear nodes that
//        receive half of its force;
//   World::init's RNG seeding (src/World.cpp:287-317).
#include "host_build.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <queue>
#include <numeric>

namespace ffea {

namespace {

// glibc rand(): the TYPE_3 additive feedback generator r_i = r_{i-31} + r_{i-3}
// (degree 31, separation 3), seeded by r_i = 16807 r_{i-1} mod (2^31-1),
// first 310 outputs discarded, output r_i >> 1.  Restated from the published
// description so seeding does not touch the process-wide libc state.
struct GlibcRand {
    int32_t ring[31];
    int f = 3, b = 0;
    explicit GlibcRand(uint32_t seed)
    {
        if (seed == 0) seed = 1;
        int32_t r[31];
        r[0] = (int32_t)seed;
        for (int i = 1; i < 31; i++) {
            int32_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
            int32_t w = 16807 * lo - 2836 * hi;
            if (w < 0) w += 2147483647;
            r[i] = w;
        }
        std::memcpy(ring, r, sizeof(ring));
        for (int i = 0; i < 310; i++) next();
    }
    int next()
    {
        uint32_t v = (uint32_t)ring[f] + (uint32_t)ring[b];
        ring[f] = (int32_t)v;
        f = (f + 1) % 31;
        b = (b + 1) % 31;
        return (int)(v >> 1);
    }
};

// local corner pairs of the secondary slots n4..n9 (src/tetra_element_linear.cpp:567-591)
const int kMid[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

int32_t round_up(int32_t x, int32_t m) { return (x + m - 1) / m * m; }

}  // namespace

std::vector<int32_t> plan_parts(const std::vector<int32_t> &counts, int32_t ctas, int32_t max_rows)
{
    const int nb = (int)counts.size();
    const int32_t max_slices = std::max(1, max_rows / 32);
    std::vector<int32_t> slices(nb), k(nb);
    int64_t total = 0;
    for (int b = 0; b < nb; b++) {
        slices[b] = std::max(1, (counts[b] + 31) / 32);
        k[b] = (slices[b] + max_slices - 1) / max_slices;
        total += k[b];
    }
    {
        // longest segment first: (slices per segment rounded up, blob).  Up
        // to one segment per CTA, or, with more segments than CTAs, up to a
        // multiple of the CTA count, so that every CTA of the memory-resident
        // solve gets the same number of (shorter) segments
        const int64_t target = total <= ctas ? ctas : ((total + ctas - 1) / ctas) * ctas;
        std::priority_queue<std::pair<int32_t, int>> q;
        for (int b = 0; b < nb; b++) q.push({(slices[b] + k[b] - 1) / k[b], -b});
        while (total < target && !q.empty()) {
            const int b = -q.top().second;
            q.pop();
            // at least two slices per segment once a blob is split, so the
            // last segment keeps more than 32 real rows: a segment is also an
            // aggregate of the two-level preconditioner, whose six rigid
            // modes are independent only on a few non-collinear nodes (2
            // rows would make the coarse matrix singular)
            if (2 * (k[b] + 1) > slices[b]) continue;
            k[b]++;
            total++;
            q.push({(slices[b] + k[b] - 1) / k[b], -b});
        }
    }
    return k;
}

namespace {

// First row of part j when n rows are cut into k parts on 32-row boundaries.
int32_t part_start(int32_t n, int32_t k, int32_t j)
{
    const int64_t slices = std::max(1, (n + 31) / 32);
    return (int32_t)std::min<int64_t>(32 * (slices * j / k), n);
}

// Recursive coordinate bisection of ids[begin, end) into parts [p0, p1): the
// set is sorted along its longest extent and split at the row count of the
// first half of the parts.  Inside a part, rows run lexicographically over a
// grid of spacing h (x slowest, z fastest), so consecutive rows are mostly
// neighbours.  Ties break on the id: the order is the same on every host.
void rcb(const double *pos, std::vector<int32_t> &ids, int32_t begin, int32_t end, int32_t n, int32_t k, int32_t p0,
         int32_t p1, double h)
{
    if (end - begin <= 1) return;
    if (p1 - p0 == 1) {
        auto cell = [&](int32_t i, int c) { return (int64_t)std::floor(pos[3 * (size_t)i + c] / h); };
        std::sort(ids.begin() + begin, ids.begin() + end, [&](int32_t a, int32_t b) {
            for (int c = 0; c < 3; c++) {
                const int64_t ca = cell(a, c), cb = cell(b, c);
                if (ca != cb) return ca < cb;
            }
            return a < b;
        });
        return;
    }
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int32_t i = begin; i < end; i++)
        for (int c = 0; c < 3; c++) {
            lo[c] = std::min(lo[c], pos[3 * (size_t)ids[i] + c]);
            hi[c] = std::max(hi[c], pos[3 * (size_t)ids[i] + c]);
        }
    int axis = 0;
    for (int c = 1; c < 3; c++)
        if (hi[c] - lo[c] > hi[axis] - lo[axis]) axis = c;
    std::sort(ids.begin() + begin, ids.begin() + end, [&](int32_t a, int32_t b) {
        const double xa = pos[3 * (size_t)a + axis], xb = pos[3 * (size_t)b + axis];
        if (xa != xb) return xa < xb;
        return a < b;
    });
    const int32_t pm = (p0 + p1) / 2;
    const int32_t mid = begin + (part_start(n, k, pm) - part_start(n, k, p0));
    rcb(pos, ids, begin, mid, n, k, p0, pm, h);
    rcb(pos, ids, mid, end, n, k, pm, p1, h);
}

}  // namespace

int32_t plan_cg_segments(HostBatch &H)
{
    H.seg_row0.clear();
    H.seg_rows.clear();
    H.seg_blob.clear();
    for (int b = 0; b < H.num_blobs; b++) {
        BlobParams &bp = H.bp[b];
        const int32_t k = H.parts[b];
        bp.seg_off = (int32_t)H.seg_row0.size();
        bp.seg_cnt = k;
        for (int j = 0; j < k; j++) {
            const int32_t r0 = part_start(bp.node_cnt, k, j), r1 = part_start(bp.node_cnt, k, j + 1);
            H.seg_row0.push_back(bp.node_off + r0);
            H.seg_rows.push_back(std::max(0, r1 - r0));
            H.seg_blob.push_back(b);
        }
    }
    return (int32_t)H.seg_row0.size();
}

int64_t build_coarse(HostBatch &H)
{
    const int32_t nseg = (int32_t)H.seg_row0.size();
    H.seg_of_row.assign(H.nl_pad, -1);
    H.phi.assign(4 * (size_t)H.nl_pad, 0.f);
    for (int32_t s = 0; s < nseg; s++) {
        const int32_t r0 = H.seg_row0[s], n = H.seg_rows[s];
        double c[3] = {0, 0, 0};
        for (int32_t r = r0; r < r0 + n; r++)
            for (int k = 0; k < 3; k++) c[k] += H.pos[3 * (size_t)r + k];
        for (int k = 0; k < 3; k++) c[k] /= std::max(1, n);
        double r2 = 0.0;
        for (int32_t r = r0; r < r0 + n; r++)
            for (int k = 0; k < 3; k++) {
                const double dx = H.pos[3 * (size_t)r + k] - c[k];
                r2 += dx * dx;
            }
        const double R = n > 0 && r2 > 0 ? std::sqrt(r2 / n) : 1.0;
        for (int32_t r = r0; r < r0 + n; r++) {
            H.seg_of_row[r] = s;
            for (int k = 0; k < 3; k++) H.phi[4 * (size_t)r + k] = (float)((H.pos[3 * (size_t)r + k] - c[k]) / R);
            H.phi[4 * (size_t)r + 3] = 1.f;
        }
    }
    // couplings through the matrix pattern
    H.seg_nbr_ptr.assign(nseg + 1, 0);
    H.seg_nbr.clear();
    const int32_t nslices = (int32_t)H.slice_len.size();
    for (int32_t s = 0; s < nseg; s++) {
        std::vector<int32_t> nb{s};
        const int32_t r0 = H.seg_row0[s], n = H.seg_rows[s];
        for (int32_t r = r0; r < r0 + n; r++) {
            const int32_t sl = r / 32, lane = r % 32;
            if (sl >= nslices) continue;
            for (int32_t j = 0; j < H.slice_len[sl]; j++) {
                const int32_t q = H.sell_col[H.slice_ptr[sl] + 32 * j + lane];
                const int32_t t = H.seg_of_row[q];
                if (t >= 0) nb.push_back(t);
            }
        }
        std::sort(nb.begin(), nb.end());
        nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
        H.seg_nbr.insert(H.seg_nbr.end(), nb.begin(), nb.end());
        H.seg_nbr_ptr[s + 1] = (int32_t)H.seg_nbr.size();
    }
    int64_t coff = 0, xoff = 0, hxoff = 0;
    for (int b = 0; b < H.num_blobs; b++) {
        BlobParams &bp = H.bp[b];
        bp.coarse_off = (int32_t)coff;
        bp.coarse_n = 6 * bp.seg_cnt;
        bp.coarse_xoff = (int32_t)xoff;
        bp.coarse_hxoff = (int32_t)hxoff;
        coff += bp.coarse_n;
        xoff += (int64_t)bp.coarse_n * bp.coarse_n;
        hxoff += (int64_t)bp.coarse_n * ((bp.coarse_n + 7) / 8 * 8);
    }
    H.coarse_htotal = hxoff;
    return xoff;
}

void ffea_seed_words(int32_t rng_seed, uint64_t out[6])
{
    // sixseed[i] = (rand() + rand()) % twoMax[i/3] with a wrapping int sum
    // converted to unsigned long (src/World.cpp:299-305).
    GlibcRand g((uint32_t)rng_seed);
    const uint64_t two_max[2] = {4294967087ull, 4294944443ull};
    for (int i = 0; i < 6; i++) {
        int a = g.next();
        int c = g.next();
        int32_t s = (int32_t)((uint32_t)a + (uint32_t)c);
        out[i] = ((uint64_t)(int64_t)s) % two_max[i / 3];
    }
}

bool build_batch(int32_t num_blobs, const ffea_gpu_mesh *meshes, const ffea_gpu_params *params, int32_t rng_mode,
                 int32_t cg_ctas, HostBatch &out, std::string &err)
{
    if (num_blobs <= 0 || num_blobs > MAX_BLOBS) {
        err = "num_blobs must be in [1, 2^20]";
        return false;
    }
    HostBatch &H = out;
    H = HostBatch();
    H.num_blobs = num_blobs;
    H.precision = params[0].precision;
    H.rng_mode = rng_mode;
    H.bp.resize(num_blobs);
    H.maps.resize(num_blobs);

    // ---- pass 1: classify nodes, sizes ----------------------------------------
    std::vector<std::vector<int32_t>> lin_ids(num_blobs);  // per blob: orig -> local linear id
    std::vector<int32_t> nl(num_blobs), ne(num_blobs);
    int32_t node_off = 0, elem_off = 0, tile_off = 0;
    for (int b = 0; b < num_blobs; b++) {
        const ffea_gpu_mesh &m = meshes[b];
        const ffea_gpu_params &p = params[b];
        if (p.precision != H.precision) {
            err = "all blobs of a batch must use the same precision";
            return false;
        }
        if (m.num_nodes <= 0 || m.num_elements <= 0 || !m.pos || !m.topology || !m.material) {
            err = "blob " + std::to_string(b) + ": empty mesh or missing pos/topology/material";
            return false;
        }
        if (p.solver != SOLVER_NOMASS && p.solver != SOLVER_MASS && p.solver != SOLVER_LUMPED) {
            err = "unknown solver kind";
            return false;
        }
        if (!(p.dt > 0) || p.max_iterations_cg <= 0) {
            err = "dt must be > 0 and max_iterations_cg >= 1";
            return false;
        }
        const int64_t draws = (p.calc_noise == 1 ? 7ll * m.num_elements : 0) +
                              ((p.calc_noise == 1 && p.calc_stokes == 1) ? 3ll * m.num_nodes : 0);
        if (draws >= (1ll << 31)) {
            err = "blob too large for the per-step RNG offset range";
            return false;
        }
        std::vector<int8_t> kind(m.num_nodes, 0);  // 1 linear, 2 secondary
        for (int64_t e = 0; e < m.num_elements; e++)
            for (int j = 0; j < 10; j++) {
                int32_t n = m.topology[10 * e + j];
                if (n < 0 || n >= m.num_nodes) {
                    err = "blob " + std::to_string(b) + ": element " + std::to_string(e) +
                          " references an out of bounds node index";
                    return false;
                }
                int8_t k = j < 4 ? 1 : 2;
                if (kind[n] && kind[n] != k) {
                    err = "blob " + std::to_string(b) + ": node " + std::to_string(n) +
                          " is a corner of one element and a midpoint of another";
                    return false;
                }
                kind[n] = k;
            }
        for (int64_t e = 0; e < m.num_elements; e++) {
            const int32_t *t = &m.topology[10 * e];
            for (int a = 0; a < 4; a++)
                for (int c = a + 1; c < 4; c++)
                    if (t[a] == t[c]) {
                        err = "blob " + std::to_string(b) + ": element " + std::to_string(e) + " repeats a corner node";
                        return false;
                    }
        }
        lin_ids[b].assign(m.num_nodes, -1);
        int32_t cnt = 0;
        for (int32_t n = 0; n < m.num_nodes; n++)
            if (kind[n] == 1) lin_ids[b][n] = cnt++;  // provisional: original order
        nl[b] = cnt;
        ne[b] = m.num_elements;
        BlobParams &bp = H.bp[b];
        bp.dt = p.dt;
        bp.kT = p.kT;
        bp.epsilon2 = p.epsilon2;
        bp.max_iter = p.max_iterations_cg;
        bp.calc_noise = p.calc_noise;
        bp.calc_stokes = p.calc_stokes;
        bp.solver = p.solver;
        bp.true_residual = p.true_residual;
        bp.node_off = node_off;
        bp.node_cnt = cnt;
        bp.node_pad = round_up(cnt, NODE_TILE);
        bp.elem_off = elem_off;
        bp.elem_cnt = m.num_elements;
        bp.elem_pad = round_up(m.num_elements, ELEM_TILE);
        bp.tile_off = tile_off;
        bp.tile_cnt = bp.node_pad / NODE_TILE;
        bp.num_nodes_total = m.num_nodes;
        node_off += bp.node_pad;
        elem_off += bp.elem_pad;
        tile_off += bp.tile_cnt;
        if (p.solver == SOLVER_MASS) H.any_mass = 1;
        else if (p.solver == SOLVER_LUMPED) H.any_lumped = 1;
        else H.any_nomass = 1;
        if ((int64_t)node_off >= (1ll << 30) || (int64_t)elem_off >= (1ll << 28)) {
            err = "batch too large";
            return false;
        }
    }
    H.nl_pad = node_off;
    H.ne_pad = elem_off;
    H.n_tiles = tile_off;
    H.n_etiles = elem_off / ELEM_TILE;

    // ---- linear node order: each blob's CG segments are compact blocks ---------
    H.parts = plan_parts(nl, std::max(1, cg_ctas), CG_SEG_MAX_ROWS);
    for (int b = 0; b < num_blobs; b++) {
        const ffea_gpu_mesh &m = meshes[b];
        const int32_t n = nl[b];
        std::vector<double> lp(3 * (size_t)n);
        std::vector<int32_t> orig_of(n);
        for (int32_t v = 0; v < m.num_nodes; v++) {
            const int32_t l = lin_ids[b][v];
            if (l < 0) continue;
            orig_of[l] = v;
            for (int c = 0; c < 3; c++) lp[3 * (size_t)l + c] = m.pos[3 * (size_t)v + c];
        }
        // grid spacing of the in-segment order: mean corner-edge length
        double hsum = 0.0;
        int64_t hcnt = 0;
        for (int64_t e = 0; e < std::min<int64_t>(m.num_elements, 4096); e++) {
            const int32_t *t = &m.topology[10 * e];
            for (int a = 0; a < 4; a++)
                for (int c = a + 1; c < 4; c++) {
                    double d2 = 0.0;
                    for (int x = 0; x < 3; x++) {
                        const double dd = m.pos[3 * (size_t)t[a] + x] - m.pos[3 * (size_t)t[c] + x];
                        d2 += dd * dd;
                    }
                    hsum += std::sqrt(d2);
                    hcnt++;
                }
        }
        const double h = hcnt && hsum > 0 ? hsum / (double)hcnt : 1.0;
        std::vector<int32_t> ids(n);
        std::iota(ids.begin(), ids.end(), 0);
        rcb(lp.data(), ids, 0, n, n, H.parts[b], 0, H.parts[b], h);
        for (int32_t r = 0; r < n; r++) lin_ids[b][orig_of[ids[r]]] = r;
    }

    // ---- materials (deduplicated table) ---------------------------------------
    std::map<std::vector<double>, uint16_t> mat_index;
    H.mat_id.assign(H.ne_pad, 0);
    H.conn.assign(4 * (size_t)H.ne_pad, 0);
    H.etile_blob.assign(H.n_etiles, 0);
    H.tile_blob.assign(H.n_tiles, 0);
    for (int b = 0; b < num_blobs; b++) {
        const ffea_gpu_mesh &m = meshes[b];
        const BlobParams &bp = H.bp[b];
        for (int t = 0; t < bp.elem_pad / ELEM_TILE; t++) H.etile_blob[bp.elem_off / ELEM_TILE + t] = b;
        for (int t = 0; t < bp.tile_cnt; t++) H.tile_blob[bp.tile_off + t] = b;
        for (int64_t e = 0; e < m.num_elements; e++) {
            std::vector<double> key(m.material + 5 * e, m.material + 5 * e + 5);
            auto it = mat_index.find(key);
            uint16_t id;
            if (it == mat_index.end()) {
                if (H.materials.size() >= 65535) {
                    err = "more than 65535 distinct element materials";
                    return false;
                }
                id = (uint16_t)H.materials.size();
                mat_index.emplace(key, id);
                H.materials.push_back(Material{key[0], key[1], key[2], key[3], key[4]});
            } else {
                id = it->second;
            }
            const size_t ge = (size_t)bp.elem_off + e;
            H.mat_id[ge] = id;
            for (int a = 0; a < 4; a++) H.conn[4 * ge + a] = bp.node_off + lin_ids[b][m.topology[10 * e + a]];
        }
        // padding elements reference the blob's first node; they are skipped by count
        for (int64_t e = m.num_elements; e < bp.elem_pad; e++)
            for (int a = 0; a < 4; a++) H.conn[4 * ((size_t)bp.elem_off + e) + a] = bp.node_off;
    }
    if (H.materials.empty()) H.materials.push_back(Material{0, 0, 0, 0, 0});

    // ---- nodes ---------------------------------------------------------------
    H.pos.assign(3 * (size_t)H.nl_pad, 0.0);
    H.vel.assign(3 * (size_t)H.nl_pad, 0.0);
    H.drag.assign(H.nl_pad, 0.0);
    H.flags.assign(H.nl_pad, NODE_PINNED);
    H.orig.assign(H.nl_pad, -1);
    for (int b = 0; b < num_blobs; b++) {
        const ffea_gpu_mesh &m = meshes[b];
        const BlobParams &bp = H.bp[b];
        BlobMap &map = H.maps[b];
        map.num_nodes_total = m.num_nodes;
        map.num_elements = m.num_elements;
        map.lin_of_orig.assign(m.num_nodes, -1);
        map.topology.assign(m.topology, m.topology + 10 * (size_t)m.num_elements);
        map.pinned_orig.assign(m.num_nodes, 0);
        map.drag_orig.assign(m.num_nodes, 0.0);
        if (m.stokes_drag) map.drag_orig.assign(m.stokes_drag, m.stokes_drag + m.num_nodes);
        for (int i = 0; i < m.num_pinned; i++) {
            int32_t pn = m.pinned[i];
            if (pn < 0 || pn >= m.num_nodes) {
                err = "pinned node index out of range";
                return false;
            }
            map.pinned_orig[pn] = 1;
        }
        for (int32_t n = 0; n < m.num_nodes; n++) {
            int32_t l = lin_ids[b][n];
            if (l < 0) continue;
            const int32_t g = bp.node_off + l;
            map.lin_of_orig[n] = g;
            for (int c = 0; c < 3; c++) {
                H.pos[3 * (size_t)g + c] = m.pos[3 * (size_t)n + c];
                H.vel[3 * (size_t)g + c] = m.vel ? m.vel[3 * (size_t)n + c] : 0.0;
            }
            H.drag[g] = m.stokes_drag ? m.stokes_drag[n] : 0.0;
            H.flags[g] = map.pinned_orig[n] ? NODE_PINNED : 0;
            H.orig[g] = n;
        }
    }

    // ---- gather lists: node -> (elem, corner) in element order ------------------
    {
        std::vector<int32_t> cnt(H.nl_pad + 1, 0);
        for (int b = 0; b < num_blobs; b++) {
            const BlobParams &bp = H.bp[b];
            for (int64_t e = 0; e < bp.elem_cnt; e++)
                for (int a = 0; a < 4; a++) cnt[H.conn[4 * ((size_t)bp.elem_off + e) + a] + 1]++;
        }
        std::partial_sum(cnt.begin(), cnt.end(), cnt.begin());
        H.gather_ptr = cnt;
        H.gather_idx.assign(cnt.back(), 0);
        std::vector<int32_t> fill(H.nl_pad, 0);
        for (int b = 0; b < num_blobs; b++) {
            const BlobParams &bp = H.bp[b];
            for (int64_t e = 0; e < bp.elem_cnt; e++) {
                const size_t ge = (size_t)bp.elem_off + e;
                for (int a = 0; a < 4; a++) {
                    int32_t g = H.conn[4 * ge + a];
                    H.gather_idx[H.gather_ptr[g] + fill[g]++] = (int32_t)(ge * 4 + a);
                }
            }
        }
    }

    // ---- secondary nodes with a drag: fold half of their noise onto the two
    //      corners of the first element that holds them ---------------------------
    {
        std::vector<std::vector<std::pair<int32_t, double>>> fold(H.nl_pad);
        for (int b = 0; b < num_blobs; b++) {
            const ffea_gpu_mesh &m = meshes[b];
            const ffea_gpu_params &p = params[b];
            if (!m.stokes_drag || p.calc_stokes != 1 || p.calc_noise != 1) continue;
            std::vector<uint8_t> seen(m.num_nodes, 0);
            for (int64_t e = 0; e < m.num_elements; e++)
                for (int j = 4; j < 10; j++) {
                    int32_t s = m.topology[10 * e + j];
                    if (seen[s]) continue;
                    seen[s] = 1;
                    if (m.stokes_drag[s] == 0.0) continue;
                    for (int k = 0; k < 2; k++) {
                        int32_t corner = m.topology[10 * e + kMid[j - 4][k]];
                        // noise amplitude of the secondary node, the expression of
                        // src/Blob.cpp:3896 evaluated once here instead of every step
                        fold[H.maps[b].lin_of_orig[corner]].push_back(
                            {s, std::sqrt((24 * p.kT * m.stokes_drag[s]) / (p.dt))});
                    }
                }
        }
        H.fold_ptr.assign(H.nl_pad + 1, 0);
        for (int32_t g = 0; g < H.nl_pad; g++) H.fold_ptr[g + 1] = H.fold_ptr[g] + (int32_t)fold[g].size();
        for (int32_t g = 0; g < H.nl_pad; g++)
            for (auto &pr : fold[g]) {
                H.fold_sec.push_back(pr.first);
                H.fold_amp.push_back(pr.second);
            }
        // the same amplitude for the linear nodes' own draws
        H.node_amp.assign(H.nl_pad, 0.0);
        for (int b = 0; b < num_blobs; b++) {
            const ffea_gpu_params &p = params[b];
            if (p.calc_stokes != 1 || p.calc_noise != 1) continue;
            const BlobParams &bp = H.bp[b];
            for (int32_t g = bp.node_off; g < bp.node_off + bp.node_cnt; g++)
                if (H.drag[g] != 0.0) H.node_amp[g] = std::sqrt((24 * p.kT * H.drag[g]) / (p.dt));
        }
    }

    // ---- edges and their (elem, a, b) terms -------------------------------------
    {
        struct Term {
            int64_t key;
            int32_t cidx;
        };
        std::vector<Term> terms;
        size_t total = 0;
        for (int b = 0; b < num_blobs; b++) total += 6 * (size_t)H.bp[b].elem_cnt;
        terms.reserve(total);
        for (int b = 0; b < num_blobs; b++) {
            const BlobParams &bp = H.bp[b];
            for (int64_t e = 0; e < bp.elem_cnt; e++) {
                const size_t ge = (size_t)bp.elem_off + e;
                for (int a = 0; a < 4; a++)
                    for (int c = a + 1; c < 4; c++) {
                        int32_t na = H.conn[4 * ge + a], nc = H.conn[4 * ge + c];
                        int32_t lo = na < nc ? na : nc, hi = na < nc ? nc : na;
                        int la = na < nc ? a : c, lc = na < nc ? c : a;  // local corner of lo / hi
                        terms.push_back(Term{(int64_t)lo * H.nl_pad + hi, (int32_t)(ge * 16 + la * 4 + lc)});
                    }
            }
        }
        std::stable_sort(terms.begin(), terms.end(), [](const Term &x, const Term &y) { return x.key < y.key; });
        for (size_t i = 0; i < terms.size(); i++) {
            if (i == 0 || terms[i].key != terms[i - 1].key) {
                H.edge_p.push_back((int32_t)(terms[i].key / H.nl_pad));
                H.edge_q.push_back((int32_t)(terms[i].key % H.nl_pad));
                H.edge_cptr.push_back((int32_t)i);
            }
            H.edge_cidx.push_back(terms[i].cidx);
        }
        H.edge_cptr.push_back((int32_t)terms.size());
        H.n_edges = (int32_t)H.edge_p.size();
        if ((int64_t)terms.size() >= (1ll << 31)) {
            err = "too many edge terms";
            return false;
        }
        // SELL-32 rows: neighbours in ascending column order
        std::vector<int32_t> deg(H.nl_pad + 1, 0);
        for (int32_t e = 0; e < H.n_edges; e++) {
            deg[H.edge_p[e] + 1]++;
            deg[H.edge_q[e] + 1]++;
        }
        std::partial_sum(deg.begin(), deg.end(), deg.begin());
        std::vector<int64_t> adj(deg.back());  // (col << 32) | edge
        std::vector<int32_t> fill(H.nl_pad, 0);
        for (int32_t e = 0; e < H.n_edges; e++) {
            const int32_t p = H.edge_p[e], q = H.edge_q[e];
            adj[deg[p] + fill[p]++] = ((int64_t)q << 32) | (uint32_t)e;
            adj[deg[q] + fill[q]++] = ((int64_t)p << 32) | (uint32_t)e;
        }
        for (int32_t r = 0; r < H.nl_pad; r++) std::sort(adj.begin() + deg[r], adj.begin() + deg[r + 1]);
        const int32_t nslices = H.nl_pad / 32;
        H.slice_ptr.assign(nslices + 1, 0);
        H.slice_len.assign(nslices, 0);
        for (int32_t sl = 0; sl < nslices; sl++) {
            int32_t L = 0;
            for (int32_t r = 32 * sl; r < 32 * sl + 32; r++) L = std::max(L, deg[r + 1] - deg[r]);
            H.slice_len[sl] = L;
            if ((int64_t)H.slice_ptr[sl] + 32ll * L >= (1ll << 31)) {
                err = "matrix too large for 32-bit SELL offsets";
                return false;
            }
            H.slice_ptr[sl + 1] = H.slice_ptr[sl] + 32 * L;
        }
        H.sell_col.assign(H.slice_ptr[nslices], 0);
        H.edge_pos_pq.assign(H.n_edges, 0);
        H.edge_pos_qp.assign(H.n_edges, 0);
        for (int32_t r = 0; r < H.nl_pad; r++) {
            const int32_t sl = r / 32, lane = r % 32;
            for (int32_t j = 0; j < H.slice_len[sl]; j++) H.sell_col[H.slice_ptr[sl] + 32 * j + lane] = r;  // padding: own row
            for (int32_t j = 0; j < deg[r + 1] - deg[r]; j++) {
                const int64_t v = adj[deg[r] + j];
                const int32_t col = (int32_t)(v >> 32), e = (int32_t)(v & 0xffffffff);
                const int32_t off = H.slice_ptr[sl] + 32 * j + lane;
                H.sell_col[off] = col;
                if (r == H.edge_p[e]) H.edge_pos_pq[e] = off;
                else H.edge_pos_qp[e] = off;
            }
        }
    }

    // ---- RNG streams ----------------------------------------------------------------
    {
        H.num_streams = (rng_mode == FFEA_GPU_RNG_SHARED) ? 1 : num_blobs;
        H.stream_state.assign(6 * (size_t)H.num_streams, 0);
        std::vector<uint64_t> per_stream_draws(H.num_streams, 0);
        // element draws of every blob first, then node draws (World::run order)
        uint64_t acc = 0;
        for (int b = 0; b < num_blobs; b++) {
            const ffea_gpu_params &p = params[b];
            BlobParams &bp = H.bp[b];
            bp.stream = (rng_mode == FFEA_GPU_RNG_SHARED) ? 0 : b;
            uint64_t base = (rng_mode == FFEA_GPU_RNG_SHARED) ? acc : 0;
            bp.elem_draw_base = (uint32_t)base;
            // a blob with every node pinned skips its element loop and with
            // it the element draws (src/Blob.cpp:643-645)
            bp.all_pinned = meshes[b].num_pinned == meshes[b].num_nodes ? 1 : 0;
            uint64_t ed = (p.calc_noise == 1 && !bp.all_pinned) ? 7ull * meshes[b].num_elements : 0;
            if (rng_mode == FFEA_GPU_RNG_SHARED) acc += ed;
            else per_stream_draws[b] = ed;
        }
        for (int b = 0; b < num_blobs; b++) {
            const ffea_gpu_params &p = params[b];
            BlobParams &bp = H.bp[b];
            uint64_t nd = (p.calc_noise == 1 && p.calc_stokes == 1) ? 3ull * meshes[b].num_nodes : 0;
            if (rng_mode == FFEA_GPU_RNG_SHARED) {
                bp.node_draw_base = (uint32_t)acc;
                acc += nd;
            } else {
                bp.node_draw_base = (uint32_t)per_stream_draws[b];
                per_stream_draws[b] += nd;
            }
        }
        if (rng_mode == FFEA_GPU_RNG_SHARED) {
            if (acc >= (1ull << 32)) {
                err = "shared RNG stream: more than 2^32 draws per step";
                return false;
            }
            per_stream_draws[0] = acc;
        }
        // runs of the noise kernel: each generates NOISE_RUN consecutive
        // draws of one blob's element or node range after one jump
        H.noise_run_off.assign(2 * (size_t)num_blobs + 1, 0);
        int64_t runs = 0, nodes = 0;
        for (int b = 0; b < num_blobs; b++) {
            const ffea_gpu_params &p = params[b];
            const int64_t ed = (p.calc_noise == 1 && !H.bp[b].all_pinned) ? 7ll * meshes[b].num_elements : 0;
            const int64_t nd = (p.calc_noise == 1 && p.calc_stokes == 1) ? 3ll * meshes[b].num_nodes : 0;
            // the node kernel reads the draws of nodes with a Stokes drag only
            // (a zero drag multiplies its draws by zero): generate the draws
            // up to the last such node; the stream still advances by all
            // 3 N_t draws of the step (stream_step)
            int64_t nd_used = 0;
            if (nd && meshes[b].stokes_drag)
                for (int32_t n = meshes[b].num_nodes - 1; n >= 0; n--)
                    if (meshes[b].stokes_drag[n] != 0.0) {
                        nd_used = 3ll * (n + 1);
                        break;
                    }
            H.noise_run_off[2 * b] = (int32_t)runs;
            runs += (ed + NOISE_RUN - 1) / NOISE_RUN;
            H.noise_run_off[2 * b + 1] = (int32_t)runs;
            runs += (nd_used + NOISE_RUN - 1) / NOISE_RUN;
            H.bp[b].noise_node_off = (int32_t)nodes;
            if (nd) nodes += meshes[b].num_nodes;
        }
        if (runs >= (1ll << 31) || nodes >= (1ll << 31)) {
            err = "too many random draws per step";
            return false;
        }
        H.noise_run_off[2 * (size_t)num_blobs] = (int32_t)runs;
        H.noise_nodes = nodes;
        H.stream_step.resize(H.num_streams);
        for (int s = 0; s < H.num_streams; s++) {
            uint64_t six[6];
            ffea_seed_words(params[s].rng_seed, six);
            for (int i = 0; i < 6; i++) H.stream_state[6 * (size_t)s + i] = (uint32_t)six[i];
            H.stream_step[s] = mrg::jm_pow(mrg::jm_step(), per_stream_draws[s]);
        }
    }
    return true;
}

}  // namespace ffea
