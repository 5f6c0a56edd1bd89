// mavi_invasions.cu — invasion detection of the rings model: check_invasions!
// (src/rings/integration.jl:378-509) on the device, scheduled by
// update_invasions! (:511-520) from the host side of mavi_step, and the two
// C-ABI entry points of include/mavi_cuda.h that configure and read it.
//
// A check runs three kernels over the replicas that are due:
//   k_inv_prepare  one thread per ring: the continuous polygon
//                  (update_continuos_pos!, :118-138), its bounding box and,
//                  with ring chunks, the chunk of the ring's centre
//                  (update_particle_chunk!, src/chunks.jl:120-147, on
//                  RingsInfo.cms) with a per-chunk count;
//   k_inv_lists    one block per replica: the rings of get_rings_ids, and the
//                  ring-chunk lists in ascending ring order (update_chunks!,
//                  src/rings/integration.jl:18-23) with each ring's place;
//   k_inv_pairs    one warp per ring: the pairs check_invasions! visits, each
//                  through find_invasions! (:443-470) with the exact
//                  point_line_intersect (:378-418) in FP64, lanes over points.
// Each record carries the reference's visiting order as a sort key; the host
// sorts the (short) list into the order the reference pushes it.
//
// Pair filter (exact): point_line_intersect needs y1 < p.y < y2 strictly
// and x_inter > p.x with x_inter strictly inside the edge's x-range, so a
// point with p.y <= ymin, p.y >= ymax or p.x >= xmax of the other polygon's
// vertices crosses no edge. Such points, and ring pairs whose boxes rule out
// every point, are skipped without changing any count.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mavi_system.cuh"

namespace mavi {

struct InvRepD {
    int32_t rep, use_chunks, rows, cols;
    int64_t chunk0;
    double blx, bly, h, cl, ch;
    int32_t from_sources, _pad;
};

struct InvRecord {      // sort key (k0..k4, pi) then the Invasion
    int32_t k0, k1, k2, k3, k4, pi, invasor, invaded;
};

struct InvDev {
    double2* cont;
    double* bb;
    int32_t *chunk_of, *rank, *list, *count, *start;
    const int32_t* nbr;
    int32_t* num_ids;
    InvRecord* rec;
    int32_t* nrec;
    int64_t cap;
};

constexpr int kInvPrepThreads = 128;
constexpr int kInvListThreads = 1024;
constexpr int kInvPairThreads = 256;

// point_line_intersect (src/rings/integration.jl:378-418), FP64 without
// contraction: the crossing of the ray from p towards +x with the edge a-b.
__device__ __forceinline__ bool inv_point_line(double px, double py, double2 a, double2 b) {
    const double dx = __dsub_rn(b.x, a.x), dy = __dsub_rn(b.y, a.y);
    double ylo = a.y, yhi = b.y;
    if (dy < 0) { ylo = b.y; yhi = a.y; }
    if (dx == 0) return (a.x > px) & (ylo < py) & (py < yhi);
    if (dy == 0) return false;
    const double c = __dsub_rn(__dmul_rn(dy, a.x), __dmul_rn(dx, a.y));
    const double xi = __ddiv_rn(__dadd_rn(c, __dmul_rn(dx, py)), dy);
    double xlo = a.x, xhi = b.x;
    if (dx < 0) { xlo = b.x; xhi = a.x; }
    return (xi > px) & (xlo < xi) & (xi < xhi) & (ylo < py) & (py < yhi);
}

__device__ __forceinline__ bool inv_active(const Ctx& C, int64_t g) {
    return C.ring_active ? C.ring_active[g] != 0 : true;
}

// update_cms! for one ring at the check (src/rings/integration.jl:366-372):
// with periodic walls the continuous positions of the previous
// update_continuos_pos! (ring_centre reads them from the *_cur state), else
// the mean of the current positions.
__device__ __forceinline__ double2 inv_centre(const Ctx& C, const DevRep& R, int32_t ring, int32_t n) {
    if (R.periodic) return ring_centre(C, R, ring, n);
    const int64_t u0 = R.slot0 + (int64_t)ring * R.nmax;
    const double2 q0 = C.pos_u[u0];
    double sx = q0.x, sy = q0.y;
    for (int32_t p = 1; p < n; p++) {
        const double2 q = C.pos_u[u0 + p];
        sx += q.x; sy += q.y;
    }
    return make_double2(sx / n, sy / n);
}

__global__ void __launch_bounds__(kInvPrepThreads) k_inv_prepare(Ctx C, const InvRepD* __restrict__ IR, InvDev B) {
    const InvRepD I = IR[blockIdx.y];
    const DevRep& R = C.reps[I.rep];
    const int32_t k = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
    if (k >= R.num_rings) return;
    const int64_t g = R.ring0 + k;
    const int32_t n = C.rcfg[I.rep].num_particles[C.ring_types[g] - 1];
    const int64_t u0 = R.slot0 + (int64_t)k * R.nmax;
    // ring_points: continuous positions with periodic walls, else positions
    double2 prev = C.pos_u[u0];
    double cx = prev.x, cy = prev.y;
    double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
    for (int32_t p = 0; p < n; p++) {
        if (p > 0) {
            const double2 q = C.pos_u[u0 + p];
            if (R.periodic) {
                double dx = __dsub_rn(q.x, prev.x), dy = __dsub_rn(q.y, prev.y);
                if (R.min_image) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
                cx = __dadd_rn(cx, dx);
                cy = __dadd_rn(cy, dy);
            } else {
                cx = q.x; cy = q.y;
            }
            prev = q;
        }
        B.cont[u0 + p] = make_double2(cx, cy);
        if (cx < xmin) xmin = cx;    // NaN vertices stay out of the box: their edges never count
        if (cx > xmax) xmax = cx;
        if (cy < ymin) ymin = cy;
        if (cy > ymax) ymax = cy;
    }
    B.bb[4 * g + 0] = xmin; B.bb[4 * g + 1] = xmax;
    B.bb[4 * g + 2] = ymin; B.bb[4 * g + 3] = ymax;
    if (!I.use_chunks) return;
    int32_t cell = -1;
    if (inv_active(C, g)) {
        const double2 m = (I.from_sources && R.src_ne > 0) ? C.ring_cms[g] : inv_centre(C, R, k, n);
        const double qr = julia_div(__dadd_rn(__dadd_rn(-m.y, I.bly), I.h), I.ch);
        const double qc = julia_div(__dsub_rn(m.x, I.blx), I.cl);
        const bool finite = isfinite(qr) && isfinite(qc) && fabs(qr) < 4e18 && fabs(qc) < 4e18;
        int64_t row = finite ? (int64_t)qr + 1 : 0, col = finite ? (int64_t)qc + 1 : 0;
        row -= (row == (int64_t)I.rows + 1) ? 1 : 0;
        col -= (col == (int64_t)I.cols + 1) ? 1 : 0;
        if (!finite || row < 1 || row > I.rows || col < 1 || col > I.cols) {
            // the reference's chunk_particles[p_i, row, col] raises a BoundsError
            raise_error(C.err, finite ? MAVI_ERR_OUT_OF_GRID : MAVI_ERR_NONFINITE, -1,
                        finite ? row * 1000003 + col : 0);
        } else {
            cell = (int32_t)((col - 1) * I.rows + (row - 1));   // the column-major traversal order
            atomicAdd(&B.count[I.chunk0 + cell], 1);
        }
    }
    B.chunk_of[g] = cell;
}

__global__ void __launch_bounds__(kInvListThreads) k_inv_lists(Ctx C, const InvRepD* __restrict__ IR, InvDev B) {
    __shared__ int smem[32];
    const InvRepD I = IR[blockIdx.x];
    const DevRep& R = C.reps[I.rep];
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int32_t nr = R.num_rings;
    // length(get_rings_ids(state)): the active rings
    int a = 0;
    for (int32_t k = tid; k < nr; k += nthr) a += inv_active(C, R.ring0 + k) ? 1 : 0;
    int total;
    block_exclusive_scan(a, smem, total);
    if (tid == 0) B.num_ids[blockIdx.x] = total;
    if (!I.use_chunks) return;
    const int64_t nch = (int64_t)I.rows * I.cols;
    int32_t* count = B.count + I.chunk0;
    int32_t* start = B.start + I.chunk0;
    int base = 0;
    for (int64_t c0 = 0; c0 < nch; c0 += nthr) {
        const int64_t c = c0 + tid;
        const int v = c < nch ? count[c] : 0;
        const int ex = block_exclusive_scan(v, smem, total);
        if (c < nch) { start[c] = base + ex; count[c] = 0; }
        base += total;
    }
    __syncthreads();
    int32_t* list = B.list + R.ring0;
    for (int32_t k = tid; k < nr; k += nthr) {
        const int32_t c = B.chunk_of[R.ring0 + k];
        if (c >= 0) list[start[c] + atomicAdd(&count[c], 1)] = k;
    }
    __syncthreads();
    // update_chunks! appends in ascending ring order: sort each list, then places
    for (int64_t c = tid; c < nch; c += nthr) {
        int32_t* L = list + start[c];
        const int32_t m = count[c];
        for (int32_t i = 1; i < m; i++) {
            const int32_t v = L[i];
            int32_t j = i - 1;
            while (j >= 0 && L[j] > v) { L[j + 1] = L[j]; j--; }
            L[j + 1] = v;
        }
        for (int32_t i = 0; i < m; i++) B.rank[R.ring0 + L[i]] = i;
    }
}

// One direction of find_invasions!: the points of ring a (polygons_intersect,
// :420-441) inside ring b, one lane per point.
__device__ __forceinline__ void inv_direction(const DevRep& R, const InvDev& B, int32_t a, int32_t b, int32_t na,
                                              int32_t nb, const int32_t key[4], int32_t dir, int lane) {
    const int64_t ga = R.ring0 + a, gb = R.ring0 + b;
    const double bxmax = B.bb[4 * gb + 1], bymin = B.bb[4 * gb + 2], bymax = B.bb[4 * gb + 3];
    if (!(B.bb[4 * ga + 3] > bymin) || !(B.bb[4 * ga + 2] < bymax) || !(B.bb[4 * ga + 0] < bxmax)) return;
    const double2* pa = B.cont + R.slot0 + (int64_t)a * R.nmax;
    const double2* pb = B.cont + R.slot0 + (int64_t)b * R.nmax;
    for (int32_t p = lane; p < na; p += 32) {
        const double2 q = pa[p];
        if (!(q.y > bymin) || !(q.y < bymax) || !(q.x < bxmax)) continue;
        int cnt = 0;
        double2 e0 = pb[0];
        for (int32_t e = 0; e < nb; e++) {
            const double2 e1 = pb[e + 1 == nb ? 0 : e + 1];
            cnt += inv_point_line(q.x, q.y, e0, e1) ? 1 : 0;
            e0 = e1;
        }
        if (cnt & 1) {
            const int32_t at = atomicAdd(B.nrec, 1);
            if (at < B.cap) {
                InvRecord r;
                r.k0 = key[0]; r.k1 = key[1]; r.k2 = key[2]; r.k3 = key[3]; r.k4 = dir; r.pi = p;
                r.invasor = a; r.invaded = b;
                B.rec[at] = r;
            }
        }
    }
}

__global__ void __launch_bounds__(kInvPairThreads) k_inv_pairs(Ctx C, const InvRepD* __restrict__ IR, InvDev B) {
    const InvRepD I = IR[blockIdx.y];
    const DevRep& R = C.reps[I.rep];
    const int lane = threadIdx.x & 31;
    const int32_t k = (int32_t)(blockIdx.x * (kInvPairThreads / 32) + (threadIdx.x >> 5));
    if (k >= R.num_rings) return;
    const MaviRingsCfg& rc = C.rcfg[I.rep];
    const int32_t n1 = rc.num_particles[C.ring_types[R.ring0 + k] - 1];
    auto visit = [&](int32_t r2, const int32_t key[4]) {
        const int32_t n2 = rc.num_particles[C.ring_types[R.ring0 + r2] - 1];
        // k4: the direction, and the replica's place in this check above it
        inv_direction(R, B, k, r2, n1, n2, key, 0 + 2 * (int32_t)blockIdx.y, lane);
        inv_direction(R, B, r2, k, n2, n1, key, 1 + 2 * (int32_t)blockIdx.y, lane);
    };
    if (!I.use_chunks) {
        // check_invasions!(system, ::Nothing): ring ids 1:length(get_rings_ids)
        const int32_t L = B.num_ids[blockIdx.y];
        if (k >= L) return;
        for (int32_t r2 = k + 1; r2 < L; r2++) {
            const int32_t key[4] = {k, 0, 0, r2};
            visit(r2, key);
        }
        return;
    }
    const int32_t c = B.chunk_of[R.ring0 + k];
    if (c < 0) return;
    const int32_t i = B.rank[R.ring0 + k];
    const int32_t* list = B.list + R.ring0;
    const int32_t* start = B.start + I.chunk0;
    const int32_t* count = B.count + I.chunk0;
    for (int32_t j = i + 1; j < count[c]; j++) {
        const int32_t key[4] = {c, i, 0, j};
        visit(list[start[c] + j], key);
    }
    for (int s = 0; s < 4; s++) {
        const int32_t nc = B.nbr[4 * (I.chunk0 + c) + s];
        if (nc < 0) continue;
        for (int32_t j = 0; j < count[nc]; j++) {
            const int32_t key[4] = {c, i, s + 1, j};
            visit(list[start[nc] + j], key);
        }
    }
}

// get_neighbors (src/chunks.jl:61-118) of a rows x cols grid, 0-based
// column-major chunk ids, 4 entries per chunk (-1: none). Returns false for an
// open grid of one column and several rows, whose lists index column 0.
static bool ring_chunk_neighbors(int32_t rows, int32_t cols, bool periodic, std::vector<int32_t>& nbr) {
    nbr.assign((size_t)4 * rows * cols, -1);
    std::vector<int32_t> cnt((size_t)rows * cols, 0);
    auto id = [&](int64_t r1, int64_t c1) { return (c1 - 1) * rows + (r1 - 1); };
    auto add = [&](int64_t r1, int64_t c1, int64_t nr1, int64_t nc1) {
        const int64_t c = id(r1, c1);
        nbr[4 * c + cnt[c]++] = (int32_t)id(nr1, nc1);
    };
    if (periodic) {
        auto gid = [](int64_t x, int64_t nt) -> int64_t {
            if (x == 0) return nt;
            if (x % (nt + 1) == 0) return 1;
            return x;
        };
        for (int64_t i = 1; i <= rows; i++)
            for (int64_t j = 1; j <= cols; j++) {
                add(i, j, gid(i + 1, rows), gid(j, cols));
                add(i, j, gid(i + 1, rows), gid(j + 1, cols));
                add(i, j, gid(i, rows), gid(j + 1, cols));
                add(i, j, gid(i - 1, rows), gid(j + 1, cols));
            }
        return true;
    }
    if (cols < 2 && rows > 1) return false;
    for (int64_t i = 1; i <= rows - 1; i++) {
        add(i, 1, i + 1, 1);
        add(i, 1, i + 1, 2);
        add(i, 1, i, 2);
        for (int64_t j = 2; j <= cols - 1; j++) {
            add(i, j, i + 1, j - 1);
            add(i, j, i + 1, j);
            add(i, j, i + 1, j + 1);
            add(i, j, i, j + 1);
        }
        // neighbors[i, num_cols] is assigned (replacing column 1's list when cols == 1)
        const int64_t c = id(i, cols);
        for (int s = 0; s < 4; s++) nbr[4 * c + s] = -1;
        cnt[c] = 0;
        add(i, cols, i + 1, cols - 1);
        add(i, cols, i + 1, cols);
    }
    for (int64_t j = 1; j <= cols - 1; j++) add(rows, j, rows, j + 1);
    return true;
}

static void free_dev(MaviSystem* s, void* p) {
    if (!p) return;
    cudaFree(p);
    s->allocs.erase(std::remove(s->allocs.begin(), s->allocs.end(), p), s->allocs.end());
}

static void sort_records(std::vector<InvRecord>& r) {
    std::sort(r.begin(), r.end(), [](const InvRecord& a, const InvRecord& b) {
        if (a.k0 != b.k0) return a.k0 < b.k0;
        if (a.k1 != b.k1) return a.k1 < b.k1;
        if (a.k2 != b.k2) return a.k2 < b.k2;
        if (a.k3 != b.k3) return a.k3 < b.k3;
        if (a.k4 != b.k4) return a.k4 < b.k4;
        return a.pi < b.pi;
    });
}

int run_invasions(MaviSystem* s, const std::vector<int32_t>& due, bool from_sources) {
    if (due.empty()) return MAVI_OK;
    constexpr size_t kMaxGridY = 65535;   // the replicas of one check ride on gridDim.y
    if (due.size() > kMaxGridY) {
        for (size_t a = 0; a < due.size(); a += kMaxGridY) {
            std::vector<int32_t> part(due.begin() + a, due.begin() + std::min(due.size(), a + kMaxGridY));
            int rc = run_invasions(s, part, from_sources);
            if (rc) return rc;
        }
        return MAVI_OK;
    }
    MaviSystem::InvBuffers& b = s->invb;
    std::vector<InvRepD> reps(due.size());
    int32_t max_rings = 0;
    for (size_t q = 0; q < due.size(); q++) {
        const MaviSystem::InvCfg& c = s->inv[due[q]];
        InvRepD& d = reps[q];
        d.rep = due[q];
        d.use_chunks = c.cols > 0 ? 1 : 0;
        d.rows = c.rows; d.cols = c.cols; d.chunk0 = c.chunk0;
        d.blx = c.blx; d.bly = c.bly; d.h = c.h; d.cl = c.cl; d.ch = c.ch;
        d.from_sources = from_sources ? 1 : 0;
        max_rings = std::max(max_rings, s->reps_h[due[q]].num_rings);
    }
    if (max_rings == 0) {
        for (int32_t r : due) {
            if (s->inv[r].cols > 0) s->inv[r].list.clear();
            s->inv[r].last_check = s->num_steps[r];
        }
        return MAVI_OK;
    }
    CUDA_TRY(s, cudaMemcpyAsync(b.reps, reps.data(), sizeof(InvRepD) * reps.size(), cudaMemcpyHostToDevice, s->stream));
    if (b.nch > 0) CUDA_TRY(s, cudaMemsetAsync(b.count, 0, sizeof(int32_t) * b.nch, s->stream));
    InvDev D{b.cont, b.bb, b.chunk_of, b.rank, b.list, b.count, b.start, b.nbr, b.num_ids,
             static_cast<InvRecord*>(b.rec), b.nrec, b.rec_cap};
    const InvRepD* dr = static_cast<const InvRepD*>(b.reps);
    const unsigned ndue = (unsigned)due.size();
    k_inv_prepare<<<dim3(nblocks(max_rings, kInvPrepThreads), ndue), kInvPrepThreads, 0, s->stream>>>(s->C, dr, D);
    k_inv_lists<<<ndue, kInvListThreads, 0, s->stream>>>(s->C, dr, D);
    int32_t nrec = 0;
    for (int attempt = 0; attempt < 2; attempt++) {
        CUDA_TRY(s, cudaMemsetAsync(b.nrec, 0, sizeof(int32_t), s->stream));
        k_inv_pairs<<<dim3(nblocks(max_rings, kInvPairThreads / 32), ndue), kInvPairThreads, 0, s->stream>>>(s->C, dr, D);
        CUDA_TRY(s, cudaGetLastError());
        CUDA_TRY(s, cudaMemcpyAsync(&nrec, b.nrec, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
        int rc = device_error_status(s);   // waits
        if (rc) return rc;
        if (nrec <= b.rec_cap) break;
        // more invasions than the record buffer holds: grow it and pair again
        free_dev(s, b.rec);
        b.rec = nullptr;
        b.rec_cap = (int64_t)nrec * 2;
        if (dalloc(s, reinterpret_cast<InvRecord**>(&b.rec), b.rec_cap) != cudaSuccess)
            return fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for %lld invasion records", (long long)b.rec_cap);
        D.rec = static_cast<InvRecord*>(b.rec);
        D.cap = b.rec_cap;
    }
    if (nrec > b.rec_cap)   // the second pass finds what the first did; never copy past the buffer
        return fail(s, MAVI_ERR_CUDA, "invasion records: %d found, room for %lld", nrec, (long long)b.rec_cap);
    std::vector<InvRecord> rec((size_t)nrec);
    if (nrec > 0)
        CUDA_TRY(s, cudaMemcpyAsync(rec.data(), b.rec, sizeof(InvRecord) * nrec, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    // records of several replicas share the buffer: split by replica first
    std::vector<std::vector<InvRecord>> per(due.size());
    for (const InvRecord& r : rec) per[(size_t)r.k4 >> 1].push_back(r);
    for (size_t q = 0; q < due.size(); q++) {
        MaviSystem::InvCfg& c = s->inv[due[q]];
        std::vector<InvRecord>& v = per[q];
        for (InvRecord& r : v) r.k4 &= 1;
        sort_records(v);
        if (c.cols > 0) c.list.clear();   // check_invasions!(system, ::Chunks) empties the list first
        const int32_t nmax = s->reps_h[due[q]].nmax;
        for (const InvRecord& r : v) {
            MaviInvasion m{};
            m.invasor = r.invasor + 1;
            m.invaded = r.invaded + 1;
            m.p_id = r.invasor * nmax + r.pi + 1;
            c.list.push_back(m);
        }
        c.last_check = s->num_steps[due[q]];
    }
    return MAVI_OK;
}

}  // namespace mavi

using namespace mavi;

extern "C" {

int mavi_rings_invasions_config(MaviSystem* s, int32_t replica, int32_t enable, int64_t steps_to_update,
                                int32_t num_cols, int32_t num_rows) {
    if (!s || replica < 0 || replica >= s->R) return MAVI_ERR_INVALID_ARG;
    if (!s->is_rings) return fail(s, MAVI_ERR_UNSUPPORTED, "invasion detection belongs to the rings model");
    if (num_cols < 0 || num_rows < 0 || (num_cols == 0) != (num_rows == 0))
        return fail(s, MAVI_ERR_INVALID_ARG, "ring chunks need num_cols >= 1 and num_rows >= 1 (or both 0: none)");
    if ((int64_t)num_cols * num_rows > (1 << 24))
        return fail(s, MAVI_ERR_INVALID_ARG, "%d x %d ring chunks exceed the 2^24 limit", num_cols, num_rows);
    if (s->inv.empty()) s->inv.resize(s->R);
    MaviSystem::InvCfg& c = s->inv[replica];
    const MaviReplicaParams& p = s->params[replica];
    std::vector<int32_t> nbr;
    if (enable && num_cols > 0) {
        // Chunks over the space's bounding box with the main wall's neighbour
        // lists (src/rings/rings.jl:189-204)
        if (!ring_chunk_neighbors(num_rows, num_cols, p.spaces[0].wall == MAVI_WALL_PERIODIC, nbr))
            return fail(s, MAVI_ERR_UNSUPPORTED, "an open ring-chunk grid of one column and %d rows indexes column 0",
                        num_rows);
    }
    c.on = enable != 0;
    c.steps = steps_to_update;
    c.cols = enable ? num_cols : 0;
    c.rows = enable ? num_rows : 0;
    c.list.clear();
    if (enable && num_cols > 0) {
        // get_bounding_box of the space (the particle grid's box too)
        const DevRep& R = s->reps_h[replica];
        c.len = R.bb_len; c.h = R.bb_h; c.blx = R.bb_blx; c.bly = R.bb_bly;
        c.cl = c.len / num_cols;
        c.ch = c.h / num_rows;
    }
    // (re)lay the shared arrays: ring chunks of every configured replica
    MaviSystem::InvBuffers& b = s->invb;
    int64_t nch = 0;
    std::vector<int32_t> all_nbr;
    for (int r = 0; r < s->R; r++) {
        MaviSystem::InvCfg& q = s->inv[r];
        q.chunk0 = nch;
        if (!q.on || q.cols == 0) continue;
        std::vector<int32_t> t;
        ring_chunk_neighbors(q.rows, q.cols, s->params[r].spaces[0].wall == MAVI_WALL_PERIODIC, t);
        all_nbr.insert(all_nbr.end(), t.begin(), t.end());
        nch += (int64_t)q.rows * q.cols;
    }
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    free_dev(s, b.count); free_dev(s, b.start); free_dev(s, b.nbr);
    b.count = b.start = b.nbr = nullptr;
    b.nch = nch;
    if (nch > 0) {
        if (dalloc(s, &b.count, nch) != cudaSuccess || dalloc(s, &b.start, nch) != cudaSuccess ||
            dalloc(s, &b.nbr, 4 * nch) != cudaSuccess)
            return fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for %lld ring chunks", (long long)nch);
        CUDA_TRY(s, cudaMemcpyAsync(b.nbr, all_nbr.data(), sizeof(int32_t) * all_nbr.size(), cudaMemcpyHostToDevice,
                                    s->stream));
    }
    if (!b.cont) {
        if (dalloc(s, &b.cont, s->Nslots) != cudaSuccess || dalloc(s, &b.bb, 4 * s->total_rings) != cudaSuccess ||
            dalloc(s, &b.chunk_of, s->total_rings) != cudaSuccess || dalloc(s, &b.rank, s->total_rings) != cudaSuccess ||
            dalloc(s, &b.list, s->total_rings) != cudaSuccess || dalloc(s, &b.num_ids, s->R) != cudaSuccess ||
            dalloc(s, reinterpret_cast<InvRepD**>(&b.reps), s->R) != cudaSuccess ||
            dalloc(s, &b.nrec, 1) != cudaSuccess)
            return fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for the invasion buffers");
        b.rec_cap = std::max<int64_t>(1024, s->total_rings);
        if (dalloc(s, reinterpret_cast<InvRecord**>(&b.rec), b.rec_cap) != cudaSuccess)
            return fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for the invasion records");
    }
    // the step's k_sources keeps RingsInfo.cms for the check
    s->reps_h[replica].inv_cms = c.on ? 1 : 0;
    CUDA_TRY(s, cudaMemcpyAsync(const_cast<DevRep*>(s->C.reps), s->reps_h.data(), sizeof(DevRep) * s->R,
                                cudaMemcpyHostToDevice, s->stream));
    // RingsSystem(): last_check = num_steps, then update_invasions!
    c.last_check = s->num_steps[replica];
    if (c.on && s->num_steps[replica] - c.last_check >= c.steps) {
        std::vector<int32_t> due{replica};
        int rc = run_invasions(s, due, false);
        if (rc) return rc;
    }
    return device_error_status(s);
}

int mavi_rings_invasions(MaviSystem* s, int32_t replica, MaviInvasion* out, int64_t capacity, int64_t* count,
                         int64_t* last_check) {
    if (!s || replica < 0 || replica >= s->R || capacity < 0 || (capacity > 0 && !out)) return MAVI_ERR_INVALID_ARG;
    int rc = device_error_status(s);   // steps still in flight may hold a check
    if (rc) return rc;
    if (s->inv.empty()) {
        if (count) *count = 0;
        if (last_check) *last_check = 0;
        return MAVI_OK;
    }
    const MaviSystem::InvCfg& c = s->inv[replica];
    const int64_t n = (int64_t)c.list.size();
    for (int64_t k = 0; k < std::min(n, capacity); k++) out[k] = c.list[k];
    if (count) *count = n;
    if (last_check) *last_check = c.last_check;
    return MAVI_OK;
}

}  // extern "C"
