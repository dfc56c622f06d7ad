// Influence-zone kernel: one warp per query.
//
// Follows the influence-zone filter of rknn-inf (rknn-inf/inf.cpp:201-585)
// over the engine's uniform facility grid instead of an R*-tree:
//   * best-first search from the query facility q; grid cells play the role
//     of R*-tree leaf nodes (their MBR is the tight box of their facilities)
//     and are pushed lazily, ring by ring, before any entry whose key could
//     follow them;
//   * the same three pruning rules for points and cells (inf.cpp:262-354,
//     460-552): > 2 x furthest zone vertex -> prune; < 2 x nearest bisector ->
//     keep; otherwise the vertex test over vertices with count k-1 and the
//     eight extreme boundary vertices;
//   * an accepted facility adds its perpendicular bisector (inf.h:150-192),
//     bumps the counts of the vertices on its invalid side, adds its
//     intersections with the space boundary and with every earlier bisector
//     (deduplicated at 1e-9, inf.cpp:366-428), and drops vertices whose count
//     reaches k.
// Every decision is taken on the double-precision values the reference
// computes (no contraction: this file is built with -fmad=false).  A
// float32 evaluation with a proven error bound settles each decision first;
// only the undecided ones run in FP64.  Bisector-bisector intersections whose
// float32 interval is certified to lie on the invalid side of at least k
// bisectors are discarded before the FP64 division: the reference creates and
// then erases them in the same step.
//
// Epilogue: the bisectors become exact half-planes relative to q for the
// verification kernel, and a ring scan over the user grid keeps every cell
// that is not certified to lie on the strict far side of >= k bisectors.  The
// region with fewer than k violated half-planes is star-shaped around q (each
// half-plane's invalid side is convex and excludes q), so a full ring of
// pruned cells closes it; users outside the kept cells cannot be results.
#include "rknn_common.cuh"
#include "zone.cuh"
#include "zone_geom.cuh"
#include <cfloat>

namespace rknn {



// ============================================================================
// Lanes hand zone state to each other through shared memory between warp
// barriers.
#define WSYNC() __syncwarp()

__device__ __forceinline__ void zone_body(const ZoneArgs& A)
{
    pdl_trigger();
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
#ifdef RKNN_CHECKED
    if (threadIdx.x == 0 && blockIdx.x == 0) g_fault = A.fault;
    __syncthreads();
    if (!g_fault) g_fault = A.fault;
#endif
    const ZoneLayout LY = zone_layout(A.caps);
    // every state pointer derives from the __shared__ array itself
    Slice S = carve(smem + (size_t)wib * LY.bytes, A.caps);
    const int VC = A.caps.vc, LC = A.caps.lc, PC = A.caps.pc;
    const long long NCF = (long long)A.gf.gx * A.gf.gy, NCU = (long long)A.gu.gx * A.gu.gy;
    (void)NCF; (void)NCU;     // bounds of the checked build's index checks
    const double sx0 = A.sx0, sy0 = A.sy0, sx1 = A.sx1, sy1 = A.sy1;
    // largest rounding error of a vertex coordinate stored as float
    const float E = kU32 * (float)fmax(fmax(fabs(sx0), fabs(sx1)), fmax(fabs(sy0), fabs(sy1))) * 1.01f + 1e-37f;
    const float fsx0 = __double2float_rd(sx0), fsy0 = __double2float_rd(sy0);
    const float fsx1 = __double2float_ru(sx1), fsy1 = __double2float_ru(sy1);
    const double slack = 1e-5 * ((double)A.gf.cs + fmax(fmax(fabs(sx0), fabs(sx1)), fmax(fabs(sy0), fabs(sy1))));
    // coordinates within EPS in double are within EPS + 2E as floats
    const float tolE = (1e-9f + 2.0f * E) * (1.0f + 0x1p-20f);

    for (;;) {
        int slot = 0;
        if (lane == 0) slot = atomicAdd(A.work_counter, 1);
        slot = __shfl_sync(FULL, slot, 0);
        if (slot >= A.nq) break;
        const int s = A.order ? A.order[slot] : slot;
        const int qin = A.q_in[s];
        const int k = A.k_in[s];
        QDesc* qd = A.qd + s;
        ZStats zs = {};
        int qflags = 0;
        if (qin < 0 || qin >= A.nf || k <= 0) {
            if (lane == 0) {
                QDesc d = {};
                d.qpos = -1;
                d.k = k;
                d.flags = QF_BAD_QUERY;
                *qd = d;
                A.zst[s] = zs;
                A.segs[(size_t)s * A.seg_cap] = make_int2(0, 0);
            }
            continue;
        }
        const int qpos = A.fpos[GX(qin, A.nf, 105)];
        const float2 qf = A.fxy[GX(qpos, A.nf, 101)];
        const double qx = qf.x, qy = qf.y;
        const uint32_t ku = (uint32_t)k;
        // Warp-uniform scalars live in registers (identical in every lane);
        // lane 0 alone touches the heap and broadcasts what it changes.
        int nV = 4, nL = 0, nP = 0, nCons = -1, flags = 0;
        double far_ = 0.0, nearb = DBL_MAX;

        // ---- init: four space corners (inf.cpp:211-226) -------------------
        double d2c = 0.0;
        if (lane < 4) {
            const double x = (lane & 1) ? sx1 : sx0;
            const double y = (lane & 2) ? sy1 : sy0;
            d2c = d2_64(x, y, qx, qy);
            IX(S.vd, lane) = make_double2(x, y);
            IX(S.v4, lane) = make_float4((float)x, (float)y, (float)d2c,
                                         vpack(0, VB_BND | edge_bits(x, y, sx0, sy0, sx1, sy1)));
        }
        WSYNC();
        far_ = __dsqrt_rn(warp_max(d2c));
        // integer thresholds of rules 1 and 2 on the queue keys
        Cut K1 = sqrt_cut(2.0 * far_, false);
        Cut K2 = sqrt_cut(2.0 * DBL_MAX, true);  // nearest bisector: none yet (threshold +inf)

        long long tph = clock64();
#define PHASE(i) do { long long t_ = clock64(); zs.cyc[i] += t_ - tph; tph = t_; } while (0)
        const int qcx = cell_coord(qf.x, A.gf.x0, A.gf.inv, A.gf.gx);
        const int qcy = cell_coord(qf.y, A.gf.y0, A.gf.inv, A.gf.gy);
        const int rmaxf = max(max(qcx, A.gf.gx - 1 - qcx), max(qcy, A.gf.gy - 1 - qcy));
        int ring = 0;        // next facility ring to expand
        bool ring_open;
        uint64_t ring_key;
        ring_gate(ring, rmaxf, (double)A.gf.cs, slack, far_, ring_open, ring_key);

        // ---- best-first search --------------------------------------------
        for (;;) {
            // make the top poppable: expand rings whose cells could precede it
            for (;;) {
                if (!ring_open) break;
                if (nP > 0) {
                    uint64_t top = 0;
                    if (lane == 0) top = IX(S.pqk, 0);
                    top = __shfl_sync(FULL, top, 0);
                    if (top < ring_key) break;
                }
                // expand ring `ring`: 8*ring cells (1 for ring 0)
                const int ncell = ring == 0 ? 1 : 8 * ring;
                for (int t0 = 0; t0 < ncell; t0 += 32) {
                    const int t = t0 + lane;
                    int cxx = 0, cyy = 0;
                    bool ok = t < ncell;
                    if (ok) {
                        if (ring == 0) { cxx = qcx; cyy = qcy; }
                        else {
                            const int side = 2 * ring + 1;
                            if (t < side) { cxx = qcx - ring + t; cyy = qcy - ring; }
                            else if (t < 2 * side) { cxx = qcx - ring + (t - side); cyy = qcy + ring; }
                            else if (t < 2 * side + (2 * ring - 1)) { cxx = qcx - ring; cyy = qcy - ring + 1 + (t - 2 * side); }
                            else { cxx = qcx + ring; cyy = qcy - ring + 1 + (t - 2 * side - (2 * ring - 1)); }
                        }
                        ok = cxx >= 0 && cxx < A.gf.gx && cyy >= 0 && cyy < A.gf.gy;
                    }
                    int cid = 0;
                    if (ok) {
                        cid = cyy * A.gf.gx + cxx;
                        ok = A.fstart[GX(cid + 1, NCF + 1, 102)] > A.fstart[GX(cid, NCF + 1, 102)];
                    }
                    const double key = ok ? rect_d2_64(qx, qy, A.fmbr[GX(cid, NCF, 103)]) : 0.0;
                    const unsigned m = __ballot_sync(FULL, ok);
                    const int rank = __popc(m & ((1u << lane) - 1));
                    if (ok) { IX(S.tk, rank) = (uint64_t)__double_as_longlong(key); IX(S.tc, rank) = (uint32_t)cid; }
                    WSYNC();
                    if (lane == 0) {
                        for (int i = 0; i < __popc(m); ++i)
                            if (!pq_push(S.pqk.p, S.pqc.p, nP, PC, IX(S.tk, i), IX(S.tc, i))) { flags |= QF_ZONE_PQ_OVERFLOW; break; }
                    }
                    nP = __shfl_sync(FULL, nP, 0);
                    flags = __shfl_sync(FULL, flags, 0);
                    WSYNC();
                }
                ring++;
                ring_gate(ring, rmaxf, (double)A.gf.cs, slack, far_, ring_open, ring_key);
                if (flags) break;
            }
            PHASE(0);
            if (flags || nP == 0) break;
            uint64_t keybits = 0;
            uint32_t code = 0;
            if (lane == 0) {
                keybits = IX(S.pqk, 0);
                code = IX(S.pqc, 0);
                pq_pop(S.pqk.p, S.pqc.p, nP);
            }
            keybits = __shfl_sync(FULL, keybits, 0);
            code = __shfl_sync(FULL, code, 0);
            nP = __shfl_sync(FULL, nP, 0);
            const double key = __longlong_as_double((long long)keybits);

            const bool is_point = (code & KIND_POINT) != 0;
            const int id = (int)(code & ~KIND_POINT);
            double px = 0, py = 0;
            float4 mbr = make_float4(0, 0, 0, 0);
            if (is_point) {
                if (id == qpos) continue;
                const float2 pf = A.fxy[GX(id, A.nf, 101)];
                px = pf.x; py = pf.y;
                if (A.skip_coincident && pf.x == qf.x && pf.y == qf.y) continue;
                zs.pts++;
            } else {
                mbr = A.fmbr[GX(id, NCF, 103)];
                zs.cells++;
            }
            // rules 1 and 2 (inf.cpp:262-267, 460-465): key is the squared distance
            bool prune;
            PHASE(1);
            // Rule 1 prunes this entry.  Every entry still queued has a key
            // >= this one, and every cell not yet expanded lies beyond the
            // heap's top (the expansion loop above guarantees it), so rule 1
            // prunes all of them as well and the zone is final: stop here
            // instead of draining the queue.
            bool r1;
            if (keybits >= K1.hi) r1 = true;
            else if (keybits <= K1.lo) r1 = false;
            else r1 = sqrt_rn64(key) > 2.0 * far_;
            if (r1) break;
            // rule 2: keep when nearer than twice the nearest bisector
            bool r2;
            if (keybits >= K2.hi) r2 = false;
            else if (keybits <= K2.lo) r2 = true;
            else r2 = sqrt_rn64(key) < 2.0 * nearb;
            if (r2) prune = false;
            else {
                // ---- vertex test (inf.cpp:268-353, 466-551) -------------
                if (nCons < 0) {
                    // One pass in vertex order: vertices with count k-1 are
                    // considered; boundary vertices with count < k are listed.
                    int nC = 0, nB = 0;
                    for (int i0 = 0; i0 < nV; i0 += 32) {
                        const int i = i0 + lane;
                        uint32_t cnt = 0, fl = 0;
                        const bool in = i < nV;
                        if (in) {
                            const float w = IX(S.v4, i).w;
                            cnt = vcnt_of(w);
                            fl = vfl_of(w);
                        }
                        // the zone-boundary test (vertex_test 1) also considers
                        // every space-boundary vertex below count k
                        const bool c = in && (cnt == ku - 1 || (A.vertex_test && (fl & VB_BND) && cnt < ku));
                        const bool b = in && !A.vertex_test && (fl & VB_BND) && cnt < ku;
                        const unsigned mc = __ballot_sync(FULL, c), mb = __ballot_sync(FULL, b);
                        const unsigned below = (1u << lane) - 1;
                        if (c) IX(S.cons, nC + __popc(mc & below)) = (uint16_t)i;
                        if (b) IX(S.blist, nB + __popc(mb & below)) = (uint16_t)i;
                        nC += __popc(mc);
                        nB += __popc(mb);
                    }
                    WSYNC();
                    // Extreme boundary points (inf.cpp:283-321): lane j < 8 keeps
                    // extreme j over the list in vertex order, the first strict
                    // min / max winning as the reference's pointer updates do:
                    // left min/max y, right min/max y, bottom min/max x, top min/max x.
                    // The list is read 32 entries at a time and broadcast.
                    int best = -1;
                    {
                        const bool byY = lane < 4;
                        const bool wantMin = (lane & 1) == 0;
                        const uint32_t ebit = lane < 2 ? VB_EL : lane < 4 ? VB_ER : lane < 6 ? VB_EB : VB_ET;
                        long long bk = 0;
                        for (int t0 = 0; t0 < nB; t0 += 32) {
                            const int t = t0 + lane;
                            int vi = 0;
                            uint32_t fl = 0;
                            long long kx = 0, ky = 0;
                            if (t < nB) {
                                vi = IX(S.blist, t);
                                fl = vfl_of(IX(S.v4, vi).w);
                                const double2 p = IX(S.vd, vi);
                                kx = order_key(p.x);
                                ky = order_key(p.y);
                            }
                            const int n = min(32, nB - t0);
                            for (int u = 0; u < n; ++u) {
                                const int ui = __shfl_sync(FULL, vi, u);
                                const uint32_t uf = __shfl_sync(FULL, fl, u);
                                const long long ukx = __shfl_sync(FULL, kx, u);
                                const long long uky = __shfl_sync(FULL, ky, u);
                                if (lane < 8 && (uf & ebit)) {
                                    const long long kk = byY ? uky : ukx;
                                    if (best < 0 || (wantMin ? kk < bk : kk > bk)) { best = ui; bk = kk; }
                                }
                            }
                        }
                    }
                    int ext[8];
                    float ex[8], ey[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        ext[j] = __shfl_sync(FULL, best, j);
                        ex[j] = 0.0f; ey[j] = 0.0f;
                        if (ext[j] >= 0) {
                            const float4 e = IX(S.v4, ext[j]);
                            ex[j] = e.x; ey[j] = e.y;
                        }
                    }
                    // boundary vertices (count < k, not already considered)
                    // within EPS of an extreme point (inf.cpp:326-346)
                    for (int t0 = 0; t0 < nB; t0 += 32) {
                        const int t = t0 + lane;
                        bool c = false;
                        int vi = 0;
                        if (t < nB) {
                            vi = IX(S.blist, t);
                            const float4 v = IX(S.v4, vi);
                            if (vcnt_of(v.w) != ku - 1) {
#pragma unroll
                                for (int j = 0; j < 8; ++j) {
                                    if (c || ext[j] < 0 || fabsf(v.x - ex[j]) > tolE || fabsf(v.y - ey[j]) > tolE) continue;
                                    const double2 a = IX(S.vd, vi), b = IX(S.vd, ext[j]);
                                    if (fabs(__dsub_rn(a.x, b.x)) < EPS && fabs(__dsub_rn(a.y, b.y)) < EPS) c = true;
                                }
                            }
                        }
                        const unsigned m = __ballot_sync(FULL, c);
                        if (c) IX(S.cons, nC + __popc(m & ((1u << lane) - 1))) = (uint16_t)vi;
                        nC += __popc(m);
                    }
                    nCons = nC;
                    WSYNC();
                }
                const int nC = nCons;
                bool hit = false;
                const float px32 = (float)px, py32 = (float)py;
                for (int t = lane; t < nC && !hit; t += 32) {
                    const int i = IX(S.cons, t);
                    const float4 v = IX(S.v4, i);
                    int r;
                    if (is_point) r = closer32(px32 - v.x, py32 - v.y, E, v.z);
                    else r = closer32(rect_dx32(v.x, mbr.x, mbr.z), rect_dx32(v.y, mbr.y, mbr.w), E, v.z);
                    if (r < 0) {
                        const double2 p = IX(S.vd, i);
                        double dx64 = 0, dy64 = 0;
                        if (is_point) {
                            dx64 = __dsub_rn(px, p.x);
                            dy64 = __dsub_rn(py, p.y);
                        } else {
                            if (p.x < (double)mbr.x) dx64 = __dsub_rn((double)mbr.x, p.x);
                            else if (p.x > (double)mbr.z) dx64 = __dsub_rn(p.x, (double)mbr.z);
                            if (p.y < (double)mbr.y) dy64 = __dsub_rn((double)mbr.y, p.y);
                            else if (p.y > (double)mbr.w) dy64 = __dsub_rn(p.y, (double)mbr.w);
                        }
                        r = closer64(dx64, dy64, p.x, p.y, qx, qy);
                    }
                    hit = r != 0;
                }
                prune = !__any_sync(FULL, hit);
                PHASE(2);
            }
            if (prune) continue;

            if (!is_point) {
                // push the cell's facilities (inf.cpp:556-565)
                const int p0 = A.fstart[GX(id, NCF + 1, 102)], p1 = A.fstart[GX(id + 1, NCF + 1, 102)];
                for (int t0 = p0; t0 < p1; t0 += 32) {
                    const int t = t0 + lane;
                    if (t < p1) {
                        const float2 pf = A.fxy[GX(t, A.nf, 101)];
                        IX(S.tk, lane) = (uint64_t)__double_as_longlong(d2_64(qx, qy, (double)pf.x, (double)pf.y));
                        IX(S.tc, lane) = KIND_POINT | (uint32_t)t;
                    }
                    WSYNC();
                    if (lane == 0) {
                        const int cnt = min(32, p1 - t0);
                        for (int i = 0; i < cnt; ++i)
                            if (!pq_push(S.pqk.p, S.pqc.p, nP, PC, IX(S.tk, i), IX(S.tc, i))) { flags |= QF_ZONE_PQ_OVERFLOW; break; }
                    }
                    nP = __shfl_sync(FULL, nP, 0);
                    flags = __shfl_sync(FULL, flags, 0);
                    WSYNC();
                }
                if (flags) break;
                continue;
            }

            // ================= accept facility `id`: add its bisector ======
            if (nL >= LC) { flags |= QF_ZONE_L_OVERFLOW; break; }
            Line64 nb = {0.0, 0.0, 0, 0};
            if (lane == 0) nb = make_bisector(qx, qy, px, py);
            nb.a = __shfl_sync(FULL, nb.a, 0);
            nb.b = __shfl_sync(FULL, nb.b, 0);
            nb.vert = __shfl_sync(FULL, nb.vert, 0);
            nb.valid = __shfl_sync(FULL, nb.valid, 0);
            const float na32 = (float)nb.a, nb32 = (float)nb.b;
            const float nab = fabsf(na32);
            zs.nb++;

            // (1) count pass over the existing vertices (inf.cpp:359-364)
            const int nV0 = nV;
            for (int i = lane; i < nV0; i += 32) {
                const float4 v = IX(S.v4, i);
                float r32, err;
                if (nb.vert) {
                    r32 = v.x - nb32;
                    err = 3.0f * kU32 * (fabsf(v.x) + fabsf(nb32)) + 1e-37f;
                } else {
                    const float t = nab * fabsf(v.x);
                    r32 = v.y - fmaf(na32, v.x, nb32);
                    err = 5.0f * kU32 * (fabsf(v.y) + t + fabsf(nb32)) + 1e-37f;
                }
                bool valid;
                if (r32 > err) valid = nb.valid == 1;
                else if (r32 < -err) valid = nb.valid == 0;
                else {
                    const double2 p = IX(S.vd, i);
                    valid = valid64(nb.a, nb.b, nb.vert, nb.valid, p.x, p.y);
                }
                // near the new line: may coincide (within 1e-9) with one of its intersections
                const float tol = (1.0f + nab) * 1.2e-9f + err;
                uint32_t fl = vfl_of(v.w) & ~VB_ON;
                if (fabsf(r32) <= tol || !(fabsf(r32) < FLT_MAX)) fl |= VB_ON;
                IX(S.v4, i).w = vpack(vcnt_of(v.w) + (valid ? 0u : 1u), fl);
            }
            WSYNC();

            PHASE(3);
            // (2) candidate intersections: boundary edges (bottom, top, left,
            //     right; inf.h:340-374) then every earlier bisector in order
            const int C = 4 + nL;
            // float interval of the new line's coefficients (directed rounding)
            const float a1l = __double2float_rd(nb.a), a1h = __double2float_ru(nb.a);
            const float b1l = __double2float_rd(nb.b), b1h = __double2float_ru(nb.b);
            for (int c = lane; c < C; c += 32) {
                double x = 0, y = 0;
                bool ok = false;
                uint8_t cf = 0;
                if (c < 4) {
                    const double ea = 0, eb = (c == 0) ? sy0 : (c == 1) ? sy1 : (c == 2) ? sx0 : sx1;
                    const int ev = c >= 2;
                    if (intersect64(nb.a, nb.b, nb.vert, ea, eb, ev, x, y)) {
                        ok = (c < 2) ? (x >= sx0 && x <= sx1) : (y >= sy0 && y <= sy1);
                    }
                    cf = VB_BND;
                    zs.cand += ok;
                } else {
                    const int j = c - 4;
                    const double2 e = IX(S.ld, j);
                    const float4 e4 = IX(S.l4, j);
                    const int ev = (__float_as_uint(e4.w) & LB_VERT) ? 1 : 0;
                    bool need64 = true;
                    if (!nb.vert && !ev) {
                        // float interval of the intersection (directed rounding)
                        const float a2l = lo32(e4.x), a2h = hi32(e4.x);
                        const float b2l = lo32(e4.y), b2h = hi32(e4.y);
                        const float dl = __fsub_rd(a1l, a2h), dh = __fsub_ru(a1h, a2l);
                        const float nl = __fsub_rd(b2l, b1h), nh = __fsub_ru(b2h, b1l);
                        if ((dl > 4e-9f || dh < -4e-9f) && fabsf(nl) < FLT_MAX && fabsf(nh) < FLT_MAX &&
                            fabsf(dl) < FLT_MAX && fabsf(dh) < FLT_MAX) {
                            // x = N / D, N in [nl, nh], D in [dl, dh] not containing 0
                            float xl, xh;
                            if (dl > 0.0f) {
                                xl = __fdiv_rd(nl, nl >= 0.0f ? dh : dl);
                                xh = __fdiv_ru(nh, nh >= 0.0f ? dl : dh);
                            } else {
                                const float pl = -dh, ph = -dl;      // |D| in [pl, ph]
                                xl = -__fdiv_ru(nh, nh >= 0.0f ? pl : ph);
                                xh = -__fdiv_rd(nl, nl >= 0.0f ? ph : pl);
                            }
                            // y = a1 x + b1 over the box
                            const float m1 = __fmul_rd(a1l, xl), m2 = __fmul_rd(a1l, xh), m3 = __fmul_rd(a1h, xl), m4 = __fmul_rd(a1h, xh);
                            const float n1 = __fmul_ru(a1l, xl), n2 = __fmul_ru(a1l, xh), n3 = __fmul_ru(a1h, xl), n4 = __fmul_ru(a1h, xh);
                            float yl = __fadd_rd(fminf(fminf(m1, m2), fminf(m3, m4)), b1l);
                            float yh = __fadd_ru(fmaxf(fmaxf(n1, n2), fmaxf(n3, n4)), b1h);
                            // pad for the FP64 rounding of the reference's evaluation
                            const float px_ = 1e-12f * fmaxf(fabsf(xl), fabsf(xh)) + 1e-37f;
                            const float py_ = 1e-12f * (fmaxf(fabsf(yl), fabsf(yh)) + fabsf(a1h) * fmaxf(fabsf(xl), fabsf(xh)) + fabsf(b1h)) + 1e-37f;
                            xl = __fsub_rd(xl, px_); xh = __fadd_ru(xh, px_);
                            yl = __fsub_rd(yl, py_); yh = __fadd_ru(yh, py_);
                            if (xl <= xh && yl <= yh && fabsf(xl) < FLT_MAX && fabsf(xh) < FLT_MAX &&
                                fabsf(yl) < FLT_MAX && fabsf(yh) < FLT_MAX) {
                                if (xh < fsx0 || xl > fsx1 || yh < fsy0 || yl > fsy1) need64 = false;  // outside
                                else {
                                    // certified violations of earlier bisectors, four
                                    // bisectors per step (overshooting k is harmless)
                                    const float xc = 0.5f * xl + 0.5f * xh, yc = 0.5f * yl + 0.5f * yh;
                                    const float rx = (0.5f * xh - 0.5f * xl) * (1.0f + 4.0f * kU32) + fabsf(xc) * 2.0f * kU32 + 1e-37f;
                                    const float ry = (0.5f * yh - 0.5f * yl) * (1.0f + 4.0f * kU32) + fabsf(yc) * 2.0f * kU32 + 1e-37f;
                                    const float KX = rx * (1.0f + kU32) + 3.01f * kU32 * fabsf(xc);
                                    const float KY = ry + 3.01f * kU32 * fabsf(yc) + 1e-37f;
                                    int cert = 0;
                                    int m = 0;
                                    for (; m + 4 <= nL && cert < k; m += 4) {
                                        const float4 q0 = IX(S.l4, m), q1 = IX(S.l4, m + 1);
                                        const float4 q2 = IX(S.l4, m + 2), q3 = IX(S.l4, m + 3);
                                        cert += inval32(q0, xc, yc, KX, KY) + inval32(q1, xc, yc, KX, KY) +
                                                inval32(q2, xc, yc, KX, KY) + inval32(q3, xc, yc, KX, KY);
                                    }
                                    for (; m < nL && cert < k; ++m) cert += inval32(IX(S.l4, m), xc, yc, KX, KY);
                                    if (cert >= k) need64 = false;
                                }
                            }
                        }
                    }
                    if (need64) {
                        zs.cand64++;
                        if (intersect64(nb.a, nb.b, nb.vert, e.x, e.y, ev, x, y))
                            ok = x >= sx0 && x <= sx1 && y >= sy0 && y <= sy1;
                    }
                    zs.cand++;
                }
                IX(S.cd, c) = make_double2(x, y);
                IX(S.c2, c) = make_float2((float)x, (float)y);
                IX(S.cfl, c) = ok ? (uint8_t)(cf | 0x80) : (uint8_t)0;
            }
            WSYNC();

            PHASE(4);
            // (3) deduplicate (|dx| < 1e-9 and |dy| < 1e-9) against existing
            //     vertices near the new line and against earlier candidates
            {
                // online vertices
                int nOn = 0;
                for (int i0 = 0; i0 < nV0; i0 += 32) {
                    const int i = i0 + lane;
                    const bool on = i < nV0 && (vfl_of(IX(S.v4, i).w) & VB_ON);
                    const unsigned m = __ballot_sync(FULL, on);
                    if (on) IX(S.cons, nOn + __popc(m & ((1u << lane) - 1))) = (uint16_t)i;   // cons reused as scratch
                    nOn += __popc(m);
                }
                WSYNC();
                nCons = -1;   // considered list must be rebuilt
                if (nOn > 0) {
                    for (int c = lane; c < C; c += 32) {
                        if (!(IX(S.cfl, c) & 0x80)) continue;
                        const float2 c32 = IX(S.c2, c);
                        bool dup = false;
                        for (int t = 0; t < nOn && !dup; ++t) {
                            const int i = IX(S.cons, t);
                            const float4 v = IX(S.v4, i);
                            if (fabsf(v.x - c32.x) > tolE || fabsf(v.y - c32.y) > tolE) continue;
                            const double2 p = IX(S.vd, i), q = IX(S.cd, c);
                            if (fabs(__dsub_rn(p.x, q.x)) < EPS && fabs(__dsub_rn(p.y, q.y)) < EPS) dup = true;
                        }
                        if (dup) IX(S.cfl, c) &= 0x7f;
                    }
                }
                WSYNC();
            }

            PHASE(5);
            // (4) counts of the surviving candidates over earlier bisectors:
            //     a float pass counts certain violations (and stops at k, which
            //     erases the candidate anyway); bisectors it cannot decide are
            //     evaluated in FP64 in a second pass
            for (int c = lane; c < C; c += 32) {
                int cnt = k;
                if (IX(S.cfl, c) & 0x80) {
                    const double2 p = IX(S.cd, c);
                    const float2 c32 = IX(S.c2, c);
                    const float KX = kU32 * fabsf(c32.x) * (1.0f + kU32) + 3.01f * kU32 * fabsf(c32.x);
                    const float KY = kU32 * fabsf(c32.y) + 3.01f * kU32 * fabsf(c32.y) + 1e-37f;
                    cnt = 0;
                    // the bisector that generated this candidate passes through
                    // it: its side is a rounding question, decided in FP64
                    const int gen = c - 4;
                    if (gen >= 0) {
                        const double2 g = IX(S.ld, gen);
                        const uint32_t lf = __float_as_uint(IX(S.l4, gen).w);
                        cnt += !valid64(g.x, g.y, lf & LB_VERT, (lf & LB_VALID) ? 1 : 0, p.x, p.y);
                    }
                    int undec = 0;
                    int m = 0;
                    for (; m + 4 <= nL && cnt < k; m += 4) {
                        const float4 q0 = IX(S.l4, m), q1 = IX(S.l4, m + 1);
                        const float4 q2 = IX(S.l4, m + 2), q3 = IX(S.l4, m + 3);
                        const int s0 = (m == gen) ? -1 : side32(q0, c32.x, c32.y, KX, KY);
                        const int s1 = (m + 1 == gen) ? -1 : side32(q1, c32.x, c32.y, KX, KY);
                        const int s2 = (m + 2 == gen) ? -1 : side32(q2, c32.x, c32.y, KX, KY);
                        const int s3 = (m + 3 == gen) ? -1 : side32(q3, c32.x, c32.y, KX, KY);
                        cnt += (s0 > 0) + (s1 > 0) + (s2 > 0) + (s3 > 0);
                        undec += (s0 == 0) + (s1 == 0) + (s2 == 0) + (s3 == 0);
                    }
                    for (; m < nL && cnt < k; ++m) {
                        const int sm = (m == gen) ? -1 : side32(IX(S.l4, m), c32.x, c32.y, KX, KY);
                        cnt += sm > 0;
                        undec += sm == 0;
                    }
                    if (cnt < k && undec > 0) {
                        for (int j = 0; j < nL && cnt < k; ++j) {
                            if (j == gen) continue;
                            const float4 q = IX(S.l4, j);
                            if (side32(q, c32.x, c32.y, KX, KY) != 0) continue;
                            const double2 g = IX(S.ld, j);
                            const uint32_t lf = __float_as_uint(q.w);
                            cnt += !valid64(g.x, g.y, lf & LB_VERT, (lf & LB_VALID) ? 1 : 0, p.x, p.y);
                        }
                    }
                }
                IX(S.ccnt, c) = cnt;
            }
            WSYNC();
            // (4b) a candidate closer than 1e-9 to an earlier one is not added
            // (the reference keeps the first).  Only a kept candidate can change
            // the vertex set, so the float prefilter runs for those; any hit
            // triggers the exact sequential resolution over all candidates.
            {
                bool anyclose = false;
                for (int c = lane; c < C; c += 32) {
                    if (!(IX(S.cfl, c) & 0x80) || IX(S.ccnt, c) >= k) continue;
                    // doubles within 1e-9 give floats within 1e-9 + u(|x1|+|x2|)
                    const float2 c32 = IX(S.c2, c);
                    const float tx = 3.0f * kU32 * fabsf(c32.x) + 2e-9f, ty = 3.0f * kU32 * fabsf(c32.y) + 2e-9f;
                    for (int c2 = 0; c2 < c; ++c2) {
                        if (!(IX(S.cfl, c2) & 0x80)) continue;
                        const float2 o = IX(S.c2, c2);
                        if (fabsf(o.x - c32.x) <= tx && fabsf(o.y - c32.y) <= ty) { anyclose = true; break; }
                    }
                }
                if (__any_sync(FULL, anyclose)) {
                    if (lane == 0) {
                        for (int c = 0; c < C; ++c) {
                            if (!(IX(S.cfl, c) & 0x80)) continue;
                            const double2 p = IX(S.cd, c);
                            for (int c2 = 0; c2 < c; ++c2) {
                                if (!(IX(S.cfl, c2) & 0x80)) continue;
                                const double2 o = IX(S.cd, c2);
                                if (fabs(__dsub_rn(o.x, p.x)) < EPS && fabs(__dsub_rn(o.y, p.y)) < EPS) { IX(S.cfl, c) &= 0x7f; break; }
                            }
                        }
                    }
                    WSYNC();
                }
            }

            // (5) erase old vertices with count >= k (order kept), then append
            //     the new vertices with count < k in candidate order
            int w = 0;
            for (int i0 = 0; i0 < nV0; i0 += 32) {
                const int i = i0 + lane;
                bool keep = false;
                float4 v = make_float4(0, 0, 0, 0);
                double2 p = make_double2(0, 0);
                if (i < nV0) {
                    v = IX(S.v4, i);
                    keep = vcnt_of(v.w) < ku;
                    if (keep) p = IX(S.vd, i);
                }
                const unsigned m = __ballot_sync(FULL, keep);
                WSYNC();
                if (keep) {
                    const int o = w + __popc(m & ((1u << lane) - 1));
                    v.w = vpack(vcnt_of(v.w), vfl_of(v.w) & ~VB_ON);
                    IX(S.vd, o) = p;
                    IX(S.v4, o) = v;
                }
                w += __popc(m);
                WSYNC();
            }
            int nnew = 0;
            for (int c0 = 0; c0 < C; c0 += 32) {
                const int c = c0 + lane;
                const bool keep = c < C && (IX(S.cfl, c) & 0x80) && IX(S.ccnt, c) < k;
                const unsigned m = __ballot_sync(FULL, keep);
                const int o = w + nnew + __popc(m & ((1u << lane) - 1));
                if (keep && o < VC) {
                    const double2 p = IX(S.cd, c);
                    const float2 c32 = IX(S.c2, c);
                    IX(S.vd, o) = p;
                    IX(S.v4, o) = make_float4(c32.x, c32.y, (float)d2_64(p.x, p.y, qx, qy),
                                              vpack((uint32_t)IX(S.ccnt, c),
                                                    (IX(S.cfl, c) & VB_BND) | edge_bits(p.x, p.y, sx0, sy0, sx1, sy1)));
                }
                nnew += __popc(m);
            }
            zs.kept += nnew;
            nV = w + nnew;
            const bool vover = nV > VC;
            if (vover) nV = VC;

            // (6) nearest bisector distance, store the line (inf.cpp:430-434).
            //     A float estimate with an error bound skips the FP64
            //     evaluation when the new line is certainly not nearer.
            {
                double dl = nearb;
                if (lane == 0) {
                    bool need = true;
                    if (nearb < DBL_MAX) {
                        float est, err;
                        if (nb.vert) {
                            est = fabsf(qf.x - nb32);
                            err = 4.0f * kU32 * (fabsf(qf.x) + fabsf(nb32)) + 1e-30f;
                        } else {
                            const float den = sqrtf(fmaf(na32, na32, 1.0f));
                            est = fabsf(fmaf(na32, qf.x, nb32 - qf.y)) / den;
                            err = 8.0f * kU32 * ((fabsf(na32 * qf.x) + fabsf(qf.y) + fabsf(nb32)) / den + est) + 1e-30f;
                        }
                        if ((double)__fsub_rd(est, err) > nearb) need = false;   // NaN keeps need
                    }
                    if (need) {
                        const double d = line_dist64(qx, qy, nb.a, nb.b, nb.vert);
                        if (d < nearb) dl = d;
                    }
                }
                dl = __shfl_sync(FULL, dl, 0);
                if (dl != nearb) {
                    nearb = dl;
                    K2 = sqrt_cut(2.0 * nearb, true);
                }
            }
            if (lane == 0) {
                const uint32_t lf = (nb.vert ? LB_VERT : 0) | (nb.valid ? LB_VALID : 0);
                IX(S.ld, nL) = make_double2(nb.a, nb.b);
                IX(S.l4, nL) = make_float4(na32, nb32, 3.01f * kU32 * fabsf(nb32) + 1e-37f, __uint_as_float(lf));
                IX(S.lpos, nL) = id;
            }
            nL += 1;
            if (vover) flags |= QF_ZONE_V_OVERFLOW;
            if (nV > zs.vmax) zs.vmax = nV;
            WSYNC();
            // (7) furthest remaining vertex (inf.cpp:445-451).  The float
            //     squared distances are the FP64 ones rounded to nearest, a
            //     monotone map: the FP64 maximum is among the vertices whose
            //     float value is the float maximum.
            {
                float m32 = 0.0f;
                for (int i = lane; i < nV; i += 32) m32 = fmaxf(m32, IX(S.v4, i).z);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) m32 = fmaxf(m32, __shfl_xor_sync(FULL, m32, o));
                long long m = 0;
                for (int i = lane; i < nV; i += 32)
                    if (IX(S.v4, i).z == m32) {
                        const double2 p = IX(S.vd, i);
                        m = max(m, __double_as_longlong(d2_64(p.x, p.y, qx, qy)));
                    }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(FULL, m, o));
                const double f = sqrt_rn64(__longlong_as_double(m));
                if (f != far_) {
                    far_ = f;
                    K1 = sqrt_cut(2.0 * far_, false);
                    ring_gate(ring, rmaxf, (double)A.gf.cs, slack, far_, ring_open, ring_key);
                }
            }
            WSYNC();
            PHASE(6);
            if (flags) break;
        }
        WSYNC();
        qflags |= flags;
        zs.nb = nL;
        zs.cand = warp_sum(zs.cand);
        zs.cand64 = warp_sum(zs.cand64);

        // ---- epilogue 1: exact half-planes relative to q -------------------
        // m(u) = a (ux - qx) + b (uy - qy) + c = d2(u,f) - d2(u,q);  f strictly
        // nearer than q  <=>  m < 0.
        float4* planes = A.planes + (size_t)s * A.pstride;
        double cmax = 0.0;
        for (int m = lane; m < nL; m += 32) {
            int pos = IX(S.lpos, m);
            float2 f = A.fxy[GX(pos, A.nf, 101)];
            double dx = (double)f.x - qx, dy = (double)f.y - qy;
            double c = dx * dx + dy * dy;
            float4 p = make_float4((float)(-2.0 * dx), (float)(-2.0 * dy), (float)c, 0.0f);
            planes[GX(m, A.pstride, 106)] = p;
            IX(S.splanes, m) = p;
            A.bis_pos[(size_t)s * A.pstride + GX(m, A.pstride, 107)] = pos;
            cmax = fmax(cmax, c);
        }
        cmax = warp_max(cmax);
        const double Fp = sqrt(cmax) * (1.0 + 1e-6) + 1e-30;
        // per-user bound 8u (2F'(|x'|+|y'|) + F'^2)
        const float k2f = (float)(8.0 * (double)kU32 * 2.0 * Fp * (1.0 + 1e-6));
        const float kf2 = (float)(8.0 * (double)kU32 * Fp * Fp * (1.0 + 1e-6)) + 1e-30f;
        const double k2f64 = 8.0 * kU64 * 2.0 * Fp * (1.0 + 1e-6);
        const double kf264 = 8.0 * kU64 * Fp * Fp * (1.0 + 1e-6) + 1e-300;
        WSYNC();

        // ---- epilogue 2: ring scan over user cells ------------------------
        const Grid gu = A.gu;
        const int ucx = cell_coord(qf.x, gu.x0, gu.inv, gu.gx);
        const int ucy = cell_coord(qf.y, gu.y0, gu.inv, gu.gy);
        const int RM = A.rmax;
        const int W = 2 * RM + 1;
        const int nwords = (W * W + 31) / 32;
        for (int i = lane; i < nwords; i += 32) IX(S.bitmap, i) = 0u;
        WSYNC();
        const float delta = 8.0f * kU32 * (fabsf(gu.x0) + fabsf(gu.y0) + gu.cs * (float)max(gu.gx, gu.gy) + fabsf(qf.x) + fabsf(qf.y) + gu.cs) + 1e-30f;
        const int rmaxu = max(max(ucx, gu.gx - 1 - ucx), max(ucy, gu.gy - 1 - ucy));
        bool all_users = nL == 0 && A.nu > 0;
        int rend = -1;
        if (!all_users && A.nu > 0) {
            for (int r = 0;; ++r) {
                if (r > rmaxu) { rend = r - 1; break; }
                if (r > RM) { all_users = true; break; }
                int ncell = r == 0 ? 1 : 8 * r;
                bool anykeep = false;
                for (int t0 = 0; t0 < ncell; t0 += 32) {
                    int t = t0 + lane;
                    int dx = 0, dy = 0;
                    bool ok = t < ncell;
                    if (ok && r > 0) {
                        int side = 2 * r + 1;
                        if (t < side) { dx = -r + t; dy = -r; }
                        else if (t < 2 * side) { dx = -r + (t - side); dy = r; }
                        else if (t < 2 * side + (2 * r - 1)) { dx = -r; dy = -r + 1 + (t - 2 * side); }
                        else { dx = r; dy = -r + 1 + (t - 2 * side - (2 * r - 1)); }
                    }
                    int cxx = ucx + dx, cyy = ucy + dy;
                    ok = ok && cxx >= 0 && cxx < gu.gx && cyy >= 0 && cyy < gu.gy;
                    bool keep = false;
                    if (ok) {
                        float X0 = (gu.x0 + (float)cxx * gu.cs) - qf.x - delta;
                        float X1 = (gu.x0 + (float)(cxx + 1) * gu.cs) - qf.x + delta;
                        float Y0 = (gu.y0 + (float)cyy * gu.cs) - qf.y - delta;
                        float Y1 = (gu.y0 + (float)(cyy + 1) * gu.cs) - qf.y + delta;
                        int viol = 0;
                        for (int m = 0; m < nL && viol < k; ++m) {
                            float4 p = IX(S.splanes, m);
                            float X = p.x > 0.0f ? X1 : X0;
                            float Y = p.y > 0.0f ? Y1 : Y0;
                            float mx = fmaf(p.x, X, fmaf(p.y, Y, p.z));
                            float bd = 8.0f * kU32 * fmaf(fabsf(p.x), fabsf(X), fmaf(fabsf(p.y), fabsf(Y), fabsf(p.z))) + 1e-30f;
                            viol += (mx < -bd);
                        }
                        keep = viol < k;
                    }
                    if (keep) {
                        int bit = (dy + RM) * W + (dx + RM);
                        atomicOr(&IX(S.bitmap, bit >> 5), 1u << (bit & 31));
                    }
                    anykeep |= keep;
                }
                anykeep = __any_sync(FULL, anykeep);
                if (!anykeep && r >= 1) { rend = r - 1; break; }
                rend = r;
            }
            zs.rings = rend + 1;
        }
        WSYNC();

        // ---- segments: one user range per row ------------------------------
        int2* seg = A.segs + (size_t)s * A.seg_cap;
        int nseg = 0, ncand = 0;
        if (all_users) {
            seg[0] = make_int2(0, 0);
            seg[1] = make_int2(0, A.nu);
            nseg = 1;
            ncand = A.nu;
            qflags |= QF_ALL_USERS;
        } else {
            int y0 = max(0, ucy - rend), y1 = min(gu.gy - 1, ucy + rend);
            int xl0 = max(0, ucx - rend), xl1 = min(gu.gx - 1, ucx + rend);
            for (int r0 = y0; r0 <= y1; r0 += 32) {
                int row = r0 + lane;
                int st = 0, len = 0;
                if (row <= y1) {
                    int dy = row - ucy;
                    int xmin = INT_MAX, xmax = -1;
                    for (int cxx = xl0; cxx <= xl1; ++cxx) {
                        int bit = (dy + RM) * W + (cxx - ucx + RM);
                        if (IX(S.bitmap, bit >> 5) & (1u << (bit & 31))) {
                            xmin = min(xmin, cxx);
                            xmax = cxx;
                        }
                    }
                    if (xmax >= 0) {
                        st = A.ustart[GX(row * gu.gx + xmin, NCU + 1, 104)];
                        len = A.ustart[GX(row * gu.gx + xmax + 1, NCU + 1, 104)] - st;
                    }
                }
                bool has = len > 0;
                unsigned m = __ballot_sync(FULL, has);
                int pre = __popc(m & ((1u << lane) - 1));
                // prefix of lengths within the warp
                int incl = has ? len : 0;
                for (int o = 1; o < 32; o <<= 1) {
                    int v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += v;
                }
                int excl = incl - (has ? len : 0);
                if (has) seg[GX(nseg + pre, A.seg_cap, 108)] = make_int2(st, ncand + excl);
                nseg += __popc(m);
                ncand += __shfl_sync(FULL, incl, 31);
            }
            if (lane == 0) seg[GX(nseg, A.seg_cap, 109)] = make_int2(0, ncand);
        }

        PHASE(7);
#undef PHASE
        if (lane == 0) {
            QDesc d;
            d.qx = qf.x;
            d.qy = qf.y;
            d.qpos = qpos;
            d.k = k;
            d.nb = nL;
            d.nseg = nseg;
            d.k2f = k2f;
            d.kf2 = kf2;
            d.k2f64 = k2f64;
            d.kf264 = kf264;
            d.ncand = ncand;
            d.flags = qflags;
            d.rho = 0.0f;           // the zone's bisectors need not cover any disc
            d.pad = 0;
            *qd = d;
            A.zst[s] = zs;
        }
        WSYNC();
    }
}
#undef WSYNC

// at most 128 registers, so that 16 one-warp blocks fit an SM when the
// shared state allows as many
__global__ void __launch_bounds__(ZONE_WARPS * 32, 16) zone_kernel_smem(ZoneArgs a) { zone_body(a); }

}  // namespace rknn
