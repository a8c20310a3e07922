// kernel_body.cuh - the transport kernel (included by transport.cu).
//
// Layout of the work: every lane of a warp owns one history at a time.  Each loop iteration
// is one Woodcock step (src/MIDSX/Core/physics_engine.cpp:28-79) for every lane that is
// flying.  The long, rare pieces of work are "events": a real collision (interaction type,
// Rayleigh / Compton / photoelectric sampling, tallies, dose) and the start of a new history
// (history id, source sampling, per-energy table lookups).  A lane that needs an event
// parks; the warp runs the parked events once `regroup` of its lanes wait - or no lane is
// left flying - so that event code runs with many lanes active instead of one (warp ballot;
// each interaction type is then a branch of its own).
//
// Work distribution: history indices are handed out by one atomic per warp start-event
// (`chunk` indices per starting lane), so fast and slow histories balance across the whole
// grid.  A single-job launch takes its job from the kernel parameters; a batched launch
// (MULTI) maps each index to a job through the launch's prefix table and reads the job's
// geometry from shared memory, so simulations with different phantoms, sources and history
// counts run together in one persistent launch.  Per-history counters stay in 32-bit
// registers and are flushed to shared-memory per-job counters when the history ends; one
// atomic per block, job and counter at the end.

// per-energy cache: majorant and every material's total cross section and delta-scatter
// threshold (isDeltaScatter: p_delta = 1 - mu / mu_max), kept per thread in shared memory.
// Both forms multiply by one reciprocal of the majorant instead of dividing per material
// (with the same change in interaction_probs, rotate_half and the source direction: FP32
// +9.3 %, FP64 +4.6 % with the Compton trial below, on the cone-beam dose workload; the
// thresholds move by an ulp, the Woodcock steps per history by 3e-9).
template <typename R>
__device__ __forceinline__ R refresh_energy(const RunParams& P, R E, R* thr, R* mu, int stride) {
    const EnergyKey<R> key = energy_key<R>(P.T, E);  // one log10 and bucket for every table
    R mu_max = lin_lookup_key<R>(P.T, P.T.majorant, key);
    const R imax = R(1) / mu_max;
    for (int m = 0; m < P.T.n_materials; ++m) {
        R mm = lin_lookup_key<R>(P.T, P.T.mat[m].total, key);
        mu[m * stride] = mm;
        thr[m * stride] = R(1) - mm * imax;
    }
    return mu_max;
}

// The same, out of line: the single-job FP32 photon-pool kernel calls this copy (+0.8 % on
// the cone-beam dose workload: one copy of the M + 1 table lookups in the kernel's code); the
// batched kernel keeps the inlined one (out of line there: -2.7 %).
template <typename R>
__device__ __noinline__ R refresh_energy_call(const RunParams& P, R E, R* thr, R* mu, int stride) {
    return refresh_energy<R>(P, E, thr, mu, stride);
}

// setInteractionType's probabilities (physics_engine.cpp:82-109): coherent and incoherent
// cross sections (LogLogSpline) over the material's total, at one energy key.  (Inlined: an
// out-of-line copy measured 4-5 % slower, the call saving registers around it.)
template <typename R>
__device__ __forceinline__ void interaction_probs(const DevTables& T, const DevMaterial& Mt, R E, R mu_tot, R& p_coh,
                                               R& p_incoh) {
    const EnergyKey<R> key = energy_key<R>(T, E);
    // one copy of the spline evaluation, run for both cross sections
    R coh = R(0), incoh = R(0);
#pragma unroll 1
    for (int w = 0; w < 2; ++w) {
        const R v = spline_lookup_key<R>(T, w ? Mt.incoh : Mt.coh, key);
        if (w) incoh = v;
        else coh = v;
    }
    const R im = R(1) / mu_tot;  // one division for both probabilities
    p_coh = coh * im;
    p_incoh = incoh * im;
}

// scatter_direction for the coherent and incoherent branches.
template <typename R>
__device__ __forceinline__ V3<R> scatter_dir(const V3<R>& v, R mu, R u) {
    return scatter_direction(v, mu, u);
}

// Compton scattering by Kahn's method with the S(x) rejection
// (src/MIDSX/Core/photon_interactions.cpp:62-141).  Returns false at the trial cap.
template <typename R>
__device__ __forceinline__ bool sample_compton(const RunParams& P, const DevMaterial& Mt, HistoryRng& rng, R E, R& mu,
                                            R& kp, uint32_t& trials) {
    R alpha;
    if constexpr (sizeof(R) == 8)
        alpha = P.T.alpha;
    else
        alpha = P.T.alpha_f;
    const R k = E / R(kMec2);
    const R r1p = (R(1) + R(2) * k) / (R(9) + R(2) * k);
    const R s_max = lin_lookup<R>(P.T, Mt.sfunc, alpha * k * sqrt_(R(2)));
    // Kahn's trial (photon_interactions.cpp:62-141) with one division instead of six to eight:
    // with b = 1 + 2k r2 and a = 1 + 2k, chi = b (first branch) or a / b (second), 1/chi = b / a
    // there, and 1/k - 1/kp = (1 - chi)/k; 1/k, 1/a and 1/s_max are taken once per event.
    // Equal to the reference's expressions up to rounding (FP32 +2.5 % on the cone-beam dose
    // workload; FP64 histories still equal the oracle's, which keeps them, to 1e-9).
    const R ik = R(1) / k, k2 = R(2) * k, a = R(1) + k2, ia = R(1) / a, is_max = R(1) / s_max;
    for (int trial = 0; trial < P.max_trials; ++trial) {
        ++trials;
        R r1 = uniform<R>(rng), r2 = uniform<R>(rng), r3 = uniform<R>(rng);
        R chi, ichi;
        const R b = R(1) + k2 * r2;
        if (r1 <= r1p) {
            chi = b;
            ichi = R(1) / chi;
            if (!(r3 <= R(4) * ichi * (R(1) - ichi))) continue;
        } else {
            ichi = b * ia;
            chi = a / b;
            R tt = (R(1) - chi) * ik + R(1);
            if (!(R(2) * r3 <= tt * tt + ichi)) continue;
        }
        kp = k * ichi;
        mu = R(1) + (R(1) - chi) * ik;
        R x = alpha * k * sqrt_(R(1) - mu);
        R accept = lin_lookup<R>(P.T, Mt.sfunc, x) * is_max;
        if (uniform<R>(rng) <= accept) return true;
    }
    return false;
}

template <typename R, bool MX>
__device__ __forceinline__ void score_dose(unsigned long long* dose, int stride, int vox, R dep) {
    unsigned long long* rec = dose + size_t(vox) * stride;
    Acc<MX>::energy(rec, dep);
    if (stride > 1) {
        Acc<MX>::energy2(rec + 1, dep);
        count1(rec + 2);
    }
}

__device__ __forceinline__ void stat_add(unsigned long long* s, int slot, unsigned long long v) {
    if (v) atomicAdd(s + slot, v);
}

// statistics energies in fixed point (1/1024 eV); the FP32 form converts with a 32-bit
// conversion (energies below 4 MeV)
__device__ __forceinline__ unsigned long long fx_stat(double e) { return (unsigned long long)llrint(e * kFxStat); }
__device__ __forceinline__ unsigned long long fx_stat(float e) {
    return (unsigned long long)__float2uint_rn(e * float(kFxStat));
}

// Distance along the ray p + t d (t >= 0) to the closed box [lo, lo + ext], +inf if the ray
// misses it (slab method) or meets it for no more than `tol` (grazing it, or leaving it from
// a point within tol of its far side); 0 if p is inside.  The FP32 forms here, in box_span
// and in the macro-cell walk's set-up multiply by one reciprocal of each direction component
// (and of the cell size) instead of dividing twice or three times (+9 % macro-cell tracking,
// +3 % background fast tracking); the FP64 forms divide.
template <typename R>
__device__ __forceinline__ R box_entry(const V3<R>& p, const V3<R>& d, const V3<R>& lo, const V3<R>& ext, R tol) {
    R tmin = R(0), tmax = R(INFINITY);
    const R pp[3] = {p.x, p.y, p.z}, dd[3] = {d.x, d.y, d.z}, ll[3] = {lo.x, lo.y, lo.z}, ee[3] = {ext.x, ext.y, ext.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (dd[a] == R(0)) {
            if (pp[a] < ll[a] || pp[a] > ll[a] + ee[a]) return R(INFINITY);
            continue;
        }
        R t1, t2;
        if constexpr (sizeof(R) == 4) {
            const R id = adiv(R(1), dd[a]);
            t1 = (ll[a] - pp[a]) * id;
            t2 = (ll[a] + ee[a] - pp[a]) * id;
        } else {
            t1 = (ll[a] - pp[a]) / dd[a];
            t2 = (ll[a] + ee[a] - pp[a]) / dd[a];
        }
        if (t1 > t2) {
            const R t = t1;
            t1 = t2;
            t2 = t;
        }
        tmin = t1 > tmin ? t1 : tmin;
        tmax = t2 < tmax ? t2 : tmax;
    }
    return tmax > tmin + tol ? tmin : R(INFINITY);
}

// The rounding allowance of a grid's faces: 1e-4 of its smallest voxel edge.
template <typename R>
__device__ __forceinline__ R face_tol(const V3<R>& spc) {
    const R m = spc.x < spc.y ? spc.x : spc.y;
    return R(1e-4) * (m < spc.z ? m : spc.z);
}

// Distance along a ray from the background to the first grid box it enters, +inf if none.
// A grid the ray only grazes, or leaves from a point within the rounding allowance of its
// face (where a macro-cell flight ends), is not entered.
template <typename R, bool MX>
__device__ __forceinline__ R grid_entry(const Geo<R>& g, const V3<R>& p, const V3<R>& d) {
    R best = box_entry<R>(p, d, g.org, g.ext, face_tol<R>(g.spc));
    for (int k = 0; k + 1 < g.n_grids; ++k) {
        const DevGrid& G = g.extra[k];
        V3<R> o, e;
        if constexpr (MX) {
            o = {G.f_origin[0], G.f_origin[1], G.f_origin[2]};
            e = {G.f_ext[0], G.f_ext[1], G.f_ext[2]};
        } else {
            o = {G.origin[0], G.origin[1], G.origin[2]};
            e = {G.ext[0], G.ext[1], G.ext[2]};
        }
        const V3<R> sp = {R(G.spacing[0]), R(G.spacing[1]), R(G.spacing[2])};
        const R t = box_entry<R>(p, d, o, e, face_tol<R>(sp));
        best = t < best ? t : best;
    }
    return best;
}

// Ray p + t d against the closed box [lo, lo + ext]: the parameter interval [t0, t1] inside
// it (t0 > t1 when the ray misses).
template <typename R>
__device__ __forceinline__ void box_span(const V3<R>& p, const V3<R>& d, const V3<R>& lo, const V3<R>& ext, R& t0,
                                         R& t1) {
    t0 = -R(INFINITY);
    t1 = R(INFINITY);
    const R pp[3] = {p.x, p.y, p.z}, dd[3] = {d.x, d.y, d.z}, ll[3] = {lo.x, lo.y, lo.z}, ee[3] = {ext.x, ext.y, ext.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (dd[a] == R(0)) {
            if (pp[a] < ll[a] || pp[a] > ll[a] + ee[a]) {
                t0 = R(INFINITY);
                t1 = -R(INFINITY);
            }
            continue;
        }
        R u1, u2;
        if constexpr (sizeof(R) == 4) {
            const R id = adiv(R(1), dd[a]);
            u1 = (ll[a] - pp[a]) * id;
            u2 = (ll[a] + ee[a] - pp[a]) * id;
        } else {
            u1 = (ll[a] - pp[a]) / dd[a];
            u2 = (ll[a] + ee[a] - pp[a]) / dd[a];
        }
        if (u1 > u2) {
            const R t = u1;
            u1 = u2;
            u2 = t;
        }
        t0 = u1 > t0 ? u1 : t0;
        t1 = u2 < t1 ? u2 : t1;
    }
}

// Cells one flight crosses at most; a longer flight ends on a cell face (through the sliver
// below) and goes on in the photon's next step.  Short walks keep the lanes of a warp
// together: 16 against an unbounded walk measured +8 % on the cone-beam dose workload and
// +10 % on the lead radiography (8^3 cells), and 3.1e8 against 2.8e8 histories/s on the
// radiography with 4^3 cells.
constexpr int kCellWalkLimit = 16;

// A flight of the opt-in tracking modes that reaches a face (a grid entered from the
// background, a grid left, the walk limit) goes on past it for kCutSliver cm against the
// global majorant, valid everywhere, with the optical depth it has left: it ends inside that
// sliver at a tentative collision, or at the sliver's far end.  Flights therefore never stop
// on a face, so a tally plane or AACuboid face lying on a grid face sees each crossing in
// exactly one segment, whatever the rounding of the positions (about 1e-5 cm at 100 cm in
// FP32).
constexpr double kCutSliver = 1e-4;

// Macro-cell flight (MIDSX_TRACK_MACRO_CELL) from p along d with optical depth tau; the
// cells come from the job's DevGeom (kept out of Geo, which the reference path holds).  The
// grid the ray is in (first-hit order, p inside or on a face it enters through) is walked
// cell by cell (Amanatides-Woo): a cell of material mask m has the majorant
// max_{k in m} mu[k * stride] at the photon's energy, and the depth is spent there.
// Returns 0: the depth runs out at s in a cell of majorant mu_c (tentative collision);
// 1: the walk reaches the grid's face at s (or a cell face after kCellWalkLimit cells) with
// the depth tau_rem left; 2: no grid holds the ray's start (background).
template <typename R, bool MX>
__device__ __forceinline__ int cell_flight(const Geo<R>& g, const DevGeom& D, const R* mu, int stride, const V3<R>& p,
                                           const V3<R>& d, R tau, R& s, R& mu_c, R& tau_rem) {
    // which grid: the first whose box holds the start within the rounding allowance of its
    // faces (t0 <= tol) and that the ray does not leave within that allowance (t1 > tol:
    // a flight that ended on a grid's far face continues in the background)
    V3<R> org = g.org, ext = g.ext, spc = g.spc;
    int cn[3] = {D.cdims[0], D.cdims[1], D.cdims[2]};
    const uint32_t* cells = D.cells;
    R t0, t1;
    box_span<R>(p, d, org, ext, t0, t1);
    R tol = face_tol<R>(spc);
    bool found = t0 <= tol && t1 > tol && t0 <= t1;
    for (int k = 0; !found && k + 1 < g.n_grids; ++k) {
        const DevGrid& G = g.extra[k];
        if constexpr (MX) {
            org = {G.f_origin[0], G.f_origin[1], G.f_origin[2]};
            ext = {G.f_ext[0], G.f_ext[1], G.f_ext[2]};
        } else {
            org = {G.origin[0], G.origin[1], G.origin[2]};
            ext = {G.ext[0], G.ext[1], G.ext[2]};
        }
        spc = {R(G.spacing[0]), R(G.spacing[1]), R(G.spacing[2])};
        box_span<R>(p, d, org, ext, t0, t1);
        tol = face_tol<R>(spc);
        found = t0 <= tol && t1 > tol && t0 <= t1;
        if (found) {
            cn[0] = G.cdims[0];
            cn[1] = G.cdims[1];
            cn[2] = G.cdims[2];
            cells = D.cells + G.cell_offset;
        }
    }
    if (!found) return 2;
    // start cell: from the point a little inside along the ray, clamped into the grid
    R t = t0 > R(0) ? t0 : R(0);
    const R edge = R(1 << D.cell_shift);
    const R csz[3] = {spc.x * edge, spc.y * edge, spc.z * edge};
    const R pp[3] = {p.x, p.y, p.z}, dd[3] = {d.x, d.y, d.z}, oo[3] = {org.x, org.y, org.z};
    const R tend = t1 < t + tol ? t1 : t + tol;
    const R tin = t + R(0.5) * (tend - t);  // the start cell is the one holding p + tin d
    // per axis: the next cell face along the ray (tn*), the distance between faces (dt*), the
    // cell index step (inc*) and the cells left before the grid's side (left*) - scalars, so
    // that the walk stays in registers
    R tn3[3], dt3[3];
    int inc3[3], left3[3], idx = 0, stride3 = 1;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        R q;
        if constexpr (sizeof(R) == 4)
            q = (pp[a] + tin * dd[a] - oo[a]) * adiv(R(1), csz[a]);
        else
            q = (pp[a] + tin * dd[a] - oo[a]) / csz[a];
        int ci = q >= R(0) ? int(q) : 0;
        ci = ci >= cn[a] ? cn[a] - 1 : ci;
        idx += ci * stride3;
        if (dd[a] > R(0)) {
            inc3[a] = stride3;
            left3[a] = cn[a] - 1 - ci;
            if constexpr (sizeof(R) == 4) {
                const R id = adiv(R(1), dd[a]);
                tn3[a] = (oo[a] + R(ci + 1) * csz[a] - pp[a]) * id;
                dt3[a] = csz[a] * id;
            } else {
                tn3[a] = (oo[a] + R(ci + 1) * csz[a] - pp[a]) / dd[a];
                dt3[a] = csz[a] / dd[a];
            }
        } else if (dd[a] < R(0)) {
            inc3[a] = -stride3;
            left3[a] = ci;
            if constexpr (sizeof(R) == 4) {
                const R id = adiv(R(1), dd[a]);
                tn3[a] = (oo[a] + R(ci) * csz[a] - pp[a]) * id;
                dt3[a] = -csz[a] * id;
            } else {
                tn3[a] = (oo[a] + R(ci) * csz[a] - pp[a]) / dd[a];
                dt3[a] = -csz[a] / dd[a];
            }
        } else {
            inc3[a] = 0;
            left3[a] = 0;
            tn3[a] = R(INFINITY);
            dt3[a] = R(INFINITY);
        }
        stride3 *= cn[a];
    }
    R tnx = tn3[0], tny = tn3[1], tnz = tn3[2];
    const R dtx = dt3[0], dty = dt3[1], dtz = dt3[2];
    const int incx = inc3[0], incy = inc3[1], incz = inc3[2];
    int leftx = left3[0], lefty = left3[1], leftz = left3[2];
    // the next cell's mask is loaded while this cell is evaluated, and a cell with the mask of
    // the one before reuses its majorant
    uint32_t m = __ldg(cells + idx), m_prev = 0u;
    R mc = R(0);
    for (int it = 0; it < kCellWalkLimit; ++it) {
        const int a = tnx < tny ? (tnx < tnz ? 0 : 2) : (tny < tnz ? 1 : 2);
        const R tf = a == 0 ? tnx : (a == 1 ? tny : tnz);
        const int left = a == 0 ? leftx : (a == 1 ? lefty : leftz);
        const int nidx = idx + (a == 0 ? incx : (a == 1 ? incy : incz));
        const uint32_t mn = left > 0 ? __ldg(cells + nidx) : 0u;
        if (m != m_prev) {
            mc = R(0);
            for (uint32_t b = m; b; b &= b - 1u) {
                const R v = mu[(__ffs(int(b)) - 1) * stride];
                mc = v > mc ? v : mc;
            }
            m_prev = m;
        }
        R tn = tf < t1 ? tf : t1;
        tn = tn > t ? tn : t;
        const R depth = mc * (tn - t);
        if (tau < depth) {
            s = t + adiv(tau, mc);
            mu_c = mc;
            return 0;
        }
        tau -= depth;
        t = tn;
        if (tn >= t1 || left <= 0) break;
        idx = nidx;
        m = mn;
        if (a == 0) {
            --leftx;
            tnx += dtx;
        } else if (a == 1) {
            --lefty;
            tny += dty;
        } else {
            --leftz;
            tnz += dtz;
        }
    }
    s = t;
    mu_c = R(0);
    tau_rem = tau;
    return 1;
}

// ComputationalDomain::getVoxel (computational_domain.cpp:23-31) for a point of the domain:
// the first grid whose closed box holds the point gives the voxel - vox is its number in the
// phantom (grid after grid), mat its material - else the background (vox = -1).  Inside a grid
// the index is trunc(offset / spacing) (VoxelGrid::getVoxelIndex, voxel_grid.cpp:55-59),
// taken here as trunc(offset * (1 / spacing)) in both precisions: the reciprocal is the job's,
// computed once, and the index differs from the quotient's only for an offset within an ulp of
// a voxel face.  In the FP64 form, whose time goes to the FP64 pipe, this and the free path
// -ln U * (1 / mu_max) instead of two divisions per Woodcock step measured +22 %; the FP64
// histories still equal the oracle's (which divides, as the reference) to 1e-9.
// An index equal to the grid size (the point on the far face, where the reference's
// vector::at would throw) is clamped and counted.
template <typename R, bool MX>
__device__ __forceinline__ void locate(const Geo<R>& g, const V3<R>& pos, int& vox, int& mat, uint32_t& fetches,
                                       unsigned long long* st) {
    vox = -1;
    mat = g.bg;
    const V3<R> q = {pos.x - g.org.x, pos.y - g.org.y, pos.z - g.org.z};
    if (q.x >= R(0) && q.x <= g.ext.x && q.y >= R(0) && q.y <= g.ext.y && q.z >= R(0) && q.z <= g.ext.z) {
        int ix, iy, iz;
        ix = int(q.x * g.ispc.x);
        iy = int(q.y * g.ispc.y);
        iz = int(q.z * g.ispc.z);
        if (ix >= g.nx || iy >= g.ny || iz >= g.nz) {
            stat_add(st, kStEdge, 1);
            ix = min(ix, g.nx - 1);
            iy = min(iy, g.ny - 1);
            iz = min(iz, g.nz - 1);
        }
        vox = ix + iy * g.nx + iz * g.nx * g.ny;
        mat = __ldg(g.ids + vox);
        ++fetches;
        return;
    }
    for (int k = 0; k + 1 < g.n_grids; ++k) {
        const DevGrid& G = g.extra[k];
        V3<R> o, e;
        if constexpr (MX) {
            o = {G.f_origin[0], G.f_origin[1], G.f_origin[2]};
            e = {G.f_ext[0], G.f_ext[1], G.f_ext[2]};
        } else {
            o = {G.origin[0], G.origin[1], G.origin[2]};
            e = {G.ext[0], G.ext[1], G.ext[2]};
        }
        const V3<R> r = {pos.x - o.x, pos.y - o.y, pos.z - o.z};
        if (!(r.x >= R(0) && r.x <= e.x && r.y >= R(0) && r.y <= e.y && r.z >= R(0) && r.z <= e.z)) continue;
        int ix, iy, iz;
        if constexpr (MX) {
            ix = int(r.x * G.f_ispc[0]);
            iy = int(r.y * G.f_ispc[1]);
            iz = int(r.z * G.f_ispc[2]);
        } else {
            ix = int(r.x / G.spacing[0]);
            iy = int(r.y / G.spacing[1]);
            iz = int(r.z / G.spacing[2]);
        }
        if (ix >= G.dims[0] || iy >= G.dims[1] || iz >= G.dims[2]) {
            stat_add(st, kStEdge, 1);
            ix = min(ix, G.dims[0] - 1);
            iy = min(iy, G.dims[1] - 1);
            iz = min(iz, G.dims[2] - 1);
        }
        vox = G.offset + ix + iy * G.dims[0] + iz * G.dims[0] * G.dims[1];
        mat = __ldg(g.ids + vox);
        ++fetches;
        return;
    }
}

// Shared-memory bytes of a launch: per-job counters, the batch's prefix table and geometry,
// then the per-thread energy cache.
template <typename R>
__host__ __device__ inline size_t kernel_smem(int n_jobs, bool multi, int n_materials, int block) {
    size_t b = size_t(n_jobs) * kStCount * 8;
    if (multi) b += size_t(n_jobs + 1) * 8 + size_t(n_jobs) * sizeof(Geo<R>);
    b = (b + 15) & ~size_t(15);
    return b + size_t(2) * n_materials * block * sizeof(R);
}

template <typename R, bool MULTI>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 3) transport_kernel(const RunParams P) {
    constexpr bool MX = sizeof(R) == 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int njobs = MULTI ? P.n_jobs : 1;
    unsigned long long* s_stats = reinterpret_cast<unsigned long long*>(smem_raw);
    unsigned long long* s_prefix = s_stats + njobs * kStCount;
    Geo<R>* s_geo = reinterpret_cast<Geo<R>*>(s_prefix + (MULTI ? njobs + 1 : 0));
    size_t head = size_t(njobs) * kStCount * 8 + (MULTI ? size_t(njobs + 1) * 8 + size_t(njobs) * sizeof(Geo<R>) : 0);
    R* cache = reinterpret_cast<R*>(smem_raw + ((head + 15) & ~size_t(15)));
    const int stride = blockDim.x;
    const int M = P.T.n_materials;
    R* thr = cache + threadIdx.x;
    R* mucache = cache + M * stride + threadIdx.x;
    for (int i = threadIdx.x; i < njobs * kStCount; i += blockDim.x) s_stats[i] = 0;
    if (MULTI) {
        for (int i = threadIdx.x; i <= njobs; i += blockDim.x) s_prefix[i] = P.prefix[i];
        for (int i = threadIdx.x; i < njobs; i += blockDim.x) s_geo[i] = make_geo<R>(P.jobs[i].G);
    }
    __syncthreads();
    const Geo<R>& g0 = job0_geo(P, R(0));  // single-job launches
    const unsigned long long epoch = P.epoch ? *P.epoch : 0ull;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;

    bool alive = false, pending = false, exhausted = false;
    unsigned long long next = 0, end = 0, gidx = 0;
    int job = 0, ntal = 0;
    HistoryRng rng;
    V3<R> pos, dir, p0;
    R E = R(0), mu_max = R(0), inv_mu_max = R(0), s = R(0);
    int n_coh = 0, n_incoh = 0, vox = -1, mat = 0;
    uint32_t steps = 0, fetches = 0, trials = 0, words = 0;
    uint32_t spar = 0u;  // step parity at the start of the flight segment (HistoryRng)
    R hist_dep = R(0);
    unsigned mask = 0xffffffffu;

    auto end_history = [&]() {
        if (!MULTI && P.trace) P.trace[gidx] = hist_dep;
        unsigned long long* st = s_stats + job * kStCount;
        stat_add(st, kStSteps, steps);
        stat_add(st, kStFetches, fetches);
        stat_add(st, kStTrials, trials);
        stat_add(st, kStWords, words);
        alive = false;
        pending = false;
    };

    for (;;) {
        const bool done = !alive && exhausted;
        mask = __ballot_sync(mask, !done);
        if (done) break;
        const Geo<R>& g = MULTI ? s_geo[job] : g0;
        unsigned long long* st = s_stats + job * kStCount;
        bool finish = false;  // the history ends in this iteration
        if (alive && !pending) {
            // one Woodcock step: getFreePath, move, domain test, voxel fetch, isDeltaScatter
            if (steps >= uint32_t(P.max_steps)) {
                stat_add(st, kStStepCap, 1);
                finish = true;
            } else {
                // the step's uniforms: word pair (0, 1) or (2, 3) of its block (HistoryRng)
                const uint32_t si = steps + spar;
                ++steps;
                const Philox4 q = rng.step_block(si);
                const uint64_t w1 = uint64_t((si & 1u) ? q.v[2] : q.v[0]) << 32;
                const uint64_t w2 = uint64_t((si & 1u) ? q.v[3] : q.v[1]) << 32;
                // getFreePath.  The FP32 form uses the hardware log2 (absolute error ~1e-7 near
                // U = 1, clamped at zero so that a step never goes backwards).
                if constexpr (MX)
                    s = fmaxf(-__logf(to_uniform(w1, R(0))), 0.0f) * inv_mu_max;
                else
                    s = -log_(to_uniform(w1, R(0))) * inv_mu_max;
                p0 = pos;
                pos = {pos.x + s * dir.x, pos.y + s * dir.y, pos.z + s * dir.z};
                if (!(pos.x >= R(0) && pos.x <= g.dom.x && pos.y >= R(0) && pos.y <= g.dom.y && pos.z >= R(0) &&
                      pos.z <= g.dom.z)) {
                    if (ntal) {
                        const DevTally* tal = MULTI ? P.jobs[job].tallies : P.job0.tallies;
                        score_tallies<R, MX>(tal, ntal, p0, dir, s, E, scatter_class(n_coh, n_incoh), 0, false, R(0),
                                             words);
                    }
                    stat_add(st, kStEscE, fx_stat(E));
                    finish = true;
                } else {
                    locate<R, MX>(g, pos, vox, mat, fetches, st);
                    if (to_uniform(w2, R(0)) < thr[mat * stride]) {
                        if (ntal) {
                            const DevTally* tal = MULTI ? P.jobs[job].tallies : P.job0.tallies;
                            score_tallies<R, MX>(tal, ntal, p0, dir, s, E, scatter_class(n_coh, n_incoh), 0, false,
                                                 R(0), words);
                        }
                    } else {
                        pending = true;  // a real collision: an event
                    }
                }
            }
        }
        if (finish) end_history();
        // events: run the parked collisions and history starts once enough lanes wait
        const bool want = pending || (!alive && !exhausted);
        const unsigned wmask = __ballot_sync(mask, want);
        const unsigned fmask = __ballot_sync(mask, alive && !pending);
        const bool go = __popc(wmask) >= P.regroup || fmask == 0u;
        const unsigned start_mask = go ? (wmask & ~__ballot_sync(mask, alive)) : 0u;
        if (want && go) {
            finish = false;
            if (!alive) {
                // hand out history indices: one atomic per warp for the lanes that hold none
                const unsigned need = __ballot_sync(start_mask, next >= end);
                if (next >= end) {
                    const int leader = __ffs(need) - 1;
                    unsigned long long base = 0;
                    if (int(lane) == leader)
                        base = atomicAdd(P.counter, (unsigned long long)__popc(need) * (unsigned long long)P.chunk);
                    base = __shfl_sync(need, base, leader);
                    next = base + (unsigned long long)__popc(need & lanes_below) * P.chunk;
                    end = next + P.chunk;
                    if (end > P.total) end = P.total;
                }
                if (next >= P.total) {
                    exhausted = true;
                } else {
                    gidx = next++;
                    uint64_t seed, hid;
                    if (MULTI) {
                        int lo = 0, hi = njobs;  // last job with prefix <= gidx
                        while (hi - lo > 1) {
                            int mid = (lo + hi) >> 1;
                            if (s_prefix[mid] <= gidx) lo = mid;
                            else hi = mid;
                        }
                        job = lo;
                        const DevJob& J = P.jobs[job];
                        seed = J.seed;
                        hid = J.first + epoch * J.n + (gidx - s_prefix[job]);
                        ntal = J.n_tallies;
                    } else {
                        seed = P.job0.seed;
                        hid = P.job0.first + epoch * P.job0.n + gidx;
                        ntal = P.job0.n_tallies;
                    }
                    // PhotonSource::generatePhoton + a fresh per-history stream
                    rng.init(seed, hid);
                    sample_source<R>(MULTI ? P.jobs[job].S : P.job0.S, rng, pos, dir, E);
                    unsigned long long* sj = s_stats + job * kStCount;
                    stat_add(sj, kStHistories, 1);
                    stat_add(sj, kStSourceE, fx_stat(E));
                    n_coh = n_incoh = 0;
                    steps = fetches = trials = words = 0;
                    spar = 0u;
                    hist_dep = R(0);
                    mu_max = refresh_energy<R>(P, E, thr, mucache, stride);
                    inv_mu_max = R(1) / mu_max;
                    alive = true;
                }
            } else {
                pending = false;
                // setInteractionType (physics_engine.cpp:82-109)
                const DevMaterial& Mt = P.T.mat[mat];
                const R mu_tot = mucache[mat * stride];
                R p_coh, p_incoh;
                interaction_probs<R>(P.T, Mt, E, mu_tot, p_coh, p_incoh);
                rng.align_event();
                const R u3 = uniform<R>(rng);
                const int cls0 = scatter_class(n_coh, n_incoh);
                const R E0 = E;
                const V3<R> d0 = dir;
                R dep = R(0);
                bool energy_changed = false, failed = false;
                if (u3 < p_coh) {
                    // CoherentScattering::interact
                    ++n_coh;
                    stat_add(st, kStCoh, 1);
                    R mu;
                    if (!rita_sample<R>(P.T, Mt.rita, E, uniform<R>(rng), mu)) {
                        stat_add(st, kStRangeErr, 1);
                        failed = true;
                    } else {
                        dir = scatter_dir(dir, mu, uniform<R>(rng));
                    }
                } else if (u3 < p_coh + p_incoh) {
                    // IncoherentScattering::interact
                    ++n_incoh;
                    stat_add(st, kStIncoh, 1);
                    R mu = R(1), kp = E / R(kMec2);
                    if (!sample_compton<R>(P, Mt, rng, E, mu, kp, trials)) {
                        stat_add(st, kStTrialCap, 1);
                        failed = true;
                    } else {
                        const R k = E / R(kMec2);
                        dir = scatter_dir(dir, mu, uniform<R>(rng));
                        E = kp * R(kMec2);
                        dep = R(kMec2) * (k - kp);
                        energy_changed = true;
                    }
                } else {
                    // PhotoelectricEffect::interact
                    stat_add(st, kStPhoto, 1);
                    dep = E;
                    finish = true;
                }
                if (failed) {
                    finish = true;
                } else {
                    if (ntal) {
                        const DevTally* tal = MULTI ? P.jobs[job].tallies : P.job0.tallies;
                        score_tallies<R, MX>(tal, ntal, p0, d0, s, E0, cls0, scatter_class(n_coh, n_incoh), true, dep,
                                             words);
                    }
                    if (dep != R(0)) {
                        if (vox >= 0) {
                            stat_add(st, kStDepGrid, fx_stat(dep));
                            hist_dep += dep;
                            const DevJob& J = MULTI ? P.jobs[job] : P.job0;
                            if (J.dose_stride) {
                                score_dose<R, MX>(J.dose, J.dose_stride, vox, dep);
                                ++words;
                            }
                        } else {
                            stat_add(st, kStDepBg, fx_stat(dep));
                        }
                    }
                    if (!finish) {
                        if (!(fabs_(dir.x) <= R(2) && fabs_(dir.y) <= R(2) && fabs_(dir.z) <= R(2))) {
                            // a NaN direction (RITA rows below ~400 eV are NaN, as in the
                            // reference); its next step would leave the domain: retire the history
                            stat_add(st, kStNonFinite, 1);
                            stat_add(st, kStEscE, fx_stat(E));
                            finish = true;
                        } else if (energy_changed) {
                            mu_max = refresh_energy<R>(P, E, thr, mucache, stride);
                            inv_mu_max = R(1) / mu_max;
                        }
                    }
                }
                spar = steps & 1u;  // a new flight segment (HistoryRng)
                if (finish) end_history();
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < njobs * kStCount; i += blockDim.x) {
        const unsigned long long v = s_stats[i];
        if (v) {
            const int j = i / kStCount;
            unsigned long long* dst = MULTI ? P.jobs[j].stats : P.job0.stats;
            atomicAdd(dst + (i - j * kStCount), v);
        }
    }
}

// Graph replays of a batch advance its epoch so that each replay transports fresh histories.
__global__ void advance_epoch_kernel(unsigned long long* epoch) { *epoch += 1ull; }
