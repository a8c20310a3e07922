// tally_warp.cuh - warp-aggregated tally and dose accumulation (included by transport.cu after
// the per-lane scoring; used by the photon-pool kernel).
//
// The 32 lanes of a warp score together.  Each lane's contribution to a tally is a record: a
// layout kind, the accumulator base, a class and one or two values, from which the record's
// words (counts, fixed-point or FP64 sums, sums of squares) follow.  Lanes whose records start
// at the same word (__match_any_sync on that address: same tally, same class, same bin or
// voxel) sum their words and one of them - the lowest lane - issues the atomics; when no two
// lanes share a record every lane issues its own.  The fixed-point words are converted per
// lane before the sum, so the integer totals equal those of per-lane atomics bit for bit.
//
// Record layouts (word addresses relative to the tally's accumulator `acc`; VectorQuantity
// records are [count, sum, sum of squares], see vec_energy / vec_cosine):
//   kRecSurface  scalar surface crossing: energy record of class c at acc + 3c, cosine record
//                at acc + 12 + 3c, crossing count at acc + 24 + c
//   kRecBinned   binned surface crossing: [energy, count] at the bin's class pair
//   kRecCubDep   AACuboid deposit: energy record at acc + 3c
//   kRecCubEnter AACuboid entry: energy record at acc + 12 + 3c, entry count at acc + 24 + c
//   kRecCubHit   AACuboid interaction count at acc + 28 + c
//   kRecDose     voxel dose: sum at rec[0]; with the full record also sum of squares rec[1]
//                and count rec[2] (c = record stride)

constexpr int kRecNone = 0, kRecSurface = 1, kRecBinned = 2, kRecCubDep = 3, kRecCubEnter = 4, kRecCubHit = 5,
              kRecDose = 6;
constexpr int kRecWords = 7;  // most words of one record

// One word of a record: its address and the value bits to add (0 = nothing), and whether the
// word holds an FP64 sum (the plain form's sums; counts are integers in both forms).
template <bool MX>
struct RecWord;

template <>
struct RecWord<true> {
    __device__ static unsigned long long energy(float v) {
        return (unsigned long long)__float2uint_rn(v * float(kFxEnergy));
    }
    __device__ static unsigned long long energy2(float v) {
        return (unsigned long long)__float2uint_rn(v * v * float(kFxEnergy2));
    }
    __device__ static unsigned long long cosine(float v) {
        return (unsigned long long)__float2uint_rn(v * float(kFxCosine));
    }
    __device__ static unsigned long long cosine2(float v) {
        return (unsigned long long)__float2uint_rn(v * v * float(kFxCosine));
    }
    static constexpr bool kDouble = false;
};

template <>
struct RecWord<false> {
    __device__ static unsigned long long energy(double v) { return (unsigned long long)__double_as_longlong(v); }
    __device__ static unsigned long long energy2(double v) {
        return (unsigned long long)__double_as_longlong(v * v);
    }
    __device__ static unsigned long long cosine(double v) { return (unsigned long long)__double_as_longlong(v); }
    __device__ static unsigned long long cosine2(double v) {
        return (unsigned long long)__double_as_longlong(v * v);
    }
    static constexpr bool kDouble = true;
};

// Word j of a record (addr = nullptr when the layout has no word j).
template <typename R, bool MX>
__device__ __forceinline__ void rec_word(int kind, unsigned long long* acc, int c, R v1, R v2, int j,
                                         unsigned long long*& addr, unsigned long long& bits, bool& dbl) {
    using W = RecWord<MX>;
    addr = nullptr;
    bits = 0;
    dbl = false;
    // a VectorQuantity record [count, sum, sum of squares] of value v at base: words 0..2
    // (the word type follows from the layout alone: peers with the same record sum their words
    // as the group leader's types say, whatever the leader's own value)
    auto vec = [&](unsigned long long* base, int jj, R v, bool cosine) {
        addr = base + jj;
        dbl = jj != 0 && W::kDouble;
        if (v == R(0)) return;  // measure() skips zero values
        if (jj == 0)
            bits = 1;
        else
            bits = jj == 1 ? (cosine ? W::cosine(v) : W::energy(v)) : (cosine ? W::cosine2(v) : W::energy2(v));
    };
    switch (kind) {
        case kRecSurface:
            if (j < 3) vec(acc + 3 * c, j, v1, false);
            else if (j < 6) vec(acc + 12 + 3 * c, j - 3, v2, true);
            else if (j == 6) {
                addr = acc + 24 + c;
                bits = 1;
            }
            break;
        case kRecBinned:
            if (j == 0) {
                addr = acc;
                bits = W::energy(v1);
                dbl = W::kDouble;
            } else if (j == 1) {
                addr = acc + 1;
                bits = 1;
            }
            break;
        case kRecCubDep:
            if (j < 3) vec(acc + 3 * c, j, v1, false);
            break;
        case kRecCubEnter:
            if (j < 3) vec(acc + 12 + 3 * c, j, v1, false);
            else if (j == 3) {
                addr = acc + 24 + c;
                bits = 1;
            }
            break;
        case kRecCubHit:
            if (j == 0) {
                addr = acc + 28 + c;
                bits = 1;
            }
            break;
        case kRecDose:
            if (j == 0) {
                addr = acc;
                bits = W::energy(v1);
                dbl = W::kDouble;
            } else if (c > 1 && j == 1) {
                addr = acc + 1;
                bits = W::energy2(v1);
                dbl = W::kDouble;
            } else if (c > 1 && j == 2) {
                addr = acc + 2;
                bits = 1;
            }
            break;
        default:
            break;
    }
}

__device__ __forceinline__ void add_word(unsigned long long* addr, unsigned long long bits, bool dbl) {
    if (dbl)
        atomicAdd(reinterpret_cast<double*>(addr), __longlong_as_double((long long)bits));
    else
        atomicAdd(addr, bits);
}

// Called by all 32 lanes; kind = kRecNone for a lane without a record.  `scratch` holds 32
// words of this warp.
template <typename R, bool MX>
__device__ __forceinline__ void warp_record(int kind, unsigned long long* acc, int c, R v1, R v2,
                                            unsigned long long* scratch) {
    constexpr unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long* first = nullptr;
    if (kind != kRecNone) {
        unsigned long long* a;
        unsigned long long b;
        bool d;
        rec_word<R, MX>(kind, acc, c, v1, v2, 0, a, b, d);
        first = a;
    }
    const unsigned long long key = (unsigned long long)first;
    if (!__any_sync(FULL, key != 0ull)) return;
    const unsigned peers = __match_any_sync(FULL, key);
    if (__all_sync(FULL, key == 0ull || peers == (1u << lane))) {
        // no two lanes share a record: each lane adds its own words
        if (key)
            for (int j = 0; j < kRecWords; ++j) {
                unsigned long long* a;
                unsigned long long b;
                bool d;
                rec_word<R, MX>(kind, acc, c, v1, v2, j, a, b, d);
                if (a && b) add_word(a, b, d);
            }
        return;
    }
    const bool leader = key != 0ull && int(lane) == __ffs(peers) - 1;
    for (int j = 0; j < kRecWords; ++j) {
        unsigned long long* a = nullptr;
        unsigned long long b = 0;
        bool d = false;
        if (key) rec_word<R, MX>(kind, acc, c, v1, v2, j, a, b, d);
        scratch[lane] = b;
        __syncwarp();
        if (leader && a) {
            unsigned long long isum = 0;
            double dsum = 0.0;
            for (unsigned p = peers; p; p &= p - 1u) {
                const unsigned long long x = scratch[__ffs(p) - 1];
                if (d)
                    dsum += __longlong_as_double((long long)x);
                else
                    isum += x;
            }
            if (d) {
                if (dsum != 0.0) add_word(a, (unsigned long long)__double_as_longlong(dsum), true);
            } else if (isum) {
                add_word(a, isum, false);
            }
        }
        __syncwarp();
    }
}

// score_tallies for the whole warp: lanes with `active` score the segment [p0, p0 + s d) of
// their own job's tallies (same geometry and semantics as score_tallies), tally by tally.
// SPEC: also incident-energy spectra (per lane: a collision segment crosses a spectrum
// surface rarely), compiled only into the kernels of launches that keep spectra.
template <typename R, bool MX, bool SPEC = false>
__device__ __forceinline__ void score_tallies_warp(bool active, const DevTally* tallies, int n_tallies,
                                                   const V3<R>& p0, const V3<R>& d, R s, R E, int cls0, int cls1,
                                                   bool interact, R dep, uint32_t& words,
                                                   unsigned long long* scratch) {
    const int nt = __reduce_max_sync(0xffffffffu, active ? n_tallies : 0);
    for (int ti = 0; ti < nt; ++ti) {
        int k1 = kRecNone, k2 = kRecNone, k3 = kRecNone;
        unsigned long long* acc = nullptr;
        int c = 0;
        R v1 = R(0), v2 = R(0), e_dep = R(0);
        if (active && ti < n_tallies) {
            const DevTally& T = tallies[ti];
            acc = T.acc;
            if (T.kind == MIDSX_TALLY_VOLUME_AACUBOID) {
                // AACuboidVolumeTally::determineVolumeTraversal (volume_tally.cpp:38-91)
                R lo[3], hi[3];
                const R pp[3] = {p0.x, p0.y, p0.z};
                const R dd[3] = {d.x, d.y, d.z};
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    if (fabs_(dd[i]) < R(kEps)) {
                        lo[i] = -R(INFINITY);
                        hi[i] = R(INFINITY);
                        continue;
                    }
                    lo[i] = (pickr<R>(T.a[i], T.fa[i]) - pp[i]) / dd[i];
                    hi[i] = (pickr<R>(T.b[i], T.fb[i]) - pp[i]) / dd[i];
                    if (lo[i] > hi[i]) {
                        R tmp = lo[i];
                        lo[i] = hi[i];
                        hi[i] = tmp;
                    }
                }
                R enter = lo[0] > lo[1] ? lo[0] : lo[1];
                enter = enter > lo[2] ? enter : lo[2];
                R exit_ = hi[0] < hi[1] ? hi[0] : hi[1];
                exit_ = exit_ < hi[2] ? exit_ : hi[2];
                if (!(enter > exit_ || exit_ < R(0) || enter > s)) {
                    bool counted;
                    if (enter <= R(0)) {
                        counted = true;
                        e_dep = (exit_ >= s) ? dep : R(0);  // STAYS keeps the deposit, EXITS zeroes it
                    } else {
                        counted = false;
                        e_dep = (exit_ < s) ? R(0) : dep;   // PASSES_THROUGH zeroes, LANDS_INSIDE keeps
                    }
                    c = cls1;
                    v1 = e_dep;
                    k1 = kRecCubDep;
                    if (e_dep != R(0)) ++words;
                    if (!counted) {
                        k2 = kRecCubEnter;
                        v2 = E;
                        if (E != R(0)) ++words;
                        ++words;
                    }
                    if (interact) {
                        k3 = kRecCubHit;
                        ++words;
                    }
                }
            } else {
                // SurfaceTally::willPassThrough (surface_tally.cpp:16-34)
                const V3<R> nrm = {pickr<R>(T.norm[0], T.fnorm[0]), pickr<R>(T.norm[1], T.fnorm[1]),
                                   pickr<R>(T.norm[2], T.fnorm[2])};
                const R ec = dot(d, nrm);
                bool hit = !(fabs_(ec) < R(kEps) || ec < R(0));
                V3<R> rel = {R(0), R(0), R(0)};
                R u = R(0), v = R(0);
                if (hit) {
                    const V3<R> a = {pickr<R>(T.a[0], T.fa[0]), pickr<R>(T.a[1], T.fa[1]), pickr<R>(T.a[2], T.fa[2])};
                    const V3<R> w = {a.x - p0.x, a.y - p0.y, a.z - p0.z};
                    const R t = dot(w, nrm) / ec;
                    hit = !(t > s || t < R(0));
                    const V3<R> ip = {p0.x + t * d.x, p0.y + t * d.y, p0.z + t * d.z};
                    rel = {ip.x - a.x, ip.y - a.y, ip.z - a.z};
                }
                if (hit && T.kind == MIDSX_TALLY_SURFACE_DISC) {
                    hit = !(sqrt_(dot(rel, rel)) > pickr<R>(T.radius, T.fradius));
                } else if (hit) {
                    const V3<R> e1 = {pickr<R>(T.b[0], T.fb[0]), pickr<R>(T.b[1], T.fb[1]), pickr<R>(T.b[2], T.fb[2])};
                    const V3<R> e2 = {pickr<R>(T.c[0], T.fc[0]), pickr<R>(T.c[1], T.fc[1]), pickr<R>(T.c[2], T.fc[2])};
                    u = dot(e1, rel);
                    v = dot(e2, rel);
                    hit = !(u < R(0) || u > pickr<R>(T.e1e1, T.fe1e1) || v < R(0) || v > pickr<R>(T.e2e2, T.fe2e2));
                }
                if (hit && T.kind == MIDSX_TALLY_SURFACE_BINNED_RECT) {
                    int iu = int(u / pickr<R>(T.e1e1, T.fe1e1) * R(T.nu));
                    int iv = int(v / pickr<R>(T.e2e2, T.fe2e2) * R(T.nv));
                    iu = iu >= T.nu ? T.nu - 1 : iu;
                    iv = iv >= T.nv ? T.nv - 1 : iv;
                    acc = T.acc + (size_t(iv) * T.nu + iu) * 8 + cls0 * 2;
                    k1 = kRecBinned;
                    v1 = E;
                    ++words;
                } else if (hit) {
                    k1 = kRecSurface;
                    c = cls0;
                    v1 = E;
                    v2 = ec;
                    if (E != R(0)) ++words;
                    if (ec != R(0)) ++words;
                    ++words;
                    if constexpr (SPEC) {
                        if (T.n_energy > 0) {
                            const int kb = energy_bin<R>(T, E);
                            if (kb >= 0) {
                                unsigned long long* sp = T.acc + MIDSX_SCALAR_SLOTS + (size_t(kb) * 4 + cls0) * 2;
                                count1(sp);
                                Acc<MX>::cosine(sp + 1, ec);
                                ++words;
                            }
                        }
                    }
                }
            }
        }
        // most segments touch no tally (a detector plane is crossed once per history): the
        // warp skips the records unless a lane has one (k2 and k3 only come with k1)
        if (!__any_sync(0xffffffffu, k1 != kRecNone)) continue;
        warp_record<R, MX>(k1, acc, c, v1, v2, scratch);
        if (__any_sync(0xffffffffu, k2 != kRecNone)) warp_record<R, MX>(k2, acc, c, v2, R(0), scratch);
        if (__any_sync(0xffffffffu, k3 != kRecNone)) warp_record<R, MX>(k3, acc, c, R(0), R(0), scratch);
    }
}
