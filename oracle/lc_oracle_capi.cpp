// lc_oracle_capi.cpp — C entry points of the CPU oracle (loaded with ctypes by
// tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py).
//
// TEST INFRASTRUCTURE ONLY: the product never links or calls this library.
// See lc_oracle.hpp for what is restated and how it is pinned.
#include <omp.h>

#include <memory>

#include "lc_oracle.hpp"

using namespace lco;

struct lco_world {
    int fp64 = 0;
    std::vector<std::unique_ptr<Cloth<float>>> f32;
    std::vector<std::unique_ptr<Cloth<double>>> f64;
    int n() const { return fp64 ? (int)f64.size() : (int)f32.size(); }
};

template <class F> static int with_cloth(lco_world *w, int c, F &&fn) {
    if (!w || c < 0 || c >= w->n()) return LC_ERR_INVALID_ARG;
    if (w->fp64) return fn(*w->f64[c]);
    return fn(*w->f32[c]);
}

template <class R> static void put3(const std::vector<V3<R>> &src, double *dst) {
    if (!dst) return;
    for (size_t i = 0; i < src.size(); ++i) {
        dst[3 * i] = (double)src[i].x;
        dst[3 * i + 1] = (double)src[i].y;
        dst[3 * i + 2] = (double)src[i].z;
    }
}
template <class R> static void get3(std::vector<V3<R>> &dst, const double *src) {
    if (!src) return;
    for (size_t i = 0; i < dst.size(); ++i) dst[i] = mk<R>(R(src[3 * i]), R(src[3 * i + 1]), R(src[3 * i + 2]));
}
template <class T> static int copy_out(const T *src, uint64_t n, void *dst, uint64_t cap, uint64_t *count) {
    if (count) *count = n;
    if (dst) std::memcpy(dst, src, sizeof(T) * std::min<uint64_t>(n, cap));
    return LC_OK;
}

extern "C" {

lco_world *lco_create(const lc_cloth_desc *descs, int n, int fp64) {
    if (!descs || n <= 0) return nullptr;
    auto *w = new lco_world();
    w->fp64 = fp64 ? 1 : 0;
    for (int i = 0; i < n; ++i) {
        if (fp64) {
            w->f64.emplace_back(new Cloth<double>());
            w->f64.back()->init(descs[i]);
        } else {
            w->f32.emplace_back(new Cloth<float>());
            w->f32.back()->init(descs[i]);
        }
    }
    return w;
}

void lco_destroy(lco_world *w) { delete w; }

int lco_num_cloths(lco_world *w) { return w ? w->n() : 0; }

// nsteps FixedUpdates of every cloth; cloths run in parallel on nthreads
// host threads (0 = all).
int lco_step(lco_world *w, int nsteps, int nthreads) {
    if (!w) return LC_ERR_INVALID_ARG;
    int n = w->n();
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int c = 0; c < n; ++c) {
        for (int s = 0; s < nsteps; ++s) {
            if (w->fp64)
                w->f64[c]->step();
            else
                w->f32[c]->step();
        }
    }
    return LC_OK;
}

int lco_max_threads(void) { return omp_get_max_threads(); }

// The collision stages of every cloth on its current state (x, x_prev, v,
// triangle order), cloths in parallel on nthreads host threads (0 = all).
int lco_collide_all(lco_world *w, int nthreads) {
    if (!w) return LC_ERR_INVALID_ARG;
    int n = w->n();
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int c = 0; c < n; ++c) {
        if (w->fp64)
            w->f64[c]->collide();
        else
            w->f32[c]->collide();
    }
    return LC_OK;
}

// One teacher-forced step of every cloth, in parallel: each cloth must have
// its contacts frozen (lco_set_frozen_contacts); its collision stages are
// skipped, so its running normals and triangle order stay as set.
int lco_step_frozen_all(lco_world *w, int nthreads) {
    if (!w) return LC_ERR_INVALID_ARG;
    int n = w->n();
    for (int c = 0; c < n; ++c)
        if (!(w->fp64 ? w->f64[c]->have_frozen : w->f32[c]->have_frozen)) return LC_ERR_INVALID_ARG;
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int c = 0; c < n; ++c) {
        if (w->fp64) {
            w->f64[c]->skip_collide = true;
            w->f64[c]->step();
            w->f64[c]->skip_collide = false;
        } else {
            w->f32[c]->skip_collide = true;
            w->f32[c]->step();
            w->f32[c]->skip_collide = false;
        }
    }
    return LC_OK;
}

int lco_sizes(lco_world *w, int c, int *nv, int *nt, int *ne, int *nb) {
    return with_cloth(w, c, [&](auto &cl) {
        if (nv) *nv = cl.tp.V;
        if (nt) *nt = cl.tp.T;
        if (ne) *ne = (int)cl.tp.s1.size();
        if (nb) *nb = (int)cl.tp.b1.size();
        return LC_OK;
    });
}

int lco_get_state(lco_world *w, int c, double *x, double *xp, double *v, double *vn) {
    return with_cloth(w, c, [&](auto &cl) {
        put3(cl.x, x); put3(cl.xp, xp); put3(cl.v, v); put3(cl.vn, vn);
        return LC_OK;
    });
}

int lco_set_state(lco_world *w, int c, const double *x, const double *xp, const double *v, const double *vn) {
    return with_cloth(w, c, [&](auto &cl) {
        get3(cl.x, x); get3(cl.xp, xp); get3(cl.v, v); get3(cl.vn, vn);
        return LC_OK;
    });
}

int lco_get_perm(lco_world *w, int c, uint32_t *perm) {
    return with_cloth(w, c, [&](auto &cl) {
        std::memcpy(perm, cl.perm.data(), sizeof(uint32_t) * cl.perm.size());
        return LC_OK;
    });
}

int lco_set_perm(lco_world *w, int c, const uint32_t *perm) {
    return with_cloth(w, c, [&](auto &cl) {
        std::memcpy(cl.perm.data(), perm, sizeof(uint32_t) * cl.perm.size());
        return LC_OK;
    });
}

// Wind state (current wind vector and the variation RNG state).
int lco_get_wind(lco_world *w, int c, double wind[3], uint64_t *rng) {
    return with_cloth(w, c, [&](auto &cl) {
        wind[0] = cl.wind.x; wind[1] = cl.wind.y; wind[2] = cl.wind.z;
        if (rng) *rng = cl.rng;
        return LC_OK;
    });
}
int lco_set_wind(lco_world *w, int c, const double wind[3], uint64_t rng) {
    return with_cloth(w, c, [&](auto &cl) {
        using R = std::remove_reference_t<decltype(cl.wind.x)>;
        cl.wind = mk<R>(R(wind[0]), R(wind[1]), R(wind[2]));
        cl.rng = rng;
        return LC_OK;
    });
}

// Stage entry points for teacher-forced comparisons.
int lco_external(lco_world *w, int c) {
    return with_cloth(w, c, [&](auto &cl) { cl.external(); return LC_OK; });
}
int lco_collide(lco_world *w, int c) {
    return with_cloth(w, c, [&](auto &cl) { cl.collide(); return LC_OK; });
}
int lco_step_one(lco_world *w, int c) {
    return with_cloth(w, c, [&](auto &cl) { cl.step(); return LC_OK; });
}

// The static triangle collider of lc_batch_set_collider (cw: faces clockwise
// seen from the free side); nt = 0 removes it.
int lco_set_collider(lco_world *w, int c, const float *verts, int nv, const uint32_t *tris, int nt, int cw) {
    return with_cloth(w, c, [&](auto &cl) {
        using R = std::remove_reference_t<decltype(cl.wind.x)>;
        if (nt < 0 || nv < 0 || (nt && (!verts || !tris))) return (int)LC_ERR_INVALID_ARG;
        for (int k = 0; k < 3 * nt; ++k)
            if (tris[k] >= (uint32_t)nv) return (int)LC_ERR_INVALID_ARG;
        cl.coll_cw = cw != 0;
        cl.coll_v.resize(nt ? nv : 0);
        for (int i = 0; i < (nt ? nv : 0); ++i)
            cl.coll_v[i] = mk<R>(R(verts[3 * i]), R(verts[3 * i + 1]), R(verts[3 * i + 2]));
        cl.coll_t.assign(tris, tris + 3 * (size_t)nt);
        return (int)LC_OK;
    });
}

// The next step uses these collider contacts (lc_contact records of the
// engine's LC_DBG_COLLIDER: v[1] the triangle or -1, w the plane) instead of
// its own.
int lco_set_frozen_collider(lco_world *w, int c, const lc_contact *rec, uint64_t n) {
    return with_cloth(w, c, [&](auto &cl) {
        const int K = cl.kCollSlots;
        if (n != (uint64_t)cl.tp.V * K) return (int)LC_ERR_INVALID_ARG;
        cl.frozen_coll_tri.assign(n, -1);
        cl.frozen_coll_c.assign(n, Contact{});
        for (uint64_t i = 0; i < n; ++i) {
            cl.frozen_coll_tri[i] = rec[i].v[1];
            Contact k;
            k.v[0] = (int)(i / K); k.v[1] = k.v[2] = k.v[3] = 0;
            for (int j = 0; j < 4; ++j) k.w[j] = rec[i].w[j];
            cl.frozen_coll_c[i] = k;
        }
        cl.have_frozen_coll = true;
        return (int)LC_OK;
    });
}

// The next step of cloth c uses these contacts instead of the ones its own
// collision stage finds (contact sets frozen for position comparisons).
int lco_set_frozen_contacts(lco_world *w, int c, const lc_contact *vf, uint64_t nvf, const lc_contact *ee,
                            uint64_t nee) {
    return with_cloth(w, c, [&](auto &cl) {
        cl.frozen_vf.resize(nvf);
        cl.frozen_ee.resize(nee);
        for (uint64_t i = 0; i < nvf; ++i) std::memcpy(&cl.frozen_vf[i], &vf[i], sizeof(Contact));
        for (uint64_t i = 0; i < nee; ++i) std::memcpy(&cl.frozen_ee[i], &ee[i], sizeof(Contact));
        cl.have_frozen = true;
        return LC_OK;
    });
}

// Replays discrete decisions for the next step of cloth c (see Cloth::Forced);
// dyn holds iterations x (4 * (frozen VF + frozen EE contacts)) bytes.
int lco_set_forced(lco_world *w, int c, const uint8_t *ground, const uint32_t *ground_it, const uint8_t *lra,
                   const uint8_t *dyn, uint64_t dyn_len, const int8_t *sphere) {
    return with_cloth(w, c, [&](auto &cl) {
        const int V = cl.tp.V, F = (int)cl.tp.fixed.size();
        cl.forced.ground.assign(ground, ground + V);
        cl.forced.ground_it.assign(ground_it, ground_it + V);
        cl.forced.lra.assign(lra, lra + (size_t)V * F);
        cl.forced.dyn.assign(dyn, dyn + dyn_len);
        if (sphere) cl.forced.sphere.assign(sphere, sphere + V);
        else cl.forced.sphere.assign(V, 0);
        cl.forced.on = true;
        return LC_OK;
    });
}

int lco_set_stiffness(lco_world *w, int c, const float *ks, const float *kb) {
    return with_cloth(w, c, [&](auto &cl) {
        if (ks) for (size_t i = 0; i < cl.tp.kst.size(); ++i) cl.tp.kst[i] = ks[i];
        if (kb) for (size_t i = 0; i < cl.tp.kbd.size(); ++i) cl.tp.kbd[i] = kb[i];
        return LC_OK;
    });
}

int lco_thickness(lco_world *w, int c, float *h) {
    return with_cloth(w, c, [&](auto &cl) { *h = cl.h; return LC_OK; });
}

int lco_counters(lco_world *w, int c, uint64_t out[4]) {
    return with_cloth(w, c, [&](auto &cl) {
        out[0] = cl.pairs.size() / 2;
        out[1] = cl.vf.size();
        out[2] = cl.ee.size();
        out[3] = cl.dropped;
        if (cl.stack_overflow) return (int)LC_ERR_STACK_OVERFLOW;
        return cl.coll_overflow ? (int)LC_ERR_CAPACITY_OVERFLOW : (int)LC_OK;
    });
}

// Same selectors as lc_batch_debug_get (lc.h).
int lco_debug_get(lco_world *w, int c, int what, void *dst, uint64_t cap, uint64_t *count) {
    return with_cloth(w, c, [&](auto &cl) -> int {
        using R = std::remove_reference_t<decltype(cl.wind.x)>;
        auto f3 = [&](const std::vector<V3<R>> &src) {
            std::vector<float> tmp(3 * src.size());
            for (size_t i = 0; i < src.size(); ++i) {
                tmp[3 * i] = (float)src[i].x; tmp[3 * i + 1] = (float)src[i].y; tmp[3 * i + 2] = (float)src[i].z;
            }
            return copy_out(tmp.data(), tmp.size() / 3, dst, cap * 3, count), LC_OK;
        };
        switch (what) {
            case LC_DBG_PRED_X: return f3(cl.pred_x);
            case LC_DBG_PRED_XPREV: return f3(cl.pred_xp);
            case LC_DBG_PRED_V: return f3(cl.pred_v);
            case LC_DBG_PERM_BEFORE: return copy_out(cl.perm_before.data(), cl.perm_before.size(), dst, cap, count);
            case LC_DBG_MORTON: return copy_out(cl.morton.data(), cl.morton.size(), dst, cap, count);
            case LC_DBG_PERM: return copy_out(cl.perm.data(), cl.perm.size(), dst, cap, count);
            case LC_DBG_LEFTS: return copy_out(cl.lefts.data(), cl.lefts.size(), dst, cap, count);
            case LC_DBG_RIGHTS: return copy_out(cl.rights.data(), cl.rights.size(), dst, cap, count);
            case LC_DBG_PARENTS: return copy_out(cl.parents.data(), cl.parents.size(), dst, cap, count);
            case LC_DBG_RML: {
                std::vector<int> t(2 * cl.rmll.size());
                for (size_t i = 0; i < cl.rmll.size(); ++i) { t[2 * i] = cl.rmll[i]; t[2 * i + 1] = cl.rmlr[i]; }
                if (count) *count = cl.rmll.size();
                if (dst) std::memcpy(dst, t.data(), sizeof(int) * std::min<uint64_t>(t.size(), 2 * cap));
                return LC_OK;
            }
            case LC_DBG_NODE_AABB: {
                std::vector<float> t(6 * cl.nmin.size());
                for (size_t i = 0; i < cl.nmin.size(); ++i) {
                    t[6 * i] = (float)cl.nmin[i].x; t[6 * i + 1] = (float)cl.nmin[i].y; t[6 * i + 2] = (float)cl.nmin[i].z;
                    t[6 * i + 3] = (float)cl.nmax[i].x; t[6 * i + 4] = (float)cl.nmax[i].y; t[6 * i + 5] = (float)cl.nmax[i].z;
                }
                if (count) *count = cl.nmin.size();
                if (dst) std::memcpy(dst, t.data(), sizeof(float) * std::min<uint64_t>(t.size(), 6 * cap));
                return LC_OK;
            }
            case LC_DBG_PAIRS: {
                if (count) *count = cl.pairs.size() / 2;
                if (dst) std::memcpy(dst, cl.pairs.data(), sizeof(uint32_t) * std::min<uint64_t>(cl.pairs.size(), 2 * cap));
                return LC_OK;
            }
            case LC_DBG_VF: return copy_out(cl.vf.data(), cl.vf.size(), dst, cap, count);
            case LC_DBG_EE: return copy_out(cl.ee.data(), cl.ee.size(), dst, cap, count);
            case LC_DBG_COLLIDER: {
                const int K = cl.kCollSlots;
                const size_t n = (size_t)cl.tp.V * K;
                std::vector<Contact> out(n);
                for (size_t i = 0; i < n; ++i) {
                    Contact k{};
                    k.v[0] = (int)(i / K);
                    k.v[1] = -1;
                    if (i < cl.coll_tri.size() && cl.coll_tri[i] >= 0) {
                        k.v[1] = cl.coll_tri[i];
                        for (int j = 0; j < 4; ++j) k.w[j] = cl.coll_c[i].w[j];
                    }
                    out[i] = k;
                }
                return copy_out(out.data(), out.size(), dst, cap, count);
            }
            case LC_DBG_FEATURES: return copy_out(cl.tp.features.data(), cl.tp.features.size(), dst, cap, count);
            default: return LC_ERR_INVALID_ARG;
        }
    });
}

// Grid topology of Rendering/VisualBodyFactory.cpp:343-391.
int lco_grid_indices(int rows, int cols, uint32_t *out) {
    std::vector<u32> idx;
    grid_indices(rows, cols, idx);
    if (out) std::memcpy(out, idx.data(), idx.size() * sizeof(u32));
    return (int)(idx.size() / 3);
}

// Morton code of one point, for golden-vector checks of the encoder.
uint64_t lco_morton(float x, float y, float z, int mode) { return morton3d(x, y, z, mode); }

// The narrowphase on caller data, with full contact records: for every pair
// (triangle i, triangle j) the candidates of CreateTriangleTests
// (Collision/CudaCollisionDetection.cu:53-189) in slot order, then
//   mode 0 (CCDTriangleTests, :223-283): the feature AABB cull on the swept
//     vertex boxes of x and x_prev (Collision/FeatureList.cu:134-162,
//     Collision/CudaPrimitiveTests.cu:427-490), the sanity checks and the
//     continuous tests on x_prev and v over dt (:128-238), t = the hit's
//     coplanarity time times dt;
//   mode 1 (DCDTriangleTests, :21-94): the sanity checks and one TestVF /
//     TestEE at x_prev, t as those tests leave it (0, or the candidate's -1
//     where TestEE does not write it).
// Contacts go out as PrimitiveContact records, at most cap of each kind.
int lco_narrow_contacts(int mode, const float *x, const float *xp, const float *v, int V, const uint32_t *tris,
                        const uint8_t *feats, int T, const uint32_t *pairs, uint64_t P, float h, float dt,
                        ContactFull *vf_out, uint64_t vf_cap, uint64_t *nvf, ContactFull *ee_out, uint64_t ee_cap,
                        uint64_t *nee) {
    using Cl = Cloth<float>;
    using V3f = V3<float>;
    if (!x || !xp || !v || !tris || V < 1 || T < 1 || (P && !pairs) || (mode != 0 && mode != 1)) return LC_ERR_INVALID_ARG;
    for (int t = 0; t < 3 * T; ++t)
        if (tris[t] >= (uint32_t)V) return LC_ERR_INVALID_ARG;
    for (uint64_t q = 0; q < 2 * P; ++q)
        if (pairs[q] >= (uint32_t)T) return LC_ERR_INVALID_ARG;
    auto ld = [](const float *a, int i) { return mk<float>(a[3 * i], a[3 * i + 1], a[3 * i + 2]); };
    std::vector<V3f> pmin(V), pmax(V);
    for (int i = 0; i < V; ++i) {
        pmin[i] = subc(vmin(ld(x, i), ld(xp, i)), h);
        pmax[i] = addc(vmax(ld(x, i), ld(xp, i)), h);
    }
    uint64_t kv = 0, ke = 0;
    auto emit = [](ContactFull *out, uint64_t cap, uint64_t &k, const Contact &c, float t, V3f n) {
        if (k < cap) {
            ContactFull &o = out[k];
            for (int j = 0; j < 4; ++j) { o.v[j] = c.v[j]; o.w[j] = c.w[j]; }
            o.t = t; o.n[0] = n.x; o.n[1] = n.y; o.n[2] = n.z;
        }
        ++k;
    };
    static const int ea_v[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    static const int ea_bit[3] = {2, 0, 1};
    for (uint64_t q = 0; q < P; ++q) {
        const uint32_t ta = pairs[2 * q], tb = pairs[2 * q + 1];
        const int A[3] = {(int)tris[3 * ta], (int)tris[3 * ta + 1], (int)tris[3 * ta + 2]};
        const int B[3] = {(int)tris[3 * tb], (int)tris[3 * tb + 1], (int)tris[3 * tb + 2]};
        const uint8_t fa = feats ? feats[ta] : 0x3F, fb = feats ? feats[tb] : 0x3F;
        for (int s = 0; s < 6; ++s) {
            const int *P1 = s < 3 ? A : B, *F1 = s < 3 ? B : A;
            if (!(((s < 3 ? fa : fb) >> (5 - s % 3)) & 1)) continue;
            Contact c;
            c.v[0] = P1[s % 3]; c.v[1] = F1[0]; c.v[2] = F1[1]; c.v[3] = F1[2];
            c.w[0] = c.w[1] = c.w[2] = c.w[3] = -1.f;
            if (mode == 0) {
                V3f tmin = min3(pmin[c.v[1]], pmin[c.v[2]], pmin[c.v[3]]);
                V3f tmax = max3(pmax[c.v[1]], pmax[c.v[2]], pmax[c.v[3]]);
                if (!overlap(pmin[c.v[0]], pmax[c.v[0]], tmin, tmax)) continue;
            }
            if (c.v[0] == c.v[1] || c.v[0] == c.v[2] || c.v[0] == c.v[3]) continue;
            V3f x4 = ld(xp, c.v[0]), x1 = ld(xp, c.v[1]), x2 = ld(xp, c.v[2]), x3 = ld(xp, c.v[3]);
            V3f n = mk<float>(-1.f, -1.f, -1.f);
            if (mode == 1) {
                if (Cl::test_vf(x4, x1, x2, x3, c, h, &n)) emit(vf_out, vf_cap, kv, c, 0.f, n);
                continue;
            }
            V3f v4 = ld(v, c.v[0]), v1 = ld(v, c.v[1]), v2 = ld(v, c.v[2]), v3 = ld(v, c.v[3]);
            float times[8];
            const int nt = Cl::coplanarity_times(x1, x2, x3, x4, v1, v2, v3, v4, times);
            for (int i = 0; i < nt; ++i) {
                const float t = times[i] * dt;
                x4 = x4 + v4 * t; x1 = x1 + v1 * t; x2 = x2 + v2 * t; x3 = x3 + v3 * t;
                if (Cl::test_vf(x4, x1, x2, x3, c, h, &n)) { emit(vf_out, vf_cap, kv, c, t, n); break; }
            }
        }
        for (int s = 0; s < 9; ++s) {
            const int ia = s % 3, ib = s / 3;
            if (!(((fa >> ea_bit[ia]) & 1) & ((fb >> ea_bit[ib]) & 1))) continue;
            Contact c;
            c.v[0] = A[ea_v[ia][0]]; c.v[1] = A[ea_v[ia][1]];
            c.v[2] = B[ea_v[ib][0]]; c.v[3] = B[ea_v[ib][1]];
            c.w[0] = c.w[1] = c.w[2] = c.w[3] = -1.f;
            if (mode == 0) {
                V3f e1min = vmin(pmin[c.v[0]], pmin[c.v[1]]), e1max = vmax(pmax[c.v[0]], pmax[c.v[1]]);
                V3f e2min = vmin(pmin[c.v[2]], pmin[c.v[3]]), e2max = vmax(pmax[c.v[2]], pmax[c.v[3]]);
                if (!overlap(e1min, e1max, e2min, e2max)) continue;
            }
            if (c.v[0] == c.v[2] || c.v[0] == c.v[3] || c.v[1] == c.v[2] || c.v[1] == c.v[3]) continue;
            V3f x1 = ld(xp, c.v[0]), x2 = ld(xp, c.v[1]), x3 = ld(xp, c.v[2]), x4 = ld(xp, c.v[3]);
            V3f n = mk<float>(-1.f, -1.f, -1.f);
            if (mode == 1) {
                float t = -1.f;
                if (Cl::test_ee(x1, x2, x3, x4, c, h, &n, &t)) emit(ee_out, ee_cap, ke, c, t, n);
                continue;
            }
            V3f v1 = ld(v, c.v[0]), v2 = ld(v, c.v[1]), v3 = ld(v, c.v[2]), v4 = ld(v, c.v[3]);
            float times[8];
            const int nt = Cl::coplanarity_times(x1, x2, x3, x4, v1, v2, v3, v4, times);
            for (int i = 0; i < nt; ++i) {
                const float t = times[i] * dt;
                x1 = x1 + v1 * t; x2 = x2 + v2 * t; x3 = x3 + v3 * t; x4 = x4 + v4 * t;
                if (Cl::test_ee(x1, x2, x3, x4, c, h, &n)) { emit(ee_out, ee_cap, ke, c, t, n); break; }
            }
        }
    }
    if (nvf) *nvf = kv;
    if (nee) *nee = ke;
    return LC_OK;
}

// CudaDeformableBody::SolveCollisions on caller data (lco::solve_collisions):
// x (out), x_prev, v (in/out) 3 floats per vertex, fixed flags, contacts as
// PrimitiveContact records (12 words each).
int lco_solve_collisions(float *x, const float *xp, float *v, const uint8_t *fixed, int V, const ContactFull *vf,
                         uint64_t nvf, const ContactFull *ee, uint64_t nee, float stiffness, float mass, float dt,
                         float h) {
    if (!x || !xp || !v || !fixed || V < 1 || (nvf && !vf) || (nee && !ee)) return LC_ERR_INVALID_ARG;
    std::vector<V3<float>> X(V), XP(V), VV(V);
    for (int i = 0; i < V; ++i) {
        X[i] = mk<float>(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        XP[i] = mk<float>(xp[3 * i], xp[3 * i + 1], xp[3 * i + 2]);
        VV[i] = mk<float>(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    }
    std::vector<u8> F(fixed, fixed + V);
    std::vector<ContactFull> A(vf, vf + nvf), B(ee, ee + nee);
    for (const auto *L : {&A, &B})
        for (const auto &c : *L)
            for (int k = 0; k < 4; ++k)
                if (c.v[k] < 0 || c.v[k] >= V) return LC_ERR_INVALID_ARG;
    solve_collisions(X, XP, VV, F, A, B, stiffness, mass, dt, h);
    for (int i = 0; i < V; ++i) {
        x[3 * i] = X[i].x; x[3 * i + 1] = X[i].y; x[3 * i + 2] = X[i].z;
        v[3 * i] = VV[i].x; v[3 * i + 1] = VV[i].y; v[3 * i + 2] = VV[i].z;
    }
    return LC_OK;
}

// The LBVH chain over caller boxes that the engine's standalone entry points
// (lc_lbvh_build + lc_lbvh_pairs) run: Morton code of each box's midpoint
// min + (max - min) / 2 (identity frame, Core/CudaUtils.cu:278-325), a stable
// sort by code, the leaves' boxes gathered in the sorted order, the Karras
// hierarchy, the refit and the traversal with at most `chunk` pairs per leaf
// (Collision/CudaBVH.cu:23-188), through the restatement's FP32 code.
// Outputs (any may be NULL): sorted codes and order (T), lefts / rights
// (T-1), parents (2T-1; the root's entry -1), rightmost leaves (2 per
// internal node), node boxes (6 floats per node), pairs (2 u32 each, at most
// pair_cap) with their count.
int lco_lbvh_boxes(const float *bmin, const float *bmax, int T, int chunk, int mode, uint64_t *morton_out,
                   uint32_t *perm_out, int *lefts_out, int *rights_out, int *parents_out, int *rml_out,
                   float *node_out, uint32_t *pairs_out, uint64_t pair_cap, uint64_t *npairs) {
    if (!bmin || !bmax || T < 2 || chunk < 1 || (mode != LC_MORTON_REF63 && mode != LC_MORTON_K30))
        return LC_ERR_INVALID_ARG;
    Cloth<float> cl;
    cl.tp.T = T;
    cl.prm.BVHChunkSize = chunk;
    std::vector<u64> keys(T);
    for (int s = 0; s < T; ++s) {
        V3<float> mn = mk<float>(bmin[3 * s], bmin[3 * s + 1], bmin[3 * s + 2]);
        V3<float> mx = mk<float>(bmax[3 * s], bmax[3 * s + 1], bmax[3 * s + 2]);
        V3<float> mid = mn + (mx - mn) / 2.f;
        keys[s] = morton3d(mid.x, mid.y, mid.z, mode);
    }
    std::vector<u32> order(T);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](u32 a, u32 b) { return keys[a] < keys[b]; });
    const int nodes = 2 * T - 1;
    cl.nmin.assign(nodes, mk<float>(0, 0, 0));
    cl.nmax.assign(nodes, mk<float>(0, 0, 0));
    cl.morton.resize(T);
    for (int s = 0; s < T; ++s) {
        const u32 o = order[s];
        cl.morton[s] = keys[o];
        cl.nmin[T - 1 + s] = mk<float>(bmin[3 * o], bmin[3 * o + 1], bmin[3 * o + 2]);
        cl.nmax[T - 1 + s] = mk<float>(bmax[3 * o], bmax[3 * o + 1], bmax[3 * o + 2]);
    }
    cl.build_tree();
    cl.refit();
    cl.traverse();
    if (morton_out) std::memcpy(morton_out, cl.morton.data(), sizeof(u64) * T);
    if (perm_out) std::memcpy(perm_out, order.data(), sizeof(u32) * T);
    if (lefts_out) std::memcpy(lefts_out, cl.lefts.data(), sizeof(int) * (T - 1));
    if (rights_out) std::memcpy(rights_out, cl.rights.data(), sizeof(int) * (T - 1));
    if (parents_out) std::memcpy(parents_out, cl.parents.data(), sizeof(int) * nodes);
    if (rml_out)
        for (int i = 0; i < T - 1; ++i) { rml_out[2 * i] = cl.rmll[i]; rml_out[2 * i + 1] = cl.rmlr[i]; }
    if (node_out)
        for (int i = 0; i < nodes; ++i) {
            float *o = node_out + 6 * i;
            o[0] = cl.nmin[i].x; o[1] = cl.nmin[i].y; o[2] = cl.nmin[i].z;
            o[3] = cl.nmax[i].x; o[4] = cl.nmax[i].y; o[5] = cl.nmax[i].z;
        }
    const uint64_t np = cl.pairs.size() / 2;
    if (npairs) *npairs = np;
    if (pairs_out) std::memcpy(pairs_out, cl.pairs.data(), sizeof(u32) * 2 * std::min(np, pair_cap));
    return cl.stack_overflow ? LC_ERR_STACK_OVERFLOW : LC_OK;
}

}  // extern "C"

// ---- adjoint of the step (FP64 oracle) -------------------------------------
// Steps cloth c nsteps times, recording after each step its decisions and the
// intermediate states its adjoint needs (Cloth::Record).
extern "C" int lco_adj_record(lco_world *w, int c, int nsteps) {
    return with_cloth(w, c, [&](auto &cl) {
        for (int s = 0; s < nsteps; ++s) {
            cl.recording = true;
            cl.step();
            cl.recording = false;
            cl.records.push_back(cl.rec);
        }
        return LC_OK;
    });
}

// Steps cloth c nsteps times with the decisions recorded for steps
// [first, first + nsteps) imposed (the piecewise-smooth branch a finite
// difference of the recorded rollout has to stay on).
extern "C" int lco_adj_replay(lco_world *w, int c, int first, int nsteps) {
    return with_cloth(w, c, [&](auto &cl) {
        if (first < 0 || first + nsteps > (int)cl.records.size()) return (int)LC_ERR_INVALID_ARG;
        for (int s = 0; s < nsteps; ++s) {
            const auto &r = cl.records[first + s];
            cl.frozen_vf = r.vf;
            cl.frozen_ee = r.ee;
            cl.have_frozen = true;
            cl.forced.ground = r.ground;
            cl.forced.ground_it = r.ground_it;
            cl.forced.lra = r.lra;
            cl.forced.dyn = r.dyn;
            cl.forced.sphere.assign(cl.tp.V, 0);
            cl.forced.on = true;
            if (!r.coll_tri.empty()) {
                cl.frozen_coll_tri = r.coll_tri;
                cl.frozen_coll_c = r.coll_c;
                cl.have_frozen_coll = true;
            }
            cl.step();
        }
        return (int)LC_OK;
    });
}

// Reverse pass over every recorded step, last first.  gx, gxp, gv (3V
// doubles each) hold dL/d(x, x_prev, v) after the last recorded step and
// receive the gradients before the first; gks (stretch count) and gkb (bend
// count) accumulate dL/dk.
extern "C" int lco_adj_backward(lco_world *w, int c, double *gx, double *gxp, double *gv, double *gks,
                                double *gkb) {
    return with_cloth(w, c, [&](auto &cl) {
        using Cl = std::remove_reference_t<decltype(cl)>;
        using V = typename Cl::V;
        using R = std::remove_reference_t<decltype(cl.wind.x)>;
        const int Vn = cl.tp.V;
        std::vector<V> ax(Vn), axp(Vn), av(Vn);
        for (int i = 0; i < Vn; ++i) {
            ax[i] = mk<R>(R(gx[3 * i]), R(gx[3 * i + 1]), R(gx[3 * i + 2]));
            axp[i] = mk<R>(R(gxp[3 * i]), R(gxp[3 * i + 1]), R(gxp[3 * i + 2]));
            av[i] = mk<R>(R(gv[3 * i]), R(gv[3 * i + 1]), R(gv[3 * i + 2]));
        }
        if (cl.tp.tri_bend) return (int)LC_ERR_NOT_SUPPORTED;  // triangle bending is not differentiated
        std::vector<double> ks(cl.tp.s1.size(), 0.0), kb(cl.tp.b1.size(), 0.0);
        for (int s = (int)cl.records.size() - 1; s >= 0; --s) cl.backward(cl.records[s], ax, axp, av, ks, kb);
        for (int i = 0; i < Vn; ++i) {
            gx[3 * i] = ax[i].x; gx[3 * i + 1] = ax[i].y; gx[3 * i + 2] = ax[i].z;
            gxp[3 * i] = axp[i].x; gxp[3 * i + 1] = axp[i].y; gxp[3 * i + 2] = axp[i].z;
            gv[3 * i] = av[i].x; gv[3 * i + 1] = av[i].y; gv[3 * i + 2] = av[i].z;
        }
        for (size_t i = 0; i < ks.size(); ++i) gks[i] += ks[i];
        for (size_t i = 0; i < kb.size(); ++i) gkb[i] += kb[i];
        return (int)LC_OK;
    });
}

extern "C" int lco_adj_clear(lco_world *w, int c) {
    return with_cloth(w, c, [&](auto &cl) { cl.records.clear(); return (int)LC_OK; });
}

// Per-constraint stiffness in double (finite differences need more than float).
extern "C" int lco_set_stiffness_d(lco_world *w, int c, const double *ks, const double *kb) {
    return with_cloth(w, c, [&](auto &cl) {
        if (ks) for (size_t i = 0; i < cl.tp.kst.size(); ++i) cl.tp.kst[i] = ks[i];
        if (kb) for (size_t i = 0; i < cl.tp.kbd.size(); ++i) cl.tp.kbd[i] = kb[i];
        return (int)LC_OK;
    });
}

// ---- solver pin -------------------------------------------------------------
// The static topology of cloth c in the layouts the reference's solver kernels
// take (Physics/CudaPBD.cu:942-962, :1571-1592, :1656-1688): stretch ends s12
// (2E), rest lengths sl0 (E), bend vertices b (4B), the per-vertex slot CSR
// soff (V+1) with its entries sent (S, kind<<30 | role<<28 | constraint),
// pinned ids fixed (F), attachment lengths lra_l0 (V*F), inverse masses invm
// (V) and pinned flags (V).  counts receives {F, S}; any output may be null.
extern "C" int lco_topology(lco_world *w, int c, int *s12, double *sl0, int *b, int *soff, int *sent, int *fixed,
                            double *lra_l0, float *invm, uint8_t *pinned, int counts[2]) {
    return with_cloth(w, c, [&](auto &cl) {
        const auto &tp = cl.tp;
        const size_t E = tp.s1.size(), B = tp.b1.size();
        if (counts) { counts[0] = (int)tp.fixed.size(); counts[1] = (int)tp.sent.size(); }
        if (s12) for (size_t i = 0; i < E; ++i) { s12[2 * i] = tp.s1[i]; s12[2 * i + 1] = tp.s2[i]; }
        if (sl0) std::copy(tp.sl0.begin(), tp.sl0.end(), sl0);
        if (b)
            for (size_t i = 0; i < B; ++i) {
                b[4 * i] = tp.b1[i]; b[4 * i + 1] = tp.b2[i]; b[4 * i + 2] = tp.b3[i]; b[4 * i + 3] = tp.b4[i];
            }
        if (soff) std::copy(tp.soff.begin(), tp.soff.end(), soff);
        if (sent) std::copy(tp.sent.begin(), tp.sent.end(), sent);
        if (fixed) std::copy(tp.fixed.begin(), tp.fixed.end(), fixed);
        if (lra_l0) std::copy(tp.lra_l0.begin(), tp.lra_l0.end(), lra_l0);
        if (invm) for (int i = 0; i < tp.V; ++i) invm[i] = (float)cl.invm[i];
        if (pinned) std::copy(tp.pinned.begin(), tp.pinned.end(), pinned);
        return (int)LC_OK;
    });
}

// PBDStepSolver and the velocity update of _FinalUpdate (Physics/CudaPBD.cu:
// 632-660, :1916-1932) on a given state: x (predicted positions) and xp
// (previous positions), 3V floats each, with the given contacts.  x_out
// receives the positions after the solver iterations, v_out and xp_out the
// velocities and previous positions after the update (no world clamp).
// Decisions set by lco_set_forced beforehand are imposed; the decisions the
// solve took are kept for lco_solve_decisions.
extern "C" int lco_solve_on(lco_world *w, int c, const float *x, const float *xp, const lc_contact *vf,
                            uint64_t nvf, const lc_contact *ee, uint64_t nee, float *x_out, float *v_out,
                            float *xp_out) {
    return with_cloth(w, c, [&](auto &cl) {
        using R = std::remove_reference_t<decltype(cl.wind.x)>;
        const int Vn = cl.tp.V;
        for (int i = 0; i < Vn; ++i) {
            cl.x[i] = mk<R>(R(x[3 * i]), R(x[3 * i + 1]), R(x[3 * i + 2]));
            cl.xp[i] = mk<R>(R(xp[3 * i]), R(xp[3 * i + 1]), R(xp[3 * i + 2]));
        }
        std::vector<Contact> cvf(nvf), cee(nee);
        for (uint64_t i = 0; i < nvf; ++i) std::memcpy(&cvf[i], &vf[i], sizeof(Contact));
        for (uint64_t i = 0; i < nee; ++i) std::memcpy(&cee[i], &ee[i], sizeof(Contact));
        if (cl.forced.on && cl.forced.dyn.size() != (size_t)cl.prm.solverIterations * 4 * (nvf + nee)) {
            cl.forced.on = false;
            return (int)LC_ERR_INVALID_ARG;
        }
        cl.recording = true;
        cl.solve(cvf, cee);
        cl.recording = false;
        cl.forced.on = false;
        if (!cl.prm.sphereOn) cl.rec.sphere.assign(Vn, 0);
        const R dt = R(cl.prm.timestep);
        for (int i = 0; i < Vn; ++i) {
            const auto p = cl.x[i];
            x_out[3 * i] = (float)p.x; x_out[3 * i + 1] = (float)p.y; x_out[3 * i + 2] = (float)p.z;
            auto vel = cl.tp.pinned[i] ? mk<R>(0, 0, 0) : (p - cl.xp[i]) / dt;
            auto q = cl.tp.pinned[i] ? cl.xp[i] : p;
            v_out[3 * i] = (float)vel.x; v_out[3 * i + 1] = (float)vel.y; v_out[3 * i + 2] = (float)vel.z;
            xp_out[3 * i] = (float)q.x; xp_out[3 * i + 1] = (float)q.y; xp_out[3 * i + 2] = (float)q.z;
        }
        return (int)LC_OK;
    });
}

// The discrete decisions of the last lco_solve_on, in the layouts of
// lco_set_forced: ground (V), ground_it (V), lra (V*F), dyn (iterations x
// 4 x (VF + EE contacts); dyn_cap bytes at most, *dyn_len receives the full
// length), sphere (V).  Any output may be null.
extern "C" int lco_solve_decisions(lco_world *w, int c, uint8_t *ground, uint32_t *ground_it, uint8_t *lra,
                                   uint8_t *dyn, uint64_t dyn_cap, uint64_t *dyn_len, int8_t *sphere) {
    return with_cloth(w, c, [&](auto &cl) {
        const auto &r = cl.rec;
        if (dyn_len) *dyn_len = r.dyn.size();
        if (ground) std::copy(r.ground.begin(), r.ground.end(), ground);
        if (ground_it) std::copy(r.ground_it.begin(), r.ground_it.end(), ground_it);
        if (lra) std::copy(r.lra.begin(), r.lra.end(), lra);
        if (dyn) std::memcpy(dyn, r.dyn.data(), std::min<uint64_t>(dyn_cap, r.dyn.size()));
        if (sphere) std::copy(r.sphere.begin(), r.sphere.end(), sphere);
        return (int)LC_OK;
    });
}

// The positions after iteration k (0 = before the first) of the last
// lco_solve_on, 3V floats.
extern "C" int lco_solve_iterate(lco_world *w, int c, int k, float *x) {
    return with_cloth(w, c, [&](auto &cl) {
        if (k < 0 || k >= (int)cl.rec.xk.size()) return (int)LC_ERR_INVALID_ARG;
        const auto &xs = cl.rec.xk[k];
        for (size_t i = 0; i < xs.size(); ++i) {
            x[3 * i] = (float)xs[i].x; x[3 * i + 1] = (float)xs[i].y; x[3 * i + 2] = (float)xs[i].z;
        }
        return (int)LC_OK;
    });
}

// CudaPBD::ApplyFriction (Cloth::friction) on given velocities v (3V floats),
// ground-constraint flags (V bytes), VF contacts and their face normals
// (3 floats each); v_out receives the velocities after it.
extern "C" int lco_friction_on(lco_world *w, int c, const float *v, const uint8_t *ground, const lc_contact *vf,
                               const float *normals, uint64_t nvf, float *v_out) {
    return with_cloth(w, c, [&](auto &cl) {
        using R = std::remove_reference_t<decltype(cl.wind.x)>;
        using Vt = typename std::remove_reference_t<decltype(cl)>::V;
        const int Vn = cl.tp.V;
        for (int i = 0; i < Vn; ++i) cl.v[i] = mk<R>(R(v[3 * i]), R(v[3 * i + 1]), R(v[3 * i + 2]));
        cl.ground_flag.assign(ground, ground + Vn);
        std::vector<Contact> cvf(nvf);
        std::vector<Vt> nrm(nvf);
        for (uint64_t k = 0; k < nvf; ++k) {
            std::memcpy(&cvf[k], &vf[k], sizeof(Contact));
            for (int s = 0; s < 4; ++s)
                if (cvf[k].v[s] < 0 || cvf[k].v[s] >= Vn) return (int)LC_ERR_INVALID_ARG;
            nrm[k] = mk<R>(R(normals[3 * k]), R(normals[3 * k + 1]), R(normals[3 * k + 2]));
        }
        cl.friction(cvf, nrm);
        for (int i = 0; i < Vn; ++i) {
            v_out[3 * i] = (float)cl.v[i].x; v_out[3 * i + 1] = (float)cl.v[i].y; v_out[3 * i + 2] = (float)cl.v[i].z;
        }
        return (int)LC_OK;
    });
}

// Face normals (3 floats each) of the contacts given to lco_set_frozen_contacts,
// so that the next step's friction runs on them.
extern "C" int lco_set_frozen_normals(lco_world *w, int c, const float *n, uint64_t count) {
    return with_cloth(w, c, [&](auto &cl) {
        using R = std::remove_reference_t<decltype(cl.wind.x)>;
        cl.frozen_vf_n.resize(count);
        for (uint64_t k = 0; k < count; ++k) cl.frozen_vf_n[k] = mk<R>(R(n[3 * k]), R(n[3 * k + 1]), R(n[3 * k + 2]));
        return (int)LC_OK;
    });
}

// Bend conditioning of the next solves of cloth c (on != 0 to track it) and
// its value for the last one: min over bends and iterates of 1 - n1.n2.
extern "C" int lco_track_bend(lco_world *w, int c, int on) {
    return with_cloth(w, c, [&](auto &cl) { cl.track_bend = on != 0; return (int)LC_OK; });
}
// out[0] = smallest 1 - n1.n2, out[1] = smallest 1 + n1.n2 (Cloth::bend_min),
// out[2] = smallest |n| / h over the contacts (Cloth::contact_min).
extern "C" int lco_bend_conditioning(lco_world *w, int c, double *out) {
    return with_cloth(w, c, [&](auto &cl) {
        out[0] = cl.bend_min;
        out[1] = cl.bend_min_neg;
        out[2] = cl.contact_min;
        return (int)LC_OK;
    });
}

// Triangle bending: *is_tri = 1 when the cloth's bends are triangle bends
// (then lco_topology's b rows are (b0, b1, v, -1)) and h0 receives their rest
// heights (one per bend).
extern "C" int lco_tri_bends(lco_world *w, int c, int *is_tri, double *h0) {
    return with_cloth(w, c, [&](auto &cl) {
        if (is_tri) *is_tri = cl.tp.tri_bend ? 1 : 0;
        if (h0) std::copy(cl.tp.th0.begin(), cl.tp.th0.end(), h0);
        return (int)LC_OK;
    });
}
