// Host check of the per-bond arithmetic of the template path
// (pd_gpu1_gb300/csrc/bondtpl.h) against quadruple precision: the 2-D bond
// (bond2, exceeds) and the 3-D stretch (stretch3).
//
// Bonds of regular lattices (dx from 5e-5 to 1e-3, horizon 3.015 dx, the
// plate coordinates (i + 1/2) dx - L/2 of the reference's generators) under
// displacement fields with bond strains from 1e-7 to 5e-2: the bond vector d
// with the reference's FP64 roundings, the offset class of the lattice offset
// (its float reference vector from one row, its reference length the smallest
// of the class), and the force and extension of bond2() against
//   e = |d| - l0 and f = k2 e d / (2 |d|)  in __float128.
// Prints the worst errors per strain decade, relative to the field's strain
// scale (strain l0 for the extension, k2/2 strain l0 for the force, or the
// bond's own values where larger), and fails above 2e-13 (measured: about
// 5e-14 at every strain from 1e-6 up, 9e-14 at 1e-7).
// The break decision of exceeds() is checked against the double test
// fl(e.h + e.l) > fl(s0 l0) on extensions placed around the threshold.
// The ADR damping term (damping_term) is checked against the exact value of
// the reference's formula -u^2 (F/m - F_old/m) / (dt vh) on random operands
// over the magnitudes ADR meets (including F close to F_old and divisors
// outside the reciprocal path's range), and fails above 8 units of 2^-53.
#include <quadmath.h>

#include <array>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "bondtpl.h"

using namespace pdg::bt;
typedef __float128 q;

static q qabs(q v) { return v < 0 ? -v : v; }

struct Class {
    int ox, oy;
    bool set = false;
    Tpl T;
};

// The offset class of one lattice offset, as the set-up builds it: xf the
// float reference vector of a representative row, l0t the class's smallest l0.
static void make_tpl(Tpl& T, const double xa[2], double l0t) {
    for (int a = 0; a < 2; a++) {
        T.xf[a] = (float)xa[a];
        T.xd[a] = dbits((double)T.xf[a]);
    }
    // |xf|^2 and |xf|^2 - l0t^2 exactly in quad, then as pairs
    q s = (q)T.xf[0] * (q)T.xf[0] + (q)T.xf[1] * (q)T.xf[1];
    q c = s - (q)l0t * (q)l0t;
    double sh = (double)s, ch = (double)c;
    f2 sp = split_bits(sh), cp = split_bits(ch);
    // pairs carry the first 48 bits; add the remainder of the quad value to l
    sp.l = (float)((q)sp.l + (s - (q)sh));
    cp.l = (float)((q)cp.l + (c - (q)ch));
    T.q0h = sp.h, T.q0l = sp.l, T.c0h = cp.h, T.c0l = cp.l;
    const f2 lp = split_bits(l0t);
    T.l0h = lp.h, T.l0l = lp.l;
    T.l0d = l0t;
}

// The 3-D class template from a representative reference vector and l0t.
static void make_tpl3(Tpl3& T, const double xa[3], double l0t) {
    q sq = 0;
    for (int a = 0; a < 3; a++) {
        T.xf[a] = (float)xa[a];
        T.xd[a] = dbits((double)T.xf[a]);
        sq += (q)T.xf[a] * (q)T.xf[a];
    }
    const q c = sq - (q)l0t * (q)l0t;
    double sh = (double)sq, ch = (double)c;
    f2 sp = split_bits(sh), cp = split_bits(ch);
    sp.l = (float)((q)sp.l + (sq - (q)sh));
    cp.l = (float)((q)cp.l + (c - (q)ch));
    T.q0h = sp.h, T.q0l = sp.l, T.c0h = cp.h, T.c0l = cp.l;
    const f2 lp = split_bits(l0t);
    T.l0h = lp.h, T.l0l = lp.l;
    T.l0d = l0t;
}

// stretch3 on the bonds of a 3-D lattice (the offsets within 3.015 spacings,
// coordinates i dx - L/2 per axis), the force direction w = xf + eta, 1/L and
// e against __float128, relative to the field's strain scale.
static bool check3(std::mt19937_64& rng, double& worst_e, double& worst_f) {
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    const double dxs[] = {1e-3, 2e-3};
    const double strains[] = {1e-6, 1e-4, 1e-2};
    worst_e = worst_f = 0.0;
    for (double dx : dxs) {
        const int n = 60;
        const double L = n * dx, delta = 3.015 * dx;
        std::vector<std::array<int, 3>> offs;
        for (int oz = -3; oz <= 3; oz++)
            for (int oy = -3; oy <= 3; oy++)
                for (int ox = -3; ox <= 3; ox++)
                    if ((ox || oy || oz) &&
                        (ox * dx) * (ox * dx) + (oy * dx) * (oy * dx) + (oz * dx) * (oz * dx) < delta * delta)
                        offs.push_back({ox, oy, oz});
        auto coord = [&](int i) { return i * dx - L / 2.0; };
        for (double strain : strains) {
            const int rows = 1500;
            std::vector<std::array<int, 3>> rr(rows);
            for (auto& v : rr)
                for (int a = 0; a < 3; a++) v[a] = 3 + (int)(rng() % (n - 6));
            std::vector<double> l0min(offs.size(), 1e300);
            std::vector<std::array<double, 3>> rep(offs.size());
            for (size_t o = 0; o < offs.size(); o++)
                for (int k = 0; k < rows; k++) {
                    double xa[3], l2 = 0.0;
                    for (int a = 0; a < 3; a++) {
                        xa[a] = coord(rr[k][a] + offs[o][a]) - coord(rr[k][a]);
                        l2 += xa[a] * xa[a];
                    }
                    const double l0 = std::sqrt(l2);
                    if (k == 0) rep[o] = {xa[0], xa[1], xa[2]};
                    if (l0 < l0min[o]) l0min[o] = l0;
                }
            std::vector<Tpl3> tpl(offs.size());
            for (size_t o = 0; o < offs.size(); o++) make_tpl3(tpl[o], rep[o].data(), l0min[o]);
            for (int k = 0; k < rows; k++) {
                double g[3][3];
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) g[a][b] = strain * U(rng);
                for (size_t o = 0; o < offs.size(); o++) {
                    double xi[3], xc[3], ui[3], uc[3], xa[3], l2 = 0.0;
                    for (int a = 0; a < 3; a++) {
                        xi[a] = coord(rr[k][a]);
                        xc[a] = coord(rr[k][a] + offs[o][a]);
                    }
                    for (int a = 0; a < 3; a++) {
                        ui[a] = g[a][0] * xi[0] + g[a][1] * xi[1] + g[a][2] * xi[2] + 0.1 * strain * dx * U(rng);
                        uc[a] = g[a][0] * xc[0] + g[a][1] * xc[1] + g[a][2] * xc[2] + 0.1 * strain * dx * U(rng);
                        xa[a] = xc[a] - xi[a];
                        l2 += xa[a] * xa[a];
                    }
                    const double l0 = std::sqrt(l2);
                    const Tpl3& T = tpl[o];
                    const double dlv = l0 - T.l0d;
                    const float dl = (float)dlv;
                    if ((double)dl != dlv) {
                        std::printf("3-D: dl not a float: %g\n", dlv);
                        return false;
                    }
                    double d[3];
                    f2 eta[3];
                    for (int a = 0; a < 3; a++) {
                        d[a] = ((xc[a] + uc[a]) - xi[a]) - ui[a];
                        if (T.xd[a] == 0)
                            eta[a] = split_bits(d[a]);
                        else if (!offset_pair(d[a], T.xd[a], eta[a]))
                            eta[a] = split_bits(d[a] - dfrom(T.xd[a]));
                    }
                    f2 w[3], y, e;
                    stretch3(eta, T, dl, w, y, e);
                    const q Lq = sqrtq((q)d[0] * (q)d[0] + (q)d[1] * (q)d[1] + (q)d[2] * (q)d[2]);
                    const q eq = Lq - (q)l0;
                    const q escale = qabs(eq) > (q)(strain * l0) ? qabs(eq) : (q)(strain * l0);
                    const double re = (double)(qabs((q)e.h + (q)e.l - eq) / escale);
                    // the force direction w / L against d / L
                    q fd = 0;
                    for (int a = 0; a < 3; a++) {
                        const q got = ((q)w[a].h + (q)w[a].l) * ((q)y.h + (q)y.l);
                        const q want = (q)d[a] / Lq;
                        fd += (got - want) * (got - want);
                    }
                    // the force's error relative to its strain-scale magnitude: e times the
                    // direction error, plus the extension error (already in re)
                    const double rf = (double)(sqrtq(fd) * qabs(eq) / escale);
                    if (re > worst_e) worst_e = re;
                    if (rf > worst_f) worst_f = rf;
                }
            }
        }
    }
    return true;
}

int main() {
    std::mt19937_64 rng(2024);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    const double dxs[] = {5e-5, 1e-4, 5e-4, 1e-3};
    const double strains[] = {1e-7, 1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 5e-2};
    double worst_e = 0.0, worst_f = 0.0;
    long n = 0, fallbacks = 0;
    for (double dx : dxs) {
        const int nx = 400, ny = 160;
        const double Lx = nx * dx, Ly = ny * dx;
        const double delta = 3.015 * dx;
        // lattice offsets of the 2-D family
        std::vector<std::pair<int, int>> offs;
        for (int oy = -3; oy <= 3; oy++)
            for (int ox = -3; ox <= 3; ox++)
                if ((ox || oy) && (ox * dx) * (ox * dx) + (oy * dx) * (oy * dx) < delta * delta) offs.push_back({ox, oy});
        for (double strain : strains) {
            double we = 0.0, wf = 0.0;
            // classes: representative xf from row (0, 0) of this strain level's lattice
            std::vector<Class> cls(offs.size());
            std::vector<double> l0min(offs.size(), 1e300);
            auto coord = [&](int i, double L) { return (i + 0.5) * dx - L / 2.0; };
            // first pass: smallest l0 per class over the rows sampled below
            const int rows = 4000;
            std::vector<int> rx(rows), ry(rows);
            for (int k = 0; k < rows; k++) {
                rx[k] = 3 + (int)(rng() % (nx - 6));
                ry[k] = 3 + (int)(rng() % (ny - 6));
            }
            for (size_t o = 0; o < offs.size(); o++)
                for (int k = 0; k < rows; k++) {
                    const double xi = coord(rx[k], Lx), yi = coord(ry[k], Ly);
                    const double xc = coord(rx[k] + offs[o].first, Lx), yc = coord(ry[k] + offs[o].second, Ly);
                    const double xa = xc - xi, ya = yc - yi;
                    const double l0 = std::sqrt(xa * xa + ya * ya);
                    if (l0 < l0min[o]) l0min[o] = l0;
                    if (!cls[o].set) {
                        const double xv[2] = {xa, ya};
                        cls[o].set = true;
                        cls[o].T.xf[0] = (float)xa;  // placeholder, finished below
                        cls[o].T.xd[0] = dbits(xa);
                        cls[o].T.xd[1] = dbits(ya);
                        (void)xv;
                    }
                }
            for (size_t o = 0; o < offs.size(); o++) {
                const double xv[2] = {dfrom(cls[o].T.xd[0]), dfrom(cls[o].T.xd[1])};
                make_tpl(cls[o].T, xv, l0min[o]);
            }
            for (int k = 0; k < rows; k++) {
                const double xi = coord(rx[k], Lx), yi = coord(ry[k], Ly);
                // smooth field of the given strain plus a rough part of 10 %
                const double gx = strain * U(rng), gy = strain * U(rng), gs = strain * U(rng);
                auto disp = [&](double x, double y, double& ux, double& uy) {
                    ux = gx * x + gs * y;
                    uy = gs * x + gy * y;
                };
                double uxi, uyi;
                disp(xi, yi, uxi, uyi);
                uxi += 0.1 * strain * dx * U(rng);
                uyi += 0.1 * strain * dx * U(rng);
                for (size_t o = 0; o < offs.size(); o++) {
                    const double xc = coord(rx[k] + offs[o].first, Lx), yc = coord(ry[k] + offs[o].second, Ly);
                    double uxc, uyc;
                    disp(xc, yc, uxc, uyc);
                    uxc += 0.1 * strain * dx * U(rng);
                    uyc += 0.1 * strain * dx * U(rng);
                    const double xa = xc - xi, ya = yc - yi;
                    const double l0 = std::sqrt(xa * xa + ya * ya);
                    const Tpl& T = cls[o].T;
                    const double dlv = l0 - T.l0d;
                    const float dl = (float)dlv;
                    if ((double)dl != dlv) {
                        std::printf("dl not a float: %g\n", dlv);
                        return 1;
                    }
                    // the reference's roundings: P_c = x_c + u_c, d = (P_c - x_i) - u_i
                    const double pcx = xc + uxc, pcy = yc + uyc;
                    const double d[2] = {(pcx - xi) - uxi, (pcy - yi) - uyi};
                    f2 eta[2];
                    for (int a = 0; a < 2; a++) {
                        if (T.xd[a] == 0)
                            eta[a] = split_bits(d[a]);
                        else if (!offset_pair(d[a], T.xd[a], eta[a])) {
                            fallbacks++;
                            eta[a] = split_bits(d[a] - dfrom(T.xd[a]));
                        }
                    }
                    const double k2 = 2.0 * 0.87 * (1.0 + 1e-3 * U(rng)) / l0;  // k2 of some magnitude
                    const f2 k2half = split_bits(0.5 * k2);
                    const BondOut out = bond2(eta, T, dl, k2half);
                    // exact values
                    const q L = sqrtq((q)d[0] * (q)d[0] + (q)d[1] * (q)d[1]);
                    const q e = L - (q)l0;
                    const q kh = (q)k2half.h + (q)k2half.l;
                    const q fx = kh * e * (q)d[0] / L, fy = kh * e * (q)d[1] / L;
                    // errors relative to the field's strain scale (a bond whose stretch
                    // nearly vanishes, e.g. under rotation, is held to the same absolute
                    // accuracy as its neighbours, not to its own tiny magnitude)
                    const q escale = qabs(e) > (q)(strain * l0) ? qabs(e) : (q)(strain * l0);
                    const q fscale = escale * kh;
                    const q ee = (q)out.e.h + (q)out.e.l;
                    const double re = (double)(qabs(ee - e) / escale);
                    const q gx2 = (q)out.f[0].h + (q)out.f[0].l - fx, gy2 = (q)out.f[1].h + (q)out.f[1].l - fy;
                    const double rf = (double)(sqrtq(gx2 * gx2 + gy2 * gy2) / fscale);
                    if (re > we) we = re;
                    if (rf > wf) wf = rf;
                    n++;
                }
            }
            std::printf("dx %.0e strain %.0e: extension %.2e  force %.2e\n", dx, strain, we, wf);
            if (we > worst_e) worst_e = we;
            if (wf > worst_f) worst_f = wf;
        }
    }
    std::printf("bonds %ld, offset fallbacks %ld, worst extension %.2e, worst force %.2e\n", n, fallbacks, worst_e,
                worst_f);
    // break decisions around the threshold
    long bad = 0, checked = 0;
    for (long i = 0; i < 2000000; i++) {
        const double l0t = 1.5075e-4 * (1.0 + 1e-3 * U(rng));
        Tpl T;
        const double xv[2] = {l0t, 0.0};
        make_tpl(T, xv, l0t);
        const double s0 = std::pow(10.0, -4.0 + 3.0 * (U(rng) + 1.0) / 2.0);
        const float dl = (float)(std::ldexp((double)(rng() % 512), std::ilogb(l0t) - 52));
        const double l0 = l0t + (double)dl;
        const double ecrit = s0 * l0;
        // e near the threshold: relative offsets from 1e-16 to 1e-5 either side
        const double rel = std::pow(10.0, -16.0 + 11.0 * (U(rng) + 1.0) / 2.0) * (U(rng) < 0 ? -1.0 : 1.0);
        const double ev = ecrit * (1.0 + rel);
        const f2 e = split_bits(ev);
        const bool want = pair_sum_f64(e) > ecrit;
        const bool got = exceeds(e, s0, (float)s0, T, dl);
        checked++;
        if (want != got) bad++;
    }
    std::printf("break decisions: %ld checked, %ld differ from the double test\n", checked, bad);
    double e3 = 0.0, f3 = 0.0;
    const bool ok3 = check3(rng, e3, f3);
    std::printf("3-D stretch: worst extension %.2e, worst direction term %.2e\n", e3, f3);
    // ADR damping terms against the exact value of the reference's formula
    double worst_t = 0.0, worst_ref = 0.0;
    long t_checked = 0, t_fallback = 0;
    auto logu = [&](double lo, double hi) { return std::pow(10.0, lo + (hi - lo) * (U(rng) + 1.0) / 2.0); };
    for (long i = 0; i < 2000000; i++) {
        const double u = logu(-12.0, -1.0) * (U(rng) < 0 ? -1.0 : 1.0);
        const double fo = logu(-6.0, 12.0) * (U(rng) < 0 ? -1.0 : 1.0);
        // F near F_old (relative differences from 1e-15 to 10) or unrelated
        const double f = (i & 1) ? fo * (1.0 + logu(-15.0, 1.0) * (U(rng) < 0 ? -1.0 : 1.0))
                                 : logu(-6.0, 12.0) * (U(rng) < 0 ? -1.0 : 1.0);
        const double m = logu(-3.0, 24.0);
        const double rmass = 1.0 / m;
        const double dt = (i % 3 == 0) ? 1.0 : logu(-9.0, 0.0);
        const double vh = logu(-40.0, 40.0) * (U(rng) < 0 ? -1.0 : 1.0);  // also outside [2^-100, 2^101)
        if (f == fo) continue;
        const double got = damping_term(u, f, fo, rmass, dt, vh);
        const q exact = -((q)u * (q)u) * ((q)f - (q)fo) / (q)m / ((q)dt * (q)vh);
        const double d = dt * vh;
        if (!(std::fabs(d) >= std::ldexp(1.0, -100) && std::fabs(d) < std::ldexp(1.0, 101))) t_fallback++;
        const double rel = (double)(qabs((q)got - exact) / qabs(exact));
        if (rel > worst_t) worst_t = rel;
        // the reference's own double evaluation of its formula
        const double ref = -1.0 * u * u * (f / m - fo / m) / (dt * vh);
        const double rel_ref = (double)(qabs((q)ref - exact) / qabs(exact));
        if (rel_ref > worst_ref) worst_ref = rel_ref;
        t_checked++;
    }
    const double t_ulps = worst_t / std::ldexp(1.0, -53);
    std::printf("damping terms: %ld checked (%ld by the IEEE division), worst %.2f units of 2^-53 "
                "(the reference's double evaluation: %.3g)\n",
                t_checked, t_fallback, t_ulps, worst_ref / std::ldexp(1.0, -53));
    const bool ok = ok3 && worst_e <= 2e-13 && worst_f <= 2e-13 && e3 <= 2e-13 && f3 <= 2e-13 && bad == 0 &&
                    t_ulps <= 8.0 && t_fallback > 0;
    std::printf(ok ? "OK\n" : "FAIL\n");
    return ok ? 0 : 1;
}
