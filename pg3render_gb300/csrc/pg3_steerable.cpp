// Host-side build of the steerable sampler tables (see pg3_steerable.h).
#include "pg3_steerable.h"

#include <climits>
#include <cmath>
#include <map>
#include <utility>

namespace pg3 {

namespace {

struct D3 { double x, y, z; };
D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
D3 crs(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dt(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
D3 nrm(D3 a) { const double l = std::sqrt(dt(a, a)); return {a.x / l, a.y / l, a.z / l}; }

const float kPi = 3.14159265358979f;

// Bilinear (tent) lookup of the lat-long map, as the kernels do (src/em_image.hxx:95-143).
float emLuminanceAt(const float *rgb, uint32_t W, uint32_t H, float dx, float dy, float dz)
{
    const float phi = -std::atan2(dy, dx);
    const float theta = std::acos(std::fmin(std::fmax(dz, -1.f), 1.f));
    const float u = std::fmin(std::fmax(0.5f + phi * 0.5f * (1.f / kPi), 0.f), 1.f);
    const float v = std::fmin(std::fmax(theta * (1.f / kPi), 0.f), 1.f);
    const float xf = u * (float)W, yf = v * (float)H;
    const int cx = (int)(xf + 0.5f), cy = (int)(yf + 0.5f);
    const int x0 = cx - 1, y0 = cy - 1;
    const float xl = xf - ((float)x0 + 0.5f), yl = yf - ((float)y0 + 0.5f);
    auto wrap = [&](int x, int y, int &ox, int &oy) {
        int rx = x, ry = y;
        if (y >= (int)H) { rx = x + (int)W / 2; ry = (int)H - 1; }
        else if (y < 0) { rx = x + (int)W / 2; ry = 0; }
        int m = rx % (int)W;
        if (m < 0) m += (int)W;
        ox = m; oy = ry;
    };
    auto lum = [&](int x, int y) {
        const float *p = rgb + ((size_t)y * W + (size_t)x) * 3;
        return 0.212671f * p[0] + 0.715160f * p[1] + 0.072169f * p[2];
    };
    int ax, ay, bx, by;
    wrap(x0, y0, ax, ay);
    wrap(cx, cy, bx, by);
    const float top = (1.f - xl) * lum(ax, ay) + xl * lum(bx, ay);
    const float bot = (1.f - xl) * lum(ax, by) + xl * lum(bx, by);
    return (1.f - yl) * top + yl * bot;
}

// 9 real SH basis values (Ramamoorthi & Hanrahan 2001), scaled by s.
void shBasis(double x, double y, double z, double s, float *o)
{
    o[0] = (float)(s * 0.282095);
    o[1] = (float)(s * 0.488603 * y);
    o[2] = (float)(s * 0.488603 * z);
    o[3] = (float)(s * 0.488603 * x);
    o[4] = (float)(s * 1.092548 * x * y);
    o[5] = (float)(s * 1.092548 * y * z);
    o[6] = (float)(s * 0.315392 * (3.0 * z * z - 1.0));
    o[7] = (float)(s * 1.092548 * x * z);
    o[8] = (float)(s * 0.546274 * (x * x - y * y));
}

}  // namespace

bool buildSteerable(const float *rgb, uint32_t W, uint32_t H, uint32_t level, SteerableHost &out, std::string &err)
{
    if (level > 7) { err = "steerable subdivision level must be <= 7"; return false; }
    out = SteerableHost();
    out.level = level;

    // icosahedron: the 12 cyclic permutations of (0, +-1, +-t), normalised
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<D3> v;
    for (int s1 = -1; s1 <= 1; s1 += 2)
        for (int s2 = -1; s2 <= 1; s2 += 2) {
            v.push_back(nrm({0.0, (double)s1, s2 * t}));
            v.push_back(nrm({(double)s1, s2 * t, 0.0}));
            v.push_back(nrm({s2 * t, 0.0, (double)s1}));
        }
    double emin = 1e9;
    for (size_t i = 0; i < v.size(); ++i)
        for (size_t j = i + 1; j < v.size(); ++j) emin = std::fmin(emin, std::sqrt(dt(sub(v[i], v[j]), sub(v[i], v[j]))));
    auto adjacent = [&](size_t i, size_t j) { return std::sqrt(dt(sub(v[i], v[j]), sub(v[i], v[j]))) < emin * 1.001; };
    std::vector<int4> level0;
    for (size_t i = 0; i < v.size(); ++i)
        for (size_t j = i + 1; j < v.size(); ++j)
            for (size_t k = j + 1; k < v.size(); ++k)
                if (adjacent(i, j) && adjacent(j, k) && adjacent(i, k)) {
                    const D3 n = crs(sub(v[j], v[i]), sub(v[k], v[i]));
                    const bool ccw = dt(n, add(add(v[i], v[j]), v[k])) > 0;   // outward facing
                    level0.push_back(make_int4((int)i, ccw ? (int)j : (int)k, ccw ? (int)k : (int)j, 0));
                }
    if (level0.size() != 20) { err = "icosahedron construction failed"; return false; }

    // 4-way subdivision, children (A,ab,ca), (ab,B,bc), (ca,bc,C), (ab,bc,ca)
    std::map<std::pair<int, int>, int> mid;
    auto midpoint = [&](int a, int b) {
        const auto key = std::make_pair(std::min(a, b), std::max(a, b));
        auto it = mid.find(key);
        if (it != mid.end()) return it->second;
        v.push_back(nrm(add(v[a], v[b])));
        const int id = (int)v.size() - 1;
        mid[key] = id;
        return id;
    };
    out.tri = level0;
    out.levelOffset.push_back(0);
    std::vector<int4> cur = level0;
    for (uint32_t l = 0; l < level; ++l) {
        std::vector<int4> next;
        next.reserve(cur.size() * 4);
        for (const int4 &T : cur) {
            const int ab = midpoint(T.x, T.y), bc = midpoint(T.y, T.z), ca = midpoint(T.z, T.x);
            next.push_back(make_int4(T.x, ab, ca, 0));
            next.push_back(make_int4(ab, T.y, bc, 0));
            next.push_back(make_int4(ca, bc, T.z, 0));
            next.push_back(make_int4(ab, bc, ca, 0));
        }
        out.levelOffset.push_back((uint32_t)out.tri.size());
        out.tri.insert(out.tri.end(), next.begin(), next.end());
        cur.swap(next);
    }
    out.levelOffset.push_back((uint32_t)out.tri.size());

    // vertex weights: SH basis scaled by the map's luminance in the vertex direction
    const size_t nv = v.size();
    out.vdir.resize(nv);
    out.vw.resize(nv * 9);
    for (size_t i = 0; i < nv; ++i) {
        out.vdir[i] = make_float4((float)v[i].x, (float)v[i].y, (float)v[i].z, 0.f);
        const float L = emLuminanceAt(rgb, W, H, (float)v[i].x, (float)v[i].y, (float)v[i].z);
        shBasis(v[i].x, v[i].y, v[i].z, (double)L, &out.vw[i * 9]);
    }

    // leaf weights: planar area x mean vertex weight (src/em_steerable_sampler.hxx:1277-1296),
    // and each leaf's plane (unit normal, distance) for the solid-angle Jacobian
    const uint32_t nLeaf = (uint32_t)cur.size();
    std::vector<float> leafW((size_t)nLeaf * 9);
    out.leafPlane.resize(nLeaf);
    for (uint32_t i = 0; i < nLeaf; ++i) {
        const int4 T = cur[i];
        const D3 a = {out.vdir[T.x].x, out.vdir[T.x].y, out.vdir[T.x].z};
        const D3 b = {out.vdir[T.y].x, out.vdir[T.y].y, out.vdir[T.y].z};
        const D3 c = {out.vdir[T.z].x, out.vdir[T.z].y, out.vdir[T.z].z};
        const D3 cr = crs(sub(b, a), sub(c, a));
        const double area = 0.5 * std::sqrt(dt(cr, cr));
        const D3 nT = nrm(cr);
        out.leafPlane[i] = make_float4((float)nT.x, (float)nT.y, (float)nT.z, (float)dt(nT, a));
        for (int k = 0; k < 9; ++k)
            leafW[(size_t)i * 9 + k] = (float)(area * ((double)out.vw[T.x * 9 + k] + out.vw[T.y * 9 + k] +
                                                       out.vw[T.z * 9 + k]) / 3.0);
    }

    // 6-ary tree, bottom-up over consecutive nodes (src/em_steerable_sampler.hxx:3755-3793)
    struct Item { int id; float w[9]; };
    std::vector<Item> layer(nLeaf);
    for (uint32_t i = 0; i < nLeaf; ++i) {
        layer[i].id = ~(int)i;
        for (int k = 0; k < 9; ++k) layer[i].w[k] = leafW[(size_t)i * 9 + k];
    }
    do {
        std::vector<Item> up;
        for (size_t s = 0; s < layer.size(); s += 6) {
            const int node = (int)(out.nodeChild.size() / 6);
            Item parent;
            parent.id = node;
            for (int k = 0; k < 9; ++k) parent.w[k] = 0.f;
            for (size_t c = 0; c < 6; ++c) {
                if (s + c < layer.size()) {
                    const Item &ch = layer[s + c];
                    out.nodeChild.push_back(ch.id);
                    for (int k = 0; k < 9; ++k) {
                        out.nodeW.push_back(ch.w[k]);
                        parent.w[k] += ch.w[k];
                    }
                } else {
                    out.nodeChild.push_back(INT_MIN);
                    for (int k = 0; k < 9; ++k) out.nodeW.push_back(0.f);
                }
            }
            up.push_back(parent);
        }
        layer.swap(up);
    } while (layer.size() > 1);
    out.root = layer[0].id;
    out.rootW.assign(9, 0.f);
    {
        double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (uint32_t i = 0; i < nLeaf; ++i)
            for (int k = 0; k < 9; ++k) acc[k] += leafW[(size_t)i * 9 + k];
        for (int k = 0; k < 9; ++k) out.rootW[k] = (float)acc[k];
    }

    // leaf locator: inward edge normals of every leaf, and for every cell of a finer cube map
    // the leaves whose bounding cap meets the cell's bounding cap (a superset of the leaves
    // that touch the cell); cells with more than 8 keep the face locator
    out.leafEdge.resize((size_t)nLeaf * 3);
    std::vector<D3> capC(nLeaf);
    std::vector<double> capR(nLeaf);
    for (uint32_t i = 0; i < nLeaf; ++i) {
        const int4 T = cur[i];
        const D3 a = {out.vdir[T.x].x, out.vdir[T.x].y, out.vdir[T.x].z};
        const D3 b = {out.vdir[T.y].x, out.vdir[T.y].y, out.vdir[T.y].z};
        const D3 c = {out.vdir[T.z].x, out.vdir[T.z].y, out.vdir[T.z].z};
        const D3 e[3] = {nrm(crs(a, b)), nrm(crs(b, c)), nrm(crs(c, a))};
        for (int k = 0; k < 3; ++k)
            out.leafEdge[3 * (size_t)i + k] = make_float4((float)e[k].x, (float)e[k].y, (float)e[k].z, 0.f);
        capC[i] = nrm(add(add(a, b), c));
        capR[i] = std::acos(std::fmin(1.0, std::fmin(dt(capC[i], a), std::fmin(dt(capC[i], b), dt(capC[i], c)))));
    }
    const uint32_t LG = 4u << level;
    out.leafGrid = LG;
    out.leafCells.assign((size_t)6 * LG * LG, make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu));
    for (int f = 0; f < 6; ++f) {
        const int ax = f / 2, bx = (ax + 1) % 3, cx = (ax + 2) % 3;
        const double sg = (f & 1) ? -1.0 : 1.0;
        auto dirOf = [&](double u, double vv) {
            double p[3];
            p[ax] = sg; p[bx] = u; p[cx] = vv;
            return nrm({p[0], p[1], p[2]});
        };
        for (uint32_t iv = 0; iv < LG; ++iv)
            for (uint32_t iu = 0; iu < LG; ++iu) {
                const double u0 = -1.0 + 2.0 * iu / LG, u1 = -1.0 + 2.0 * (iu + 1) / LG;
                const double v0 = -1.0 + 2.0 * iv / LG, v1 = -1.0 + 2.0 * (iv + 1) / LG;
                const D3 cc = dirOf(0.5 * (u0 + u1), 0.5 * (v0 + v1));
                double rc = 0.0;
                for (const D3 &q : {dirOf(u0, v0), dirOf(u1, v0), dirOf(u0, v1), dirOf(u1, v1)})
                    rc = std::fmax(rc, std::acos(std::fmin(1.0, dt(cc, q))));
                uint32_t ids[8];
                int n = 0;
                bool many = false;
                for (uint32_t i = 0; i < nLeaf && !many; ++i) {
                    const double ang = std::acos(std::fmax(-1.0, std::fmin(1.0, dt(cc, capC[i]))));
                    if (ang <= capR[i] + rc + 1e-4) {
                        if (n == 8 || i >= kSteerLeafMany) many = true;
                        else ids[n++] = i;
                    }
                }
                uint4 &cell = out.leafCells[((size_t)f * LG + iv) * LG + iu];
                if (many) {
                    cell = make_uint4(0xfffefffeu, 0xfffefffeu, 0xfffefffeu, 0xfffefffeu);
                    continue;
                }
                uint32_t w[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
                for (int k = 0; k < n; ++k) {
                    const uint32_t shift = (k & 1) ? 16u : 0u;
                    w[k >> 1] = (w[k >> 1] & ~(0xffffu << shift)) | (ids[k] << shift);
                }
                cell = make_uint4(w[0], w[1], w[2], w[3]);
            }
    }

    // face locator: for every cell of a cube map over the sphere, the level-0 faces that
    // touch the cell (found by dense sampling of the cell enlarged by a margin)
    const int G = kSteerCells;
    out.faceCells.assign(2 * 6 * G * G, make_int4(-1, -1, -1, -1));
    for (int f = 0; f < 6; ++f) {
        const int ax = f / 2, bx = (ax + 1) % 3, cx = (ax + 2) % 3;
        const double s = (f & 1) ? -1.0 : 1.0;
        for (int iv = 0; iv < G; ++iv)
            for (int iu = 0; iu < G; ++iu) {
                int found[8], nf = 0;
                const int K = 24;
                for (int sv = 0; sv <= K; ++sv)
                    for (int su = 0; su <= K; ++su) {
                        const double u = -1.0 + 2.0 * (iu + (su / (double)K) * 1.1 - 0.05) / G;
                        const double vv = -1.0 + 2.0 * (iv + (sv / (double)K) * 1.1 - 0.05) / G;
                        double p[3];
                        p[ax] = s; p[bx] = u; p[cx] = vv;
                        const D3 w = nrm({p[0], p[1], p[2]});
                        for (int fi = 0; fi < 20; ++fi) {
                            const int4 t = level0[fi];
                            const D3 A = {out.vdir[t.x].x, out.vdir[t.x].y, out.vdir[t.x].z};
                            const D3 B = {out.vdir[t.y].x, out.vdir[t.y].y, out.vdir[t.y].z};
                            const D3 C = {out.vdir[t.z].x, out.vdir[t.z].y, out.vdir[t.z].z};
                            const double m = std::fmin(std::fmin(dt(w, crs(A, B)), dt(w, crs(B, C))), dt(w, crs(C, A)));
                            if (m >= -1e-3) {
                                bool have = false;
                                for (int q = 0; q < nf; ++q) have |= (found[q] == fi);
                                if (!have && nf < 8) found[nf++] = fi;
                            }
                        }
                    }
                if (nf > 8) { err = "steerable face locator: more than 8 faces in a cube-map cell"; return false; }
                int4 &c0 = out.faceCells[2 * ((f * G + iv) * G + iu)];
                int4 &c1 = out.faceCells[2 * ((f * G + iv) * G + iu) + 1];
                c0.x = nf > 0 ? found[0] : -1;
                c0.y = nf > 1 ? found[1] : -1;
                c0.z = nf > 2 ? found[2] : -1;
                c0.w = nf > 3 ? found[3] : -1;
                c1.x = nf > 4 ? found[4] : -1;
                c1.y = nf > 5 ? found[5] : -1;
                c1.z = nf > 6 ? found[6] : -1;
                c1.w = nf > 7 ? found[7] : -1;
            }
    }
    return true;
}

}  // namespace pg3
