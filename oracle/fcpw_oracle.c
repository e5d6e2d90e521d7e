/*
 * fcpw_oracle.c — TEST INFRASTRUCTURE ONLY. CPU restatement of the reference
 * (rohan-sawhney/fcpw) CPU query path, used by tests/ and by bench.py's CPU
 * baseline as the checker. Nothing in the product links or calls this file.
 *
 * It restates, in plain C99 and in FP32 with the reference's operation order
 * (Eigen fixed-size reductions halve: a0 + (a1 + a2)), the algorithms of:
 *   - Bvh::processSubtreeForClosestPoint / findClosestPointFromNode
 *     include/fcpw/aggregates/bvh.inl:1291-1418 (CPU tie-break at 1352-1356)
 *   - Baseline::findClosestPointFromNode, include/fcpw/aggregates/baseline.inl:343-382
 *   - findClosestPointTriangle, include/fcpw/geometry/triangles.inl:374-458
 *   - findClosestPointLineSegment, include/fcpw/geometry/line_segments.inl:200-226
 *   - Triangle::intersect (Moller-Trumbore), triangles.inl:222-260
 *   - LineSegment::intersect, line_segments.inl:140-175
 *   - Bvh::processSubtreeForIntersection (rays), bvh.inl:655-771
 *   - BoundingBox overlap / intersect, include/fcpw/core/bounding_volumes.h:62-114
 *   - processSubtreeForClosestSilhouettePoint, bvh.inl:1435-1596
 *   - BoundingCone::overlap, bounding_volumes.h:262-321
 *   - SilhouetteEdge / SilhouetteVertex::findClosestSilhouettePoint,
 *     silhouette_edges.inl:83-143, silhouette_vertices.inl:59-117
 *   - Bvh sphere sampling, bvh.inl:1140-1288, Triangle/LineSegment::samplePoint
 *   - Bvh refit boxes, bvh.inl:548-599; mergeBoundingCones, bounding_volumes.h:334-387
 *   - Aggregate::contains / hasLineOfSight, core/primitive.h:173-207, with the
 *     all-hits ray traversal bvh.inl:888-1029 and removeDuplicates,
 *     core/interaction.h:20-25,75-94
 * plus an FP64 brute force used as the accuracy yardstick, a sequential
 * model of the device linear-BVH build (which has no reference counterpart)
 * and the instanced scenes of Scene::build (fcpw.inl:1053-1102) with
 * TransformedAggregate (core/primitive.h:289-478).
 *
 * Inputs are the flattened tree and records in the reference's GPU interop
 * layouts (include/fcpw/gpu/bvh_interop_structures.h:55-162,730-774).
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z; } of3;
typedef struct { of3 pMin, pMax; uint32_t nPrims, offset; } onode;                       /* 32 B */
typedef struct { of3 pMin, pMax; of3 axis; float halfAngle, radius;
                 uint32_t nPrims, offset, nSil, silOff; } osnch;                           /* 60 B */
typedef struct { of3 pa, pb, pc; uint32_t index; } otri;                                  /* 40 B */
typedef struct { of3 pa, pb; uint32_t index; } oseg;                                      /* 28 B */
typedef struct { of3 p, n0, n1; uint32_t index, one; } overt;                             /* 44 B */
typedef struct { of3 pa, pb, n0, n1; uint32_t index, one; } oedge;                        /* 56 B */
typedef struct { of3 c; float r2; } osphere;                                              /* 16 B */
typedef struct { of3 o, d, dInv; float tMax; } oray;                                      /* 40 B */
typedef struct { of3 p, n; float u, v; float d; uint32_t index; } oint;                   /* 40 B */

#define OMAXF 3.402823466e+38F
#define OEPS 1.192092896e-07F
#define OPI 3.14159265358979323846f
#define OPI2 1.57079632679489661923f
#define OUMAX 0xffffffffu
#define OSTACK 64

/* ------------------------------------------------------------ vector ops */
static of3 v3(float x, float y, float z) { of3 r = {x, y, z}; return r; }
static of3 add3(of3 a, of3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static of3 sub3(of3 a, of3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static of3 mul3(of3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static of3 div3(of3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
static float minf_(float x, float y) { return y < x ? y : x; }
static float maxf_(float x, float y) { return x < y ? y : x; }
/* dim-aware reductions: 3D halves as a0 + (a1 + a2); 2D is a0 + a1 */
static float dotd(int dim, of3 a, of3 b) {
    return dim == 3 ? a.x * b.x + (a.y * b.y + a.z * b.z) : a.x * b.x + a.y * b.y;
}
static float normd(int dim, of3 a) { return sqrtf(dotd(dim, a, a)); }
static of3 normalizedd(int dim, of3 a) {
    float z = dotd(dim, a, a);
    return z > 0.0f ? div3(a, sqrtf(z)) : a;
}
static of3 cross3(of3 a, of3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static float comp(of3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

static oint default_interaction(void) {
    oint i;
    memset(&i, 0, sizeof(i));
    i.d = OMAXF;
    i.index = OUMAX;
    return i;
}

/* --------------------------------------------------- bounding box tests */
/* computeSquaredDistance, bounding_volumes.h:64-69 */
static void box_sq_dist(int dim, of3 pMin, of3 pMax, of3 c, float *d2Min, float *d2Max) {
    of3 u = sub3(pMin, c), v = sub3(c, pMax);
    of3 a = v3(maxf_(maxf_(u.x, v.x), 0.0f), maxf_(maxf_(u.y, v.y), 0.0f), maxf_(maxf_(u.z, v.z), 0.0f));
    of3 b = v3(minf_(u.x, v.x), minf_(u.y, v.y), minf_(u.z, v.z));
    *d2Min = dotd(dim, a, a);
    *d2Max = dotd(dim, b, b);
}
static float box_sq_dist_min(int dim, of3 pMin, of3 pMax, of3 c) {
    float a, b;
    box_sq_dist(dim, pMin, pMax, c, &a, &b);
    return a;
}
/* BoundingBox::intersect(ray), bounding_volumes.h:99-114 (no parallel-slab guard) */
static int box_ray(int dim, of3 pMin, of3 pMax, const oray *r, float *tMin, float *tMax) {
    float tn = -OMAXF, tf = OMAXF;
    int i;
    for (i = 0; i < dim; i++) {
        float t0 = (comp(pMin, i) - comp(r->o, i)) * comp(r->dInv, i);
        float t1 = (comp(pMax, i) - comp(r->o, i)) * comp(r->dInv, i);
        float nn = minf_(t0, t1), ff = maxf_(t0, t1);
        if (i == 0) { tn = nn; tf = ff; } else { tn = maxf_(tn, nn); tf = minf_(tf, ff); }
    }
    {
        float tNearMax = maxf_(0.0f, tn);
        float tFarMin = minf_(r->tMax, tf);
        if (tNearMax > tFarMin) return 0;
        *tMin = tNearMax;
        *tMax = tFarMin;
    }
    return 1;
}

/* ------------------------------------------------------------ primitives */
/* triangles.inl:374-458 */
static float closest_point_triangle(of3 pa, of3 pb, of3 pc, of3 x, of3 *pt, float *t0, float *t1) {
    of3 ab = sub3(pb, pa), ac = sub3(pc, pa), ax = sub3(x, pa);
    float d1 = dotd(3, ab, ax), d2 = dotd(3, ac, ax);
    of3 bx, cx;
    float d3, d4, d5, d6, vc, vb, va, denom, v, w;
    if (d1 <= 0.0f && d2 <= 0.0f) { *t0 = 1.0f; *t1 = 0.0f; *pt = pa; return normd(3, sub3(x, *pt)); }
    bx = sub3(x, pb);
    d3 = dotd(3, ab, bx); d4 = dotd(3, ac, bx);
    if (d3 >= 0.0f && d4 <= d3) { *t0 = 0.0f; *t1 = 1.0f; *pt = pb; return normd(3, sub3(x, *pt)); }
    cx = sub3(x, pc);
    d5 = dotd(3, ab, cx); d6 = dotd(3, ac, cx);
    if (d6 >= 0.0f && d5 <= d6) { *t0 = 0.0f; *t1 = 0.0f; *pt = pc; return normd(3, sub3(x, *pt)); }
    vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        v = d1 / (d1 - d3);
        *t0 = 1.0f - v; *t1 = v;
        *pt = add3(pa, mul3(ab, v));
        return normd(3, sub3(x, *pt));
    }
    vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        w = d2 / (d2 - d6);
        *t0 = 1.0f - w; *t1 = 0.0f;
        *pt = add3(pa, mul3(ac, w));
        return normd(3, sub3(x, *pt));
    }
    va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        *t0 = 0.0f; *t1 = 1.0f - w;
        *pt = add3(pb, mul3(sub3(pc, pb), w));
        return normd(3, sub3(x, *pt));
    }
    denom = 1.0f / (va + vb + vc);
    v = vb * denom;
    w = vc * denom;
    *t0 = 1.0f - v - w; *t1 = v;
    *pt = add3(add3(pa, mul3(ab, v)), mul3(ac, w));
    return normd(3, sub3(x, *pt));
}

/* line_segments.inl:200-226 (2D: z is zero throughout) */
static float closest_point_segment(int dim, of3 pa, of3 pb, of3 x, of3 *pt, float *t) {
    of3 u = sub3(pb, pa), v = sub3(x, pa);
    float c1 = dotd(dim, u, v), c2;
    if (c1 <= 0.0f) { *pt = pa; *t = 0.0f; return normd(dim, sub3(x, *pt)); }
    c2 = dotd(dim, u, u);
    if (c2 <= c1) { *pt = pb; *t = 1.0f; return normd(dim, sub3(x, *pt)); }
    *t = c1 / c2;
    *pt = add3(pa, mul3(u, *t));
    return normd(dim, sub3(x, *pt));
}

/* Triangle::intersect, triangles.inl:222-260 */
static int intersect_triangle(of3 pa, of3 pb, of3 pc, const oray *r, int occl, oint *i) {
    of3 v1 = sub3(pb, pa), v2 = sub3(pc, pa);
    of3 p = cross3(r->d, v2);
    float det = dotd(3, v1, p), invDet, v, w, t;
    of3 s, q;
    if (fabsf(det) <= OEPS) return 0;
    invDet = 1.0f / det;
    s = sub3(r->o, pa);
    v = dotd(3, s, p) * invDet;
    if (v < 0 || v > 1) return 0;
    q = cross3(s, v1);
    w = dotd(3, r->d, q) * invDet;
    if (w < 0 || v + w > 1) return 0;
    t = dotd(3, v2, q) * invDet;
    if (t >= 0.0f && t <= r->tMax) {
        if (occl) return 1;
        i->d = t;
        i->p = add3(add3(pa, mul3(v1, v)), mul3(v2, w));
        i->n = normalizedd(3, cross3(v1, v2));
        i->u = 1.0f - v - w;
        i->v = v;
        return 1;
    }
    return 0;
}

/* LineSegment::intersect, line_segments.inl:140-175 */
static int intersect_segment(of3 pa, of3 pb, const oray *r, int occl, oint *i) {
    of3 u = sub3(pa, r->o), v = sub3(pb, pa);
    float dv = r->d.x * v.y - r->d.y * v.x, ud, s, uv, t;
    if (fabsf(dv) <= OEPS) return 0;
    ud = u.x * r->d.y - u.y * r->d.x;
    s = ud / dv;
    if (s >= 0.0f && s <= 1.0f) {
        uv = u.x * v.y - u.y * v.x;
        t = uv / dv;
        if (t >= 0.0f && t <= r->tMax) {
            if (occl) return 1;
            i->d = t;
            i->p = add3(pa, mul3(v, s));
            i->n = normalizedd(2, v3(v.y, -v.x, 0.0f));
            i->u = s;
            i->v = 0.0f;
            return 1;
        }
    }
    return 0;
}

/* uniform access to primitive arrays */
typedef struct { of3 pa, pb, pc; uint32_t index; } oprim;
static oprim load_prim(int dim, const void *prims, uint32_t k) {
    oprim p;
    if (dim == 3) {
        const otri *t = (const otri *)prims + k;
        p.pa = t->pa; p.pb = t->pb; p.pc = t->pc; p.index = t->index;
    } else {
        const oseg *s = (const oseg *)prims + k;
        p.pa = s->pa; p.pb = s->pb; p.pc = v3(0, 0, 0); p.index = s->index;
    }
    return p;
}
/* findClosestPoint of one primitive; returns 1 when d*d <= r2 */
static int prim_closest(int dim, const oprim *p, of3 c, float r2, oint *i) {
    float d, t0, t1 = 0.0f;
    of3 pt;
    if (dim == 3) d = closest_point_triangle(p->pa, p->pb, p->pc, c, &pt, &t0, &t1);
    else d = closest_point_segment(2, p->pa, p->pb, c, &pt, &t0);
    if (d * d <= r2) {
        i->p = pt;
        i->u = t0;
        i->v = t1;
        i->d = d;
        i->index = p->index;
        return 1;
    }
    return 0;
}
static of3 prim_normal(int dim, const oprim *p) {
    if (dim == 3) return normalizedd(3, cross3(sub3(p->pb, p->pa), sub3(p->pc, p->pa)));
    {
        of3 s = sub3(p->pb, p->pa);
        return normalizedd(2, v3(s.y, -s.x, 0.0f));
    }
}
static float prim_area(int dim, const oprim *p) {
    if (dim == 3) return 0.5f * normd(3, cross3(sub3(p->pb, p->pa), sub3(p->pc, p->pa)));
    return normd(2, sub3(p->pb, p->pa));
}

/* node access for the two node layouts (the box/offset prefix is shared) */
typedef struct { of3 pMin, pMax; uint32_t nPrims, offset; } obox;
static obox load_node(int snch, const void *nodes, uint32_t i) {
    obox b;
    if (snch) {
        const osnch *n = (const osnch *)nodes + i;
        b.pMin = n->pMin; b.pMax = n->pMax; b.nPrims = n->nPrims; b.offset = n->offset;
    } else {
        const onode *n = (const onode *)nodes + i;
        b.pMin = n->pMin; b.pMax = n->pMax; b.nPrims = n->nPrims; b.offset = n->offset;
    }
    return b;
}

/* ------------------------------------------------------ closest point */
/* bvh.inl:1291-1418; the sphere's r2 is shrunk in place (as the reference
   does on its BoundingSphere&), *bestOut receives the winner; returns found.
   gpuOrder: children ordered as the reference's GPU traversal orders them
   (bvh.slang:458-470, by d2Min alone, the left child first on equal
   distances) instead of the CPU's d2Max tie-break when both d2Min are 0; it
   counts the visits of the GPU reference-order kernel (traversal statistics) */
static int closest_point_bvh_core(int dim, int snch, const void *nodes, const void *prims, osphere *sp_,
                                  int recordNormal, oint *bestOut, uint32_t *visited, int gpuOrder) {
    osphere s = *sp_;
    oint best = default_interaction();
    int found = 0;
    uint32_t selected = OUMAX;
    uint32_t stackNode[OSTACK];
    float stackDist[OSTACK];
    float bh[4];
    uint32_t nv = 0;
    obox root = load_node(snch, nodes, 0);
    box_sq_dist(dim, root.pMin, root.pMax, s.c, &bh[0], &bh[1]);
    if (bh[0] <= s.r2) {
        int sp = 0;
        s.r2 = minf_(s.r2, bh[1]);
        stackNode[0] = 0;
        stackDist[0] = bh[0];
        while (sp >= 0) {
            uint32_t ni = stackNode[sp];
            float cur = stackDist[sp];
            obox node;
            sp--;
            if (cur > s.r2) continue;
            node = load_node(snch, nodes, ni);
            if (node.nPrims > 0) {
                uint32_t p;
                for (p = 0; p < node.nPrims; p++) {
                    oprim pr = load_prim(dim, prims, node.offset + p);
                    oint c = default_interaction();
                    nv++;
                    if (prim_closest(dim, &pr, s.c, s.r2, &c)) {
                        found = 1;
                        s.r2 = minf_(s.r2, c.d * c.d);
                        best = c;
                        selected = node.offset + p;
                    }
                }
            } else {
                uint32_t li = ni + 1, ri = ni + node.offset, closer, other;
                obox l = load_node(snch, nodes, li), r = load_node(snch, nodes, ri);
                int hit0, hit1;
                box_sq_dist(dim, l.pMin, l.pMax, s.c, &bh[0], &bh[1]);
                hit0 = bh[0] <= s.r2;
                s.r2 = minf_(s.r2, bh[1]);
                box_sq_dist(dim, r.pMin, r.pMax, s.c, &bh[2], &bh[3]);
                hit1 = bh[2] <= s.r2;
                s.r2 = minf_(s.r2, bh[3]);
                if (hit0 && hit1) {
                    closer = li; other = ri;
                    if (!gpuOrder && bh[0] == 0.0f && bh[2] == 0.0f) {
                        if (bh[3] < bh[1]) { closer = ri; other = li; }
                    } else if (bh[2] < bh[0]) {
                        float t = bh[0]; bh[0] = bh[2]; bh[2] = t;
                        closer = ri; other = li;
                    }
                    sp++; stackNode[sp] = other; stackDist[sp] = bh[2];
                    sp++; stackNode[sp] = closer; stackDist[sp] = bh[0];
                } else if (hit0) {
                    sp++; stackNode[sp] = li; stackDist[sp] = bh[0];
                } else if (hit1) {
                    sp++; stackNode[sp] = ri; stackDist[sp] = bh[2];
                }
                nv++;
            }
        }
    }
    if (found && recordNormal) {
        oprim pr = load_prim(dim, prims, selected);
        best.n = prim_normal(dim, &pr);
    }
    if (visited) *visited = nv;
    *sp_ = s;
    *bestOut = best;
    return found;
}

static oint closest_point_bvh_one(int dim, int snch, const void *nodes, const void *prims, osphere s,
                                  int recordNormal, uint32_t *visited, int gpuOrder) {
    oint best;
    closest_point_bvh_core(dim, snch, nodes, prims, &s, recordNormal, &best, visited, gpuOrder);
    return best;
}

/* baseline.inl:343-382: linear scan in array order, later equal distances win */
static oint closest_point_brute_one(int dim, const void *prims, uint32_t nPrims, osphere s) {
    oint best = default_interaction();
    uint32_t p;
    for (p = 0; p < nPrims; p++) {
        oprim pr = load_prim(dim, prims, p);
        oint c = default_interaction();
        if (prim_closest(dim, &pr, s.c, s.r2, &c)) {
            s.r2 = minf_(s.r2, c.d * c.d);
            best = c;
        }
    }
    return best;
}

/* ---------------------------------------------------- FP64 brute force */
typedef struct { double x, y, z; } od3;
static od3 dd3(double x, double y, double z) { od3 r = {x, y, z}; return r; }
static od3 dsub(od3 a, od3 b) { return dd3(a.x - b.x, a.y - b.y, a.z - b.z); }
static od3 dadd(od3 a, od3 b) { return dd3(a.x + b.x, a.y + b.y, a.z + b.z); }
static od3 dmul(od3 a, double s) { return dd3(a.x * s, a.y * s, a.z * s); }
static double ddot(od3 a, od3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static od3 dcross(od3 a, od3 b) { return dd3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static od3 f2d(of3 a) { return dd3(a.x, a.y, a.z); }

/* same region method in double precision, vertices relative to the query */
static double closest_point_triangle_f64(od3 pa, od3 pb, od3 pc, od3 x) {
    od3 a = dsub(pa, x), b = dsub(pb, x), c = dsub(pc, x);
    od3 ab = dsub(b, a), ac = dsub(c, a), p;
    double d1 = -ddot(ab, a), d2 = -ddot(ac, a), d3, d4, d5, d6, vc, vb, va, v, w, denom;
    if (d1 <= 0 && d2 <= 0) return sqrt(ddot(a, a));
    d3 = -ddot(ab, b); d4 = -ddot(ac, b);
    if (d3 >= 0 && d4 <= d3) return sqrt(ddot(b, b));
    d5 = -ddot(ab, c); d6 = -ddot(ac, c);
    if (d6 >= 0 && d5 <= d6) return sqrt(ddot(c, c));
    vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { v = d1 / (d1 - d3); p = dadd(a, dmul(ab, v)); return sqrt(ddot(p, p)); }
    vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) { w = d2 / (d2 - d6); p = dadd(a, dmul(ac, w)); return sqrt(ddot(p, p)); }
    va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        p = dadd(b, dmul(dsub(c, b), w));
        return sqrt(ddot(p, p));
    }
    {
        /* face region: distance to the plane */
        od3 n = dcross(ab, ac);
        double nn = ddot(n, n);
        denom = 1.0 / (va + vb + vc);
        (void)denom;
        if (nn > 0) return fabs(ddot(a, n)) / sqrt(nn);
        return sqrt(ddot(a, a));
    }
}
static double closest_point_segment_f64(od3 pa, od3 pb, od3 x) {
    od3 u = dsub(pb, pa), v = dsub(x, pa), p;
    double c1 = ddot(u, v), c2, t;
    if (c1 <= 0) return sqrt(ddot(v, v));
    c2 = ddot(u, u);
    if (c2 <= c1) { od3 w = dsub(x, pb); return sqrt(ddot(w, w)); }
    t = c1 / c2;
    p = dsub(v, dmul(u, t));
    return sqrt(ddot(p, p));
}

/* Moller-Trumbore in double precision; returns t or -1 */
static double ray_triangle_f64(od3 pa, od3 pb, od3 pc, od3 o, od3 d, double tMax) {
    od3 v1 = dsub(pb, pa), v2 = dsub(pc, pa), p = dcross(d, v2), s, q;
    double det = ddot(v1, p), inv, v, w, t;
    if (fabs(det) == 0.0) return -1.0;
    inv = 1.0 / det;
    s = dsub(o, pa);
    v = ddot(s, p) * inv;
    if (v < 0 || v > 1) return -1.0;
    q = dcross(s, v1);
    w = ddot(d, q) * inv;
    if (w < 0 || v + w > 1) return -1.0;
    t = ddot(v2, q) * inv;
    return (t >= 0 && t <= tMax) ? t : -1.0;
}
static double ray_segment_f64(od3 pa, od3 pb, od3 o, od3 d, double tMax) {
    od3 u = dsub(pa, o), v = dsub(pb, pa);
    double dv = d.x * v.y - d.y * v.x, s, t;
    if (dv == 0.0) return -1.0;
    s = (u.x * d.y - u.y * d.x) / dv;
    if (s < 0 || s > 1) return -1.0;
    t = (u.x * v.y - u.y * v.x) / dv;
    return (t >= 0 && t <= tMax) ? t : -1.0;
}

/* ------------------------------------------------------------------ rays */
/* bvh.inl:655-771; r.tMax is shrunk in place, *bestOut receives the hit */
static oint ray_bvh_one(int dim, int snch, const void *nodes, const void *prims, oray r, int occl, int *hitOut);
static int ray_bvh_core(int dim, int snch, const void *nodes, const void *prims, oray *rp, int occl, oint *bestOut) {
    int hit;
    oint b = ray_bvh_one(dim, snch, nodes, prims, *rp, occl, &hit);
    /* the traversal's final tMax: the hit distance when something was hit, else unchanged */
    if (hit && !occl) rp->tMax = minf_(rp->tMax, b.d);
    *bestOut = b;
    return hit;
}
static oint ray_bvh_one(int dim, int snch, const void *nodes, const void *prims, oray r, int occl, int *hitOut) {
    oint best = default_interaction();
    int didHit = 0;
    uint32_t stackNode[OSTACK];
    float stackDist[OSTACK];
    float bh[4];
    obox root = load_node(snch, nodes, 0);
    *hitOut = 0;
    if (box_ray(dim, root.pMin, root.pMax, &r, &bh[0], &bh[1])) {
        int sp = 0;
        stackNode[0] = 0;
        stackDist[0] = bh[0];
        while (sp >= 0) {
            uint32_t ni = stackNode[sp];
            float cur = stackDist[sp];
            obox node;
            sp--;
            if (cur > r.tMax) continue;
            node = load_node(snch, nodes, ni);
            if (node.nPrims > 0) {
                uint32_t p;
                for (p = 0; p < node.nPrims; p++) {
                    oprim pr = load_prim(dim, prims, node.offset + p);
                    oint c = default_interaction();
                    int hit = dim == 3 ? intersect_triangle(pr.pa, pr.pb, pr.pc, &r, occl, &c)
                                       : intersect_segment(pr.pa, pr.pb, &r, occl, &c);
                    if (hit) {
                        c.index = pr.index;
                        if (occl) { best.index = c.index; *hitOut = 1; return best; }
                        didHit = 1;
                        r.tMax = minf_(r.tMax, c.d);
                        best = c;
                    }
                }
            } else {
                uint32_t li = ni + 1, ri = ni + node.offset;
                obox l = load_node(snch, nodes, li), rr = load_node(snch, nodes, ri);
                int hit0 = box_ray(dim, l.pMin, l.pMax, &r, &bh[0], &bh[1]);
                int hit1 = box_ray(dim, rr.pMin, rr.pMax, &r, &bh[2], &bh[3]);
                if (hit0 && hit1) {
                    uint32_t closer = li, other = ri;
                    if (bh[2] < bh[0]) {
                        float t = bh[0]; bh[0] = bh[2]; bh[2] = t;
                        t = bh[1]; bh[1] = bh[3]; bh[3] = t;
                        closer = ri; other = li;
                    }
                    sp++; stackNode[sp] = other; stackDist[sp] = bh[2];
                    sp++; stackNode[sp] = closer; stackDist[sp] = bh[0];
                } else if (hit0) {
                    sp++; stackNode[sp] = li; stackDist[sp] = bh[0];
                } else if (hit1) {
                    sp++; stackNode[sp] = ri; stackDist[sp] = bh[2];
                }
            }
        }
    }
    *hitOut = didHit;
    return best;
}

/* ------------------------------------------- contains / line of sight */
/* all hits of a ray (bvh.inl:888-1029 with recordAllHits: no tMax pruning,
   every primitive hit kept), sorted by distance, consecutive duplicates
   (|d - d'| < 1e-6 and |p - p'|^2 < 1e-6, core/interaction.h:20-25,75-94)
   removed; returns the count, or -1 past OHITS hits */
#define OHITS 256
static int ray_hit_count(int dim, int snch, const void *nodes, const void *prims, oray r) {
    float ds[OHITS];
    of3 ps[OHITS];
    int nh = 0, i, j, count;
    uint32_t stackNode[OSTACK];
    float stackDist[OSTACK];
    float bh[4];
    obox root = load_node(snch, nodes, 0);
    if (box_ray(dim, root.pMin, root.pMax, &r, &bh[0], &bh[1])) {
        int sp = 0;
        stackNode[0] = 0;
        stackDist[0] = bh[0];
        while (sp >= 0) {
            uint32_t ni = stackNode[sp];
            obox node;
            sp--;
            node = load_node(snch, nodes, ni);
            if (node.nPrims > 0) {
                uint32_t p;
                for (p = 0; p < node.nPrims; p++) {
                    oprim pr = load_prim(dim, prims, node.offset + p);
                    oint c = default_interaction();
                    int hit = dim == 3 ? intersect_triangle(pr.pa, pr.pb, pr.pc, &r, 0, &c)
                                       : intersect_segment(pr.pa, pr.pb, &r, 0, &c);
                    if (hit) {
                        if (nh >= OHITS) return -1;
                        ds[nh] = c.d;
                        ps[nh] = c.p;
                        nh++;
                    }
                }
            } else {
                uint32_t li = ni + 1, ri = ni + node.offset;
                obox l = load_node(snch, nodes, li), rr = load_node(snch, nodes, ri);
                int hit0 = box_ray(dim, l.pMin, l.pMax, &r, &bh[0], &bh[1]);
                int hit1 = box_ray(dim, rr.pMin, rr.pMax, &r, &bh[2], &bh[3]);
                if (sp + 2 >= OSTACK) return -1;
                if (hit0 && hit1) {
                    uint32_t closer = li, other = ri;
                    if (bh[2] < bh[0]) {
                        float t = bh[0]; bh[0] = bh[2]; bh[2] = t;
                        closer = ri; other = li;
                    }
                    sp++; stackNode[sp] = other; stackDist[sp] = bh[2];
                    sp++; stackNode[sp] = closer; stackDist[sp] = bh[0];
                } else if (hit0) {
                    sp++; stackNode[sp] = li; stackDist[sp] = bh[0];
                } else if (hit1) {
                    sp++; stackNode[sp] = ri; stackDist[sp] = bh[2];
                }
            }
        }
    }
    /* sort by distance (insertion sort; equal distances are duplicates or
       coincident hits, whose order does not change the count) */
    for (i = 1; i < nh; i++) {
        float d = ds[i];
        of3 p = ps[i];
        for (j = i - 1; j >= 0 && ds[j] > d; j--) { ds[j + 1] = ds[j]; ps[j + 1] = ps[j]; }
        ds[j + 1] = d;
        ps[j + 1] = p;
    }
    count = nh;
    for (i = 0; i + 1 < nh; i++) {
        of3 dp = sub3(ps[i], ps[i + 1]);
        if (fabsf(ds[i] - ds[i + 1]) < 1e-6f && dotd(dim, dp, dp) < 1e-6f) count--;
    }
    return count;
}

static oray make_ray(int dim, of3 o, of3 d, float tMax) {
    oray r;
    r.o = o;
    r.d = d;
    r.dInv = v3(1.0f / d.x, 1.0f / d.y, dim == 3 ? 1.0f / d.z : 1.0f / d.z);
    r.tMax = tMax;
    return r;
}

/* Aggregate::contains, core/primitive.h:173-193: rays along +x and +y, inside
   when both cross the boundary an odd number of times; -1 on overflow */
static int contains_one(int dim, int snch, const void *nodes, const void *prims, of3 x) {
    int h1 = ray_hit_count(dim, snch, nodes, prims, make_ray(dim, x, v3(1.0f, 0.0f, 0.0f), OMAXF));
    int h2 = ray_hit_count(dim, snch, nodes, prims, make_ray(dim, x, v3(0.0f, 1.0f, 0.0f), OMAXF));
    if (h1 < 0 || h2 < 0) return -1;
    return (h1 % 2 == 1 && h2 % 2 == 1) ? 1 : 0;
}

/* Aggregate::hasLineOfSight, core/primitive.h:196-207: an occlusion ray from xi
   towards xj with tMax = |xj - xi| */
static int line_of_sight_one(int dim, int snch, const void *nodes, const void *prims, of3 xi, of3 xj) {
    of3 dir = sub3(xj, xi);
    float dNorm = normd(dim, dir);
    int hit;
    oray r;
    dir = div3(dir, dNorm);
    if (dim == 2) dir.z = 0.0f;
    r = make_ray(dim, xi, dir, dNorm);
    ray_bvh_one(dim, snch, nodes, prims, r, 1, &hit);
    return hit ? 0 : 1;
}

/* ------------------------------------------------------------ silhouettes */
/* BoundingCone::overlap, bounding_volumes.h:262-321 */
static float project_to_plane(int dim, of3 n, of3 e) {
    if (dim == 2) {
        of3 b = v3(fabsf(-n.y), fabsf(n.x), 0.0f);
        return fabsf(dotd(2, e, b));
    } else {
        float sign = copysignf(1.0f, n.z);
        float a = -1.0f / (sign + n.z);
        float b = n.x * n.y * a;
        of3 b1 = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
        of3 b2 = v3(b, sign + n.y * n.y * a, -n.y);
        float r1 = dotd(3, e, v3(fabsf(b1.x), fabsf(b1.y), fabsf(b1.z)));
        float r2 = dotd(3, e, v3(fabsf(b2.x), fabsf(b2.y), fabsf(b2.z)));
        return sqrtf(r1 * r1 + r2 * r2);
    }
}
static int in_range(float v, float lo, float hi) { return v >= lo && v <= hi; }
static int cone_overlap(int dim, of3 axis, float halfAngle, float radius, of3 o, of3 bMin, of3 bMax, float distToBox) {
    of3 c, vca, e;
    float l, dAxisAngle, d, s;
    if (halfAngle >= OPI2 || distToBox < OEPS) return 1;
    c = mul3(add3(bMin, bMax), 0.5f);
    vca = sub3(c, o);
    l = normd(dim, vca);
    vca = div3(vca, l);
    dAxisAngle = acosf(maxf_(-1.0f, minf_(1.0f, dotd(dim, axis, vca))));
    if (in_range(OPI2, dAxisAngle - halfAngle, dAxisAngle + halfAngle)) return 1;
    if (l > radius) {
        float vh = asinf(radius / l);
        float hs = halfAngle + vh;
        return hs >= OPI2 ? 1 : in_range(OPI2, dAxisAngle - hs, dAxisAngle + hs);
    }
    e = sub3(bMax, c);
    d = dotd(dim, e, v3(fabsf(vca.x), fabsf(vca.y), fabsf(vca.z)));
    s = l - d;
    if (s <= 0.0f) return 1;
    d = project_to_plane(dim, vca, e);
    {
        float vh = atan2f(d, s);
        float hs = halfAngle + vh;
        return hs >= OPI2 ? 1 : in_range(OPI2, dAxisAngle - hs, dAxisAngle + hs);
    }
}

/* silhouette_vertices.inl:59-85 / silhouette_edges.inl:83-111 */
static int is_silhouette(int dim, of3 pa, of3 pb, of3 n0, of3 n1, of3 viewDir, float d, int flip, float precision) {
    float sign = flip ? 1.0f : -1.0f, dot0, dot1;
    of3 vd;
    if (d <= precision) {
        if (dim == 2) {
            float det = n0.x * n1.y - n0.y * n1.x;
            return sign * det > precision;
        } else {
            of3 ed = normalizedd(3, sub3(pb, pa));
            float ang = atan2f(dotd(3, ed, cross3(n0, n1)), dotd(3, n0, n1));
            return sign * ang > precision;
        }
    }
    vd = div3(viewDir, d);
    dot0 = dotd(dim, vd, n0);
    dot1 = dotd(dim, vd, n1);
    if (fabsf(dot0) <= precision) return sign * dot1 > precision;
    if (fabsf(dot1) <= precision) return sign * dot0 > precision;
    return dot0 * dot1 < 0.0f;
}

typedef struct { of3 pa, pb, n0, n1; uint32_t index, one; } osil;
static osil load_sil(int dim, const void *sils, uint32_t k) {
    osil s;
    if (dim == 3) {
        const oedge *e = (const oedge *)sils + k;
        s.pa = e->pa; s.pb = e->pb; s.n0 = e->n0; s.n1 = e->n1; s.index = e->index; s.one = e->one;
    } else {
        const overt *v = (const overt *)sils + k;
        s.pa = v->p; s.pb = v->p; s.n0 = v->n0; s.n1 = v->n1; s.index = v->index; s.one = v->one;
    }
    return s;
}
static int sil_closest(int dim, const osil *s, of3 c, float r2, int flip, float sqMinR, float precision, oint *i) {
    float d, t = 0.0f;
    of3 pt;
    int isSil;
    if (sqMinR >= r2) return 0;
    if (dim == 3) d = closest_point_segment(3, s->pa, s->pb, c, &pt, &t);
    else { pt = s->pa; d = normd(2, sub3(c, pt)); }
    if (d * d > r2) return 0;
    isSil = s->one != 0;
    if (!isSil) isSil = is_silhouette(dim, s->pa, s->pb, s->n0, s->n1, sub3(c, pt), d, flip, precision);
    if (isSil && d * d <= r2) {
        i->d = d;
        i->p = pt;
        i->index = s->index;
        i->u = dim == 3 ? t : 0.0f; /* the GPU record convention: uv = (t, 0) / (0, 0) */
        i->v = 0.0f;
        return 1;
    }
    return 0;
}

/* bvh.inl:1435-1596 */
static oint silhouette_bvh_one(int dim, const osnch *nodes, const void *sils, osphere s, int flip, float sqMinR,
                               float precision) {
    oint best = default_interaction();
    uint32_t stackNode[OSTACK];
    float stackDist[OSTACK];
    float bh[2];
    if (sqMinR >= s.r2) return best;
    bh[0] = box_sq_dist_min(dim, nodes[0].pMin, nodes[0].pMax, s.c);
    if (bh[0] <= s.r2) {
        int sp = 0;
        stackNode[0] = 0;
        stackDist[0] = bh[0];
        while (sp >= 0) {
            uint32_t ni = stackNode[sp];
            float cur = stackDist[sp];
            const osnch *node;
            sp--;
            if (cur > s.r2) continue;
            node = nodes + ni;
            if (node->nPrims > 0) {
                uint32_t p;
                for (p = 0; p < node->nSil; p++) {
                    osil sl = load_sil(dim, sils, node->silOff + p);
                    oint c = default_interaction();
                    if (sl.index == best.index) continue;
                    if (sil_closest(dim, &sl, s.c, s.r2, flip, sqMinR, precision, &c)) {
                        s.r2 = minf_(s.r2, c.d * c.d);
                        best = c;
                        if (sqMinR >= s.r2) break;
                    }
                }
            } else {
                const osnch *n0 = nodes + ni + 1, *n1 = nodes + ni + node->offset;
                int hit0 = n0->halfAngle >= 0.0f, hit1;
                if (hit0) {
                    bh[0] = box_sq_dist_min(dim, n0->pMin, n0->pMax, s.c);
                    hit0 = bh[0] <= s.r2 &&
                           cone_overlap(dim, n0->axis, n0->halfAngle, n0->radius, s.c, n0->pMin, n0->pMax, bh[0]);
                }
                hit1 = n1->halfAngle >= 0.0f;
                if (hit1) {
                    bh[1] = box_sq_dist_min(dim, n1->pMin, n1->pMax, s.c);
                    hit1 = bh[1] <= s.r2 &&
                           cone_overlap(dim, n1->axis, n1->halfAngle, n1->radius, s.c, n1->pMin, n1->pMax, bh[1]);
                }
                if (hit0 && hit1) {
                    uint32_t closer = ni + 1, other = ni + node->offset;
                    if (bh[1] < bh[0]) {
                        float t = bh[0]; bh[0] = bh[1]; bh[1] = t;
                        closer = ni + node->offset; other = ni + 1;
                    }
                    sp++; stackNode[sp] = other; stackDist[sp] = bh[1];
                    sp++; stackNode[sp] = closer; stackDist[sp] = bh[0];
                } else if (hit0) {
                    sp++; stackNode[sp] = ni + 1; stackDist[sp] = bh[0];
                } else if (hit1) {
                    sp++; stackNode[sp] = ni + node->offset; stackDist[sp] = bh[1];
                }
            }
        }
    }
    return best;
}

/* ------------------------------------------------------- sphere sampling */
/* bvh.inl:1140-1288 with no branch weight callback */
static oint sphere_sample_bvh_one(int dim, int snch, const void *nodes, const void *prims, osphere s, of3 rn,
                                  int *hitOut) {
    oint best = default_interaction();
    int hits = 0;
    uint32_t selected = OUMAX;
    float bh[4];
    obox root = load_node(snch, nodes, 0);
    box_sq_dist(dim, root.pMin, root.pMax, s.c, &bh[0], &bh[1]);
    if (bh[0] <= s.r2) {
        float d2NodeMax = bh[1], u = rn.x, traversalPdf = 1.0f;
        uint32_t ni = 0;
        int guard;
        for (guard = 0; guard < OSTACK; guard++) {
            obox node = load_node(snch, nodes, ni);
            if (node.nPrims > 0) {
                float total = 0.0f;
                uint32_t p;
                for (p = 0; p < node.nPrims; p++) {
                    oprim pr = load_prim(dim, prims, node.offset + p);
                    oint c = default_interaction();
                    int hit = 0;
                    if (d2NodeMax <= s.r2) {
                        hit = 1;
                        c.index = pr.index;
                        c.d = prim_area(dim, &pr);
                    } else if (prim_closest(dim, &pr, s.c, s.r2, &c)) {
                        hit = 1;
                        c.d = prim_area(dim, &pr);
                    }
                    if (hit) {
                        float prob;
                        hits++;
                        total += c.d;
                        prob = c.d / total;
                        if (u < prob) {
                            u = u / prob;
                            best = c;
                            best.d *= traversalPdf;
                            selected = node.offset + p;
                        } else {
                            u = (u - prob) / (1.0f - prob);
                        }
                    }
                }
                if (total > 0.0f) best.d /= total;
                break;
            } else {
                uint32_t li = ni + 1, ri = ni + node.offset;
                obox l = load_node(snch, nodes, li), r = load_node(snch, nodes, ri);
                float w0, w1, tot, p0, p1;
                w0 = 0.0f; w1 = 0.0f;
                box_sq_dist(dim, l.pMin, l.pMax, s.c, &bh[0], &bh[1]);
                if (bh[0] <= s.r2) w0 = 1.0f;
                box_sq_dist(dim, r.pMin, r.pMax, s.c, &bh[2], &bh[3]);
                if (bh[2] <= s.r2) w1 = 1.0f;
                tot = w0 + w1;
                if (!(tot > 0.0f)) break;
                p0 = w0 / tot;
                p1 = 1.0f - p0;
                if (u < p0) { u = u / p0; ni = li; traversalPdf *= p0; d2NodeMax = bh[1]; }
                else { u = (u - p0) / p1; ni = ri; traversalPdf *= p1; d2NodeMax = bh[3]; }
            }
        }
    }
    *hitOut = 0;
    if (hits > 0 && best.index != OUMAX && selected != OUMAX) {
        oprim pr = load_prim(dim, prims, selected);
        float pdf;
        if (dim == 3) {
            of3 n = cross3(sub3(pr.pb, pr.pa), sub3(pr.pc, pr.pa));
            float area = normd(3, n);
            float u1 = sqrtf(rn.y), u2 = rn.z;
            float uu = 1.0f - u1, vv = u2 * u1, ww = 1.0f - uu - vv;
            best.u = uu; best.v = vv;
            best.p = add3(add3(mul3(pr.pa, uu), mul3(pr.pb, vv)), mul3(pr.pc, ww));
            best.n = div3(n, area);
            pdf = 2.0f / area;
        } else {
            of3 sv = sub3(pr.pb, pr.pa);
            float area = normd(2, sv);
            float uu = rn.y;
            best.u = uu; best.v = 0.0f;
            best.p = add3(pr.pa, mul3(sv, uu));
            best.n = div3(v3(sv.y, -sv.x, 0.0f), area);
            pdf = 1.0f / area;
        }
        best.d *= pdf;
        *hitOut = 1;
        return best;
    }
    return default_interaction();
}

/* --------------------------------------------------------------- refit */
static void refit_rec(int dim, int snch, void *nodes, const void *prims, const void *sils, uint32_t ni, int depth);

/* leaf cone from the silhouette records: axis = normalised sum of the stored
 * face normals (bvh.slang:46-98), degenerate axis keeps halfAngle = pi (bvh.inl:505-529) */
static void leaf_cone(int dim, osnch *node, const void *sils) {
    of3 centroid = mul3(add3(node->pMin, node->pMax), 0.5f), axis = v3(0, 0, 0);
    float radius = 0.0f;
    int any = 0, two = 1;
    uint32_t k;
    for (k = 0; k < node->nSil; k++) {
        osil s = load_sil(dim, sils, node->silOff + k);
        of3 sc = dim == 3 ? mul3(add3(s.pa, s.pb), 0.5f) : s.pa;
        axis = add3(add3(axis, s.n0), s.n1);
        radius = maxf_(radius, normd(dim, sub3(sc, centroid)));
        two = two && s.one == 0;
        any = 1;
    }
    if (!any) { node->axis = v3(0, 0, 0); node->halfAngle = -OPI; node->radius = 0.0f; return; }
    node->radius = radius;
    if (!two) { node->axis = axis; node->halfAngle = OPI; return; }
    {
        float an = normd(dim, axis);
        if (an > OEPS) {
            float ha = 0.0f;
            axis = div3(axis, an);
            for (k = 0; k < node->nSil; k++) {
                osil s = load_sil(dim, sils, node->silOff + k);
                ha = maxf_(ha, acosf(maxf_(-1.0f, minf_(1.0f, dotd(dim, axis, s.n0)))));
                ha = maxf_(ha, acosf(maxf_(-1.0f, minf_(1.0f, dotd(dim, axis, s.n1)))));
            }
            node->axis = axis;
            node->halfAngle = ha;
        } else {
            node->axis = axis;
            node->halfAngle = OPI;
        }
    }
}

/* rotate<DIM>, include/fcpw/core/core.h:116-148 */
static of3 rotate_towards(int dim, of3 u, of3 v, float theta) {
    if (dim == 2) {
        float det = u.x * v.y - u.y * v.x;
        float ct, st;
        theta *= copysignf(1.0f, det);
        ct = cosf(theta); st = sinf(theta);
        return v3(ct * u.x - st * u.y, st * u.x + ct * u.y, 0.0f);
    } else {
        float ct = cosf(theta), st = sinf(theta);
        of3 w = normalizedd(3, cross3(u, v));
        of3 o = mul3(w, 1.0f - ct);
        of3 r;
        r.x = (ct + o.x * w.x) * u.x + ((o.y * w.x - st * w.z) * u.y + (o.z * w.x + st * w.y) * u.z);
        r.y = (o.x * w.y + st * w.z) * u.x + ((ct + o.y * w.y) * u.y + (o.z * w.y - st * w.x) * u.z);
        r.z = (o.x * w.z - st * w.y) * u.x + ((o.y * w.z + st * w.x) * u.y + (ct + o.z * w.z) * u.z);
        return r;
    }
}

/* mergeBoundingCones, bounding_volumes.h:334-387 */
static void merge_cones(int dim, const osnch *a0, const osnch *b0, osnch *node) {
    of3 oa = mul3(add3(a0->pMin, a0->pMax), 0.5f), ob = mul3(add3(b0->pMin, b0->pMax), 0.5f);
    of3 o = mul3(add3(node->pMin, node->pMax), 0.5f);
    of3 axA = a0->axis, axB = b0->axis;
    float hA = a0->halfAngle, hB = b0->halfAngle, rA = a0->radius, rB = b0->radius;
    node->axis = v3(0, 0, 0);
    node->halfAngle = OPI;
    node->radius = 0.0f;
    if (hA >= 0.0f && hB >= 0.0f) {
        of3 da = sub3(o, oa), db = sub3(o, ob);
        float theta, oTheta;
        node->radius = sqrtf(maxf_(rA * rA + dotd(dim, da, da), rB * rB + dotd(dim, db, db)));
        if (hB > hA) { of3 t = axA; float th = hA; axA = axB; axB = t; hA = hB; hB = th; }
        theta = acosf(maxf_(-1.0f, minf_(1.0f, dotd(dim, axA, axB))));
        if (minf_(theta + hB, OPI) <= hA) { node->axis = axA; node->halfAngle = hA; return; }
        oTheta = (hA + theta + hB) / 2.0f;
        if (oTheta >= OPI) { node->axis = axA; return; }
        node->axis = rotate_towards(dim, axA, axB, oTheta - hA);
        node->halfAngle = oTheta;
    } else if (hA >= 0.0f) {
        node->axis = axA; node->halfAngle = hA; node->radius = rA;
    } else if (hB >= 0.0f) {
        node->axis = axB; node->halfAngle = hB; node->radius = rB;
    } else {
        node->halfAngle = -OPI;
    }
}

/* refitRecursive, bvh.inl:548-581 (boxes bit-exact with the reference) */
static void refit_rec(int dim, int snch, void *nodes, const void *prims, const void *sils, uint32_t ni, int depth) {
    obox nb = load_node(snch, nodes, ni);
    of3 pMin, pMax;
    if (depth > OSTACK) return;
    if (nb.nPrims == 0) {
        uint32_t li = ni + 1, ri = ni + nb.offset;
        obox l, r;
        refit_rec(dim, snch, nodes, prims, sils, li, depth + 1);
        refit_rec(dim, snch, nodes, prims, sils, ri, depth + 1);
        l = load_node(snch, nodes, li);
        r = load_node(snch, nodes, ri);
        pMin = v3(minf_(l.pMin.x, r.pMin.x), minf_(l.pMin.y, r.pMin.y), minf_(l.pMin.z, r.pMin.z));
        pMax = v3(maxf_(l.pMax.x, r.pMax.x), maxf_(l.pMax.y, r.pMax.y), maxf_(l.pMax.z, r.pMax.z));
    } else {
        uint32_t p;
        float ez = dim == 3 ? OEPS : 0.0f;
        pMin = v3(OMAXF, OMAXF, OMAXF);
        pMax = v3(-OMAXF, -OMAXF, -OMAXF);
        for (p = 0; p < nb.nPrims; p++) {
            oprim pr = load_prim(dim, prims, nb.offset + p);
            of3 lo = v3(minf_(pr.pa.x, pr.pb.x), minf_(pr.pa.y, pr.pb.y), minf_(pr.pa.z, pr.pb.z));
            of3 hi = v3(maxf_(pr.pa.x, pr.pb.x), maxf_(pr.pa.y, pr.pb.y), maxf_(pr.pa.z, pr.pb.z));
            if (dim == 3) {
                lo = v3(minf_(lo.x, pr.pc.x), minf_(lo.y, pr.pc.y), minf_(lo.z, pr.pc.z));
                hi = v3(maxf_(hi.x, pr.pc.x), maxf_(hi.y, pr.pc.y), maxf_(hi.z, pr.pc.z));
            }
            lo = v3(lo.x - OEPS, lo.y - OEPS, lo.z - ez);
            hi = v3(hi.x + OEPS, hi.y + OEPS, hi.z + ez);
            pMin = v3(minf_(pMin.x, lo.x), minf_(pMin.y, lo.y), minf_(pMin.z, lo.z));
            pMax = v3(maxf_(pMax.x, hi.x), maxf_(pMax.y, hi.y), maxf_(pMax.z, hi.z));
        }
    }
    if (snch) {
        osnch *n = (osnch *)nodes + ni;
        n->pMin = pMin; n->pMax = pMax;
        if (nb.nPrims == 0) merge_cones(dim, n + 1, n + n->offset, n);
        else leaf_cone(dim, n, sils);
    } else {
        onode *n = (onode *)nodes + ni;
        n->pMin = pMin; n->pMax = pMax;
    }
}

/* ------------------------------------------------------- threaded drivers */
typedef struct {
    int kind, dim, snch, flag, order;
    const void *nodes, *prims, *sils;
    uint32_t nPrims;
    const void *queries;
    const void *aux;
    uint32_t begin, end;
    float f0, f1;
    oint *out;
    uint32_t *u32out;
    double *f64out;
    int *hits;
} ojob;

static void run_range(ojob *j) {
    uint32_t q;
    for (q = j->begin; q < j->end; q++) {
        switch (j->kind) {
            case 0: j->out[q] = closest_point_bvh_one(j->dim, j->snch, j->nodes, j->prims,
                                                     ((const osphere *)j->queries)[q], j->flag,
                                                     j->u32out ? j->u32out + q : 0, j->order);
                break;
            case 1: j->out[q] = closest_point_brute_one(j->dim, j->prims, j->nPrims, ((const osphere *)j->queries)[q]);
                break;
            case 2: {
                osphere s = ((const osphere *)j->queries)[q];
                double best = INFINITY;
                uint32_t bi = OUMAX, p;
                for (p = 0; p < j->nPrims; p++) {
                    oprim pr = load_prim(j->dim, j->prims, p);
                    double d = j->dim == 3 ? closest_point_triangle_f64(f2d(pr.pa), f2d(pr.pb), f2d(pr.pc), f2d(s.c))
                                           : closest_point_segment_f64(f2d(pr.pa), f2d(pr.pb), f2d(s.c));
                    if (d < best) { best = d; bi = pr.index; }
                }
                if (!(best * best <= (double)s.r2)) { best = INFINITY; bi = OUMAX; }
                j->f64out[q] = best;
                j->u32out[q] = bi;
                break;
            }
            case 3: j->out[q] = ray_bvh_one(j->dim, j->snch, j->nodes, j->prims, ((const oray *)j->queries)[q],
                                            j->flag, &j->hits[q]);
                break;
            case 4: {
                oray r = ((const oray *)j->queries)[q];
                double best = INFINITY;
                uint32_t bi = OUMAX, p;
                for (p = 0; p < j->nPrims; p++) {
                    oprim pr = load_prim(j->dim, j->prims, p);
                    double t = j->dim == 3 ? ray_triangle_f64(f2d(pr.pa), f2d(pr.pb), f2d(pr.pc), f2d(r.o), f2d(r.d), (double)r.tMax)
                                           : ray_segment_f64(f2d(pr.pa), f2d(pr.pb), f2d(r.o), f2d(r.d), (double)r.tMax);
                    if (t >= 0.0 && t < best) { best = t; bi = pr.index; }
                }
                j->f64out[q] = best;
                j->u32out[q] = bi;
                break;
            }
            case 5: j->out[q] = silhouette_bvh_one(j->dim, (const osnch *)j->nodes, j->sils,
                                                   ((const osphere *)j->queries)[q],
                                                   ((const uint32_t *)j->aux)[q] != 0, j->f0, j->f1);
                break;
            case 7: {
                const of3 *pts = (const of3 *)j->queries;
                int r = contains_one(j->dim, j->snch, j->nodes, j->prims, pts[q]);
                j->u32out[q] = r < 0 ? 2u : (uint32_t)r;
                break;
            }
            case 8: {
                const of3 *a = (const of3 *)j->queries, *b = (const of3 *)j->aux;
                j->u32out[q] = (uint32_t)line_of_sight_one(j->dim, j->snch, j->nodes, j->prims, a[q], b[q]);
                break;
            }
            case 6: j->out[q] = sphere_sample_bvh_one(j->dim, j->snch, j->nodes, j->prims,
                                                      ((const osphere *)j->queries)[q], ((const of3 *)j->aux)[q],
                                                      &j->hits[q]);
                break;
            default: break;
        }
    }
}

static void *thread_main(void *arg) {
    run_range((ojob *)arg);
    return 0;
}

static int run_threaded(ojob proto, uint32_t n, int nthreads) {
    ojob *jobs;
    pthread_t *th;
    char *started;
    int t;
    if (n == 0) return 0;
    if (nthreads < 1) nthreads = 1;
    if ((uint32_t)nthreads > n) nthreads = (int)n;
    jobs = (ojob *)malloc(sizeof(ojob) * nthreads);
    th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    started = (char *)calloc(nthreads, 1);
    if (!jobs || !th || !started) { free(jobs); free(th); free(started); return 1; }
    for (t = 0; t < nthreads; t++) {
        jobs[t] = proto;
        jobs[t].begin = (uint32_t)((uint64_t)n * t / nthreads);
        jobs[t].end = (uint32_t)((uint64_t)n * (t + 1) / nthreads);
        if (t > 0 && pthread_create(&th[t], 0, thread_main, &jobs[t]) == 0) started[t] = 1;
    }
    run_range(&jobs[0]);
    for (t = 1; t < nthreads; t++) {
        if (started[t]) pthread_join(th[t], 0);
        else run_range(&jobs[t]);
    }
    free(jobs);
    free(th);
    free(started);
    return 0;
}

/* --------------------------------------------------------------- exports */
int oracle_closest_points_bvh(int dim, int snch, const void *nodes, const void *prims, const void *spheres,
                              uint32_t n, int recordNormal, void *out, uint32_t *nodesVisited, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 0; j.dim = dim; j.snch = snch; j.flag = recordNormal;
    j.nodes = nodes; j.prims = prims; j.queries = spheres; j.out = (oint *)out; j.u32out = nodesVisited;
    return run_threaded(j, n, nthreads);
}
/* the same with the GPU reference traversal's child order (closest_point_bvh_core) */
int oracle_closest_points_bvh_gpu_order(int dim, int snch, const void *nodes, const void *prims, const void *spheres,
                                        uint32_t n, void *out, uint32_t *nodesVisited, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 0; j.dim = dim; j.snch = snch; j.order = 1;
    j.nodes = nodes; j.prims = prims; j.queries = spheres; j.out = (oint *)out; j.u32out = nodesVisited;
    return run_threaded(j, n, nthreads);
}
int oracle_closest_points_brute(int dim, const void *prims, uint32_t nPrims, const void *spheres, uint32_t n,
                                void *out, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 1; j.dim = dim; j.prims = prims; j.nPrims = nPrims; j.queries = spheres; j.out = (oint *)out;
    return run_threaded(j, n, nthreads);
}
int oracle_closest_points_brute_f64(int dim, const void *prims, uint32_t nPrims, const void *spheres, uint32_t n,
                                    double *dist, uint32_t *index, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 2; j.dim = dim; j.prims = prims; j.nPrims = nPrims; j.queries = spheres;
    j.f64out = dist; j.u32out = index;
    return run_threaded(j, n, nthreads);
}
int oracle_intersect_rays_bvh(int dim, int snch, const void *nodes, const void *prims, const void *rays, uint32_t n,
                              int occl, void *out, int *hit, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 3; j.dim = dim; j.snch = snch; j.flag = occl; j.nodes = nodes; j.prims = prims; j.queries = rays;
    j.out = (oint *)out; j.hits = hit;
    return run_threaded(j, n, nthreads);
}
int oracle_intersect_rays_brute_f64(int dim, const void *prims, uint32_t nPrims, const void *rays, uint32_t n,
                                    double *t, uint32_t *index, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 4; j.dim = dim; j.prims = prims; j.nPrims = nPrims; j.queries = rays; j.f64out = t; j.u32out = index;
    return run_threaded(j, n, nthreads);
}
int oracle_silhouettes_bvh(int dim, const void *snchNodes, const void *sils, const void *spheres,
                           const uint32_t *flip, uint32_t n, float sqMinR, float precision, void *out, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 5; j.dim = dim; j.snch = 1; j.nodes = snchNodes; j.sils = sils; j.queries = spheres; j.aux = flip;
    j.f0 = sqMinR; j.f1 = precision; j.out = (oint *)out;
    return run_threaded(j, n, nthreads);
}
int oracle_sphere_sample_bvh(int dim, int snch, const void *nodes, const void *prims, const void *spheres,
                             const void *randNums, uint32_t n, void *out, int *hit, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 6; j.dim = dim; j.snch = snch; j.nodes = nodes; j.prims = prims; j.queries = spheres; j.aux = randNums;
    j.out = (oint *)out; j.hits = hit;
    return run_threaded(j, n, nthreads);
}
/* FP64 distance from x[q] to the primitive at array position pos[q] (tie checks) */
int oracle_prim_distance_f64(int dim, const void *prims, uint32_t nPrims, const uint32_t *pos, const float *x,
                             uint32_t n, double *out) {
    uint32_t q;
    for (q = 0; q < n; q++) {
        oprim pr;
        od3 c;
        if (pos[q] >= nPrims) { out[q] = INFINITY; continue; }
        pr = load_prim(dim, prims, pos[q]);
        c = dd3(x[3 * q], x[3 * q + 1], x[3 * q + 2]);
        out[q] = dim == 3 ? closest_point_triangle_f64(f2d(pr.pa), f2d(pr.pb), f2d(pr.pc), c)
                          : closest_point_segment_f64(f2d(pr.pa), f2d(pr.pb), c);
    }
    return 0;
}

int oracle_refit(int dim, int snch, void *nodes, const void *prims, const void *sils) {
    refit_rec(dim, snch, nodes, prims, sils, 0, 0);
    return 0;
}
int oracle_record_sizes(int *sizes) {
    sizes[0] = (int)sizeof(onode); sizes[1] = (int)sizeof(osnch); sizes[2] = (int)sizeof(otri);
    sizes[3] = (int)sizeof(oseg); sizes[4] = (int)sizeof(overt); sizes[5] = (int)sizeof(oedge);
    sizes[6] = (int)sizeof(osphere); sizes[7] = (int)sizeof(oray); sizes[8] = (int)sizeof(oint);
    return 9;
}

/* contains: out[q] = 1 inside, 0 outside, 2 if a ray had more than OHITS hits */
int oracle_contains_bvh(int dim, int snch, const void *nodes, const void *prims, const void *points, uint32_t n,
                        uint32_t *out, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 7; j.dim = dim; j.snch = snch; j.nodes = nodes; j.prims = prims; j.queries = points; j.u32out = out;
    return run_threaded(j, n, nthreads);
}

int oracle_line_of_sight_bvh(int dim, int snch, const void *nodes, const void *prims, const void *points_a,
                             const void *points_b, uint32_t n, uint32_t *out, int nthreads) {
    ojob j;
    memset(&j, 0, sizeof(j));
    j.kind = 8; j.dim = dim; j.snch = snch; j.nodes = nodes; j.prims = prims; j.queries = points_a;
    j.aux = points_b; j.u32out = out;
    return run_threaded(j, n, nthreads);
}

/* ------------------------------------------------------------------------
 * Sequential model of the device linear-BVH build (fcpwgb_gpu_scene_build).
 * The reference has no such builder (it builds with binned SAH on the host,
 * bvh.inl:40-234); this model states what the device build must produce so
 * that its output can be checked byte for byte: FP32 centroids
 * ((0 + v0 + v1 [+ v2]) * (1/dim)), Morton codes of 10 (3D) or 16 (2D) bits
 * per axis within the centroid bounds, primitives ordered by (code, index),
 * the binary radix tree over those keys defined top-down (a range splits
 * where the highest bit of (code, index) that differs inside it changes),
 * subtrees of at most max_leaf primitives as leaves, leaf boxes of the
 * vertices widened by FLT_EPSILON (bounding_volumes.h:38-49), pre-order node
 * records (inner: offset = 1 + nodes of the left subtree), primitives in leaf
 * order with their original index. */
typedef struct { uint64_t key; } okey;
static int cmp_key(const void *a, const void *b) {
    uint64_t x = ((const okey *)a)->key, y = ((const okey *)b)->key;
    return x < y ? -1 : (x > y ? 1 : 0);
}
static uint32_t spread_bits(uint32_t v, int dim) {
    uint32_t r = 0;
    for (int b = 0; b < (dim == 3 ? 10 : 16); b++)
        if (v & (1u << b)) r |= 1u << (b * dim);
    return r;
}
static int clz32(uint32_t v) {
    int n = 0;
    if (v == 0) return 32;
    while (!(v & 0x80000000u)) { v <<= 1; n++; }
    return n;
}
typedef struct {
    int dim;
    uint32_t n, max_leaf;
    const float *pos;
    const int32_t *idx;
    const uint32_t *codes, *order;
    onode *nodes;
    uint32_t count;
} olbvh;
static int lb_delta(const olbvh *b, uint32_t i, uint32_t j) {
    uint32_t a = b->codes[i], c = b->codes[j];
    return a != c ? clz32(a ^ c) : 32 + clz32(i ^ j);
}
static of3 lb_vertex(const olbvh *b, int32_t v) {
    const float *p = b->pos + (size_t)v * b->dim;
    return v3(p[0], p[1], b->dim == 3 ? p[2] : 0.0f);
}
/* emits the subtree over sorted positions [lo, hi]; returns its node count */
static uint32_t lb_emit(olbvh *b, uint32_t lo, uint32_t hi) {
    uint32_t me = b->count++;
    onode *nd = &b->nodes[me];
    if (hi - lo + 1 <= b->max_leaf) {
        float l[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, h[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t k = lo; k <= hi; k++) {
            uint32_t p = b->order[k];
            for (int j = 0; j < b->dim; j++) {
                of3 v = lb_vertex(b, b->idx[(size_t)p * b->dim + j]);
                for (int a = 0; a < b->dim; a++) {
                    float c = comp(v, a);
                    l[a] = minf_(l[a], c - FLT_EPSILON);
                    h[a] = maxf_(h[a], c + FLT_EPSILON);
                }
            }
        }
        if (b->dim == 2) l[2] = h[2] = 0.0f;
        b->nodes[me].pMin = v3(l[0], l[1], l[2]);
        b->nodes[me].pMax = v3(h[0], h[1], h[2]);
        b->nodes[me].nPrims = hi - lo + 1;
        b->nodes[me].offset = lo;
        return 1;
    }
    int common = lb_delta(b, lo, hi);
    uint32_t s = lo, e = hi; /* last position whose key shares more than `common` bits with lo */
    while (e - s > 1) {
        uint32_t m = s + (e - s) / 2;
        if (lb_delta(b, lo, m) > common) s = m;
        else e = m;
    }
    uint32_t nl = lb_emit(b, lo, s);
    uint32_t left = me + 1, right = b->count;
    uint32_t nr = lb_emit(b, s + 1, hi);
    nd = &b->nodes[me];
    const onode *L = &b->nodes[left], *R = &b->nodes[right];
    nd->pMin = v3(minf_(L->pMin.x, R->pMin.x), minf_(L->pMin.y, R->pMin.y), minf_(L->pMin.z, R->pMin.z));
    nd->pMax = v3(maxf_(L->pMax.x, R->pMax.x), maxf_(L->pMax.y, R->pMax.y), maxf_(L->pMax.z, R->pMax.z));
    nd->nPrims = 0;
    nd->offset = 1 + nl;
    return 1 + nl + nr;
}
/* nodes_out: room for 2n - 1 records; prims_out: n triangles (3D) or segments
 * (2D); prim_verts_out: n * dim. Returns the node count (0 on bad input). */
uint32_t oracle_lbvh_build(int dim, const float *pos, const int32_t *idx, uint32_t n, uint32_t max_leaf,
                           void *nodes_out, void *prims_out, int32_t *prim_verts_out) {
    if (n == 0 || max_leaf == 0) return 0;
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    of3 *cent = (of3 *)malloc(sizeof(of3) * n);
    uint32_t *codes = (uint32_t *)malloc(sizeof(uint32_t) * n), *order = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint32_t *sorted = (uint32_t *)malloc(sizeof(uint32_t) * n);
    okey *keys = (okey *)malloc(sizeof(okey) * n);
    olbvh b;
    for (uint32_t p = 0; p < n; p++) {
        of3 c = v3(0.0f, 0.0f, 0.0f);
        for (int j = 0; j < dim; j++) {
            const float *v = pos + (size_t)idx[(size_t)p * dim + j] * dim;
            c = add3(c, v3(v[0], v[1], dim == 3 ? v[2] : 0.0f));
        }
        c = mul3(c, 1.0f / (float)dim);
        cent[p] = c;
        for (int a = 0; a < 3; a++) {
            lo[a] = fminf(lo[a], comp(c, a));
            hi[a] = fmaxf(hi[a], comp(c, a));
        }
    }
    const float cells = dim == 3 ? 1024.0f : 65536.0f;
    for (uint32_t p = 0; p < n; p++) {
        uint32_t q[3];
        for (int a = 0; a < 3; a++) {
            float t = (comp(cent[p], a) - lo[a]) / fmaxf(hi[a] - lo[a], 1e-30f) * cells;
            q[a] = (uint32_t)fminf(fmaxf(t, 0.0f), cells - 1.0f);
        }
        codes[p] = dim == 3 ? (spread_bits(q[0], 3) | (spread_bits(q[1], 3) << 1) | (spread_bits(q[2], 3) << 2))
                            : (spread_bits(q[0], 2) | (spread_bits(q[1], 2) << 1));
        keys[p].key = ((uint64_t)codes[p] << 32) | p;
    }
    qsort(keys, n, sizeof(okey), cmp_key);
    for (uint32_t k = 0; k < n; k++) {
        order[k] = (uint32_t)(keys[k].key & 0xffffffffu);
        sorted[k] = (uint32_t)(keys[k].key >> 32);
    }
    b.dim = dim; b.n = n; b.max_leaf = max_leaf; b.pos = pos; b.idx = idx; b.codes = sorted; b.order = order;
    b.nodes = (onode *)nodes_out; b.count = 0;
    lb_emit(&b, 0, n - 1);
    for (uint32_t k = 0; k < n; k++) {
        uint32_t p = order[k];
        of3 v[3];
        for (int j = 0; j < dim; j++) {
            prim_verts_out[(size_t)k * dim + j] = idx[(size_t)p * dim + j];
            v[j] = lb_vertex(&b, idx[(size_t)p * dim + j]);
        }
        if (dim == 3) {
            otri *t = (otri *)prims_out + k;
            t->pa = v[0]; t->pb = v[1]; t->pc = v[2]; t->index = p;
        } else {
            oseg *s = (oseg *)prims_out + k;
            s->pa = v[0]; s->pb = v[1]; s->index = p;
        }
    }
    free(cent); free(codes); free(order); free(sorted); free(keys);
    return b.count;
}

/* ------------------------------------------------------------------------
 * Scenes of several objects and instances (Scene::build, fcpw.inl:1053-1102):
 * a top-level Bvh whose leaves are aggregates (bvh.inl:1291-1418 and 655-771
 * with primitiveTypeIsAggregate), an untransformed object queried as it is,
 * an instance through TransformedAggregate (core/primitive.h:289-478): the
 * query mapped to object space with tInv (BoundingSphere::transform,
 * bounding_volumes.h:13-24; Ray::transform, ray.h:19-25), the answer mapped
 * back with t (Interaction::applyTransform, interaction.h:52-60). With a
 * single instance the instance is the scene's aggregate (no top-level tree).
 * Transform arithmetic as the affine Transform of the Eigen API the
 * reference is compiled against here: row i of t*p is
 * t(i,D) + t(i,0)*p0 + t(i,1)*p1 [+ t(i,2)*p2], in that order.
 * Matrices: 24 floats per instance, the 3x4 rows of t then of tInv (2D: the
 * translation in column 3). */
typedef struct {
    const float *t, *ti;
    uint32_t object, transformed;
} oinst;

static of3 xf_point(int dim, const float *m, of3 p) {
    float r[3] = {0.0f, 0.0f, 0.0f};
    int i;
    for (i = 0; i < dim; i++) {
        float acc = m[i * 4 + 3];
        acc += m[i * 4 + 0] * p.x;
        acc += m[i * 4 + 1] * p.y;
        if (dim == 3) acc += m[i * 4 + 2] * p.z;
        r[i] = acc;
    }
    return v3(r[0], r[1], dim == 3 ? r[2] : 0.0f);
}

static osphere xf_sphere(int dim, const float *m, osphere s) {
    osphere o;
    o.c = xf_point(dim, m, s.c);
    o.r2 = OMAXF;
    if (s.r2 < OMAXF) {
        of3 e = v3(s.c.x + sqrtf(s.r2), s.c.y + 0.0f, s.c.z + 0.0f);
        of3 d = sub3(xf_point(dim, m, e), o.c);
        o.r2 = dotd(dim, d, d);
    }
    return o;
}

static oray xf_ray(int dim, const float *m, oray r) {
    of3 to = xf_point(dim, m, r.o);
    float s = r.tMax < OMAXF ? r.tMax : 1.0f;
    of3 td = sub3(xf_point(dim, m, add3(r.o, mul3(r.d, s))), to);
    float nrm = sqrtf(dotd(dim, td, td));
    return make_ray(dim, to, div3(td, nrm), r.tMax < OMAXF ? nrm : OMAXF);
}

static void xf_interaction(int dim, const oinst *in, of3 query, oint *c) {
    float r[3] = {0.0f, 0.0f, 0.0f}, z;
    of3 d, n;
    int i;
    c->p = xf_point(dim, in->t, c->p);
    d = sub3(c->p, query);
    c->d = sqrtf(dotd(dim, d, d));
    /* Transform(tInv^T) * n: row i is tInv(D, i) = 0 plus the column sums */
    for (i = 0; i < dim; i++) {
        float acc = 0.0f;
        acc += in->ti[0 * 4 + i] * c->n.x;
        acc += in->ti[1 * 4 + i] * c->n.y;
        if (dim == 3) acc += in->ti[2 * 4 + i] * c->n.z;
        r[i] = acc;
    }
    n = v3(r[0], r[1], dim == 3 ? r[2] : 0.0f);
    z = dotd(dim, n, n);
    if (z > 0.0f) n = div3(n, sqrtf(z));
    c->n = n;
}

static int inst_closest(int dim, const oinst *in, const void *const *objNodes, const void *const *objPrims,
                        osphere *s, int recordNormal, oint *c) {
    const void *nodes = objNodes[in->object], *prims = objPrims[in->object];
    osphere sInv;
    int found;
    if (!in->transformed) return closest_point_bvh_core(dim, 0, nodes, prims, s, recordNormal, c, NULL, 0);
    sInv = xf_sphere(dim, in->ti, *s);
    found = closest_point_bvh_core(dim, 0, nodes, prims, &sInv, recordNormal, c, NULL, 0);
    s->r2 = xf_sphere(dim, in->t, sInv).r2;
    if (found) xf_interaction(dim, in, s->c, c);
    return found;
}

static int inst_ray(int dim, const oinst *in, const void *const *objNodes, const void *const *objPrims, oray *r,
                    int occl, oint *c) {
    const void *nodes = objNodes[in->object], *prims = objPrims[in->object];
    oray rInv;
    int hit;
    if (!in->transformed) return ray_bvh_core(dim, 0, nodes, prims, r, occl, c);
    rInv = xf_ray(dim, in->ti, *r);
    hit = ray_bvh_core(dim, 0, nodes, prims, &rInv, occl, c);
    r->tMax = xf_ray(dim, in->t, rInv).tMax;
    if (hit) xf_interaction(dim, in, r->o, c);
    return hit;
}

static oinst inst_of(const float *mats, const uint32_t *object, const uint32_t *transformed, uint32_t k) {
    oinst in;
    in.t = mats + (size_t)k * 24;
    in.ti = mats + (size_t)k * 24 + 12;
    in.object = object[k];
    in.transformed = transformed[k];
    return in;
}

/* out: n interactions; inst_out: the instance of each answer (OUMAX: none) */
int oracle_instanced_closest_points(int dim, const void *topNodes, const uint32_t *topRefs, uint32_t nInst,
                                    const float *mats, const uint32_t *object, const uint32_t *transformed,
                                    const void *const *objNodes, const void *const *objPrims, const void *spheres,
                                    uint32_t n, int recordNormal, void *out, uint32_t *instOut) {
    uint32_t q;
    for (q = 0; q < n; q++) {
        osphere s = ((const osphere *)spheres)[q];
        oint best = default_interaction();
        uint32_t bi = OUMAX;
        if (nInst == 1) {
            oinst in = inst_of(mats, object, transformed, 0);
            oint c = default_interaction();
            if (inst_closest(dim, &in, objNodes, objPrims, &s, recordNormal, &c)) { best = c; bi = 0; }
        } else {
            uint32_t stackNode[OSTACK];
            float stackDist[OSTACK], bh[4];
            obox root = load_node(0, topNodes, 0);
            box_sq_dist(dim, root.pMin, root.pMax, s.c, &bh[0], &bh[1]);
            if (bh[0] <= s.r2) {
                int sp = 0;
                s.r2 = minf_(s.r2, bh[1]);
                stackNode[0] = 0;
                stackDist[0] = bh[0];
                while (sp >= 0) {
                    uint32_t ni = stackNode[sp];
                    float cur = stackDist[sp];
                    obox node;
                    sp--;
                    if (cur > s.r2) continue;
                    node = load_node(0, topNodes, ni);
                    if (node.nPrims > 0) {
                        uint32_t p;
                        for (p = 0; p < node.nPrims; p++) {
                            uint32_t k = topRefs[node.offset + p];
                            oinst in = inst_of(mats, object, transformed, k);
                            oint c = default_interaction();
                            if (inst_closest(dim, &in, objNodes, objPrims, &s, recordNormal, &c)) {
                                s.r2 = minf_(s.r2, c.d * c.d);
                                best = c;
                                bi = k;
                            }
                        }
                    } else {
                        uint32_t li = ni + 1, ri = ni + node.offset, closer, other;
                        obox l = load_node(0, topNodes, li), r = load_node(0, topNodes, ri);
                        int hit0, hit1;
                        box_sq_dist(dim, l.pMin, l.pMax, s.c, &bh[0], &bh[1]);
                        hit0 = bh[0] <= s.r2;
                        s.r2 = minf_(s.r2, bh[1]);
                        box_sq_dist(dim, r.pMin, r.pMax, s.c, &bh[2], &bh[3]);
                        hit1 = bh[2] <= s.r2;
                        s.r2 = minf_(s.r2, bh[3]);
                        if (hit0 && hit1) {
                            closer = li; other = ri;
                            if (bh[0] == 0.0f && bh[2] == 0.0f) {
                                if (bh[3] < bh[1]) { closer = ri; other = li; }
                            } else if (bh[2] < bh[0]) {
                                float t = bh[0]; bh[0] = bh[2]; bh[2] = t;
                                closer = ri; other = li;
                            }
                            sp++; stackNode[sp] = other; stackDist[sp] = bh[2];
                            sp++; stackNode[sp] = closer; stackDist[sp] = bh[0];
                        } else if (hit0) {
                            sp++; stackNode[sp] = li; stackDist[sp] = bh[0];
                        } else if (hit1) {
                            sp++; stackNode[sp] = ri; stackDist[sp] = bh[2];
                        }
                    }
                }
            }
        }
        ((oint *)out)[q] = best;
        if (instOut) instOut[q] = bi;
    }
    return 0;
}

/* hit: 1 when the ray hit (with occl: is occluded) */
int oracle_instanced_rays(int dim, const void *topNodes, const uint32_t *topRefs, uint32_t nInst,
                          const float *mats, const uint32_t *object, const uint32_t *transformed,
                          const void *const *objNodes, const void *const *objPrims, const void *rays, uint32_t n,
                          int occl, void *out, int *hitOut, uint32_t *instOut) {
    uint32_t q;
    for (q = 0; q < n; q++) {
        oray r = ((const oray *)rays)[q];
        oint best = default_interaction();
        uint32_t bi = OUMAX;
        int didHit = 0;
        r = make_ray(dim, r.o, r.d, r.tMax);
        if (nInst == 1) {
            oinst in = inst_of(mats, object, transformed, 0);
            oint c = default_interaction();
            if (inst_ray(dim, &in, objNodes, objPrims, &r, occl, &c)) { best = c; bi = 0; didHit = 1; }
        } else {
            uint32_t stackNode[OSTACK];
            float stackDist[OSTACK], bh[4];
            obox root = load_node(0, topNodes, 0);
            if (box_ray(dim, root.pMin, root.pMax, &r, &bh[0], &bh[1])) {
                int sp = 0, done = 0;
                stackNode[0] = 0;
                stackDist[0] = bh[0];
                while (sp >= 0 && !done) {
                    uint32_t ni = stackNode[sp];
                    float cur = stackDist[sp];
                    obox node;
                    sp--;
                    if (cur > r.tMax) continue;
                    node = load_node(0, topNodes, ni);
                    if (node.nPrims > 0) {
                        uint32_t p;
                        for (p = 0; p < node.nPrims; p++) {
                            uint32_t k = topRefs[node.offset + p];
                            oinst in = inst_of(mats, object, transformed, k);
                            oint c = default_interaction();
                            if (inst_ray(dim, &in, objNodes, objPrims, &r, occl, &c)) {
                                didHit = 1;
                                bi = k;
                                best = c;
                                if (occl) { done = 1; break; }
                                r.tMax = minf_(r.tMax, c.d);
                            }
                        }
                    } else {
                        uint32_t li = ni + 1, ri = ni + node.offset;
                        obox l = load_node(0, topNodes, li), rr = load_node(0, topNodes, ri);
                        int hit0 = box_ray(dim, l.pMin, l.pMax, &r, &bh[0], &bh[1]);
                        int hit1 = box_ray(dim, rr.pMin, rr.pMax, &r, &bh[2], &bh[3]);
                        if (hit0 && hit1) {
                            uint32_t closer = li, other = ri;
                            if (bh[2] < bh[0]) {
                                float t = bh[0]; bh[0] = bh[2]; bh[2] = t;
                                t = bh[1]; bh[1] = bh[3]; bh[3] = t;
                                closer = ri; other = li;
                            }
                            sp++; stackNode[sp] = other; stackDist[sp] = bh[2];
                            sp++; stackNode[sp] = closer; stackDist[sp] = bh[0];
                        } else if (hit0) {
                            sp++; stackNode[sp] = li; stackDist[sp] = bh[0];
                        } else if (hit1) {
                            sp++; stackNode[sp] = ri; stackDist[sp] = bh[2];
                        }
                    }
                }
            }
        }
        ((oint *)out)[q] = best;
        if (hitOut) hitOut[q] = didHit;
        if (instOut) instOut[q] = bi;
    }
    return 0;
}
