/*
 * toast_oracle.c -- CPU restatement of the Toast++ FEM diffusion forward path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the tests, the
 * smoke check and the CPU-baseline leg of bench.py call it to check (and to
 * time beside) the CUDA path.  No product code links or calls it.
 *
 * Each function restates the reference algorithm it cites (paths are within
 * the toastpp project).  Floating-point operation order follows the reference
 * wherever it is cheap to do so, so that results agree with the reference to
 * round-off.  Parity is pinned in tests/ against the reference's shipped golden
 * vectors (test/2D/fwdfem/testdata.zip, test/3D/fwdfem/testdata.zip) and
 * against the reference compiled from source (oracle/Makefile.ref).
 *
 * Conventions: node and element indices are 0-based; complex arrays are
 * interleaved (re, im) doubles; matrices are CSR with sorted columns.
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex zd;

/* ------------------------------------------------------------------------ */
/* Mesh                                                                      */
/* ------------------------------------------------------------------------ */

typedef struct {
    int dim, n, ne, nn;       /* nn = nodes per element (3 Tri3, 4 Tet4) */
    double *x;                /* n*dim */
    int *el;                  /* ne*nn */
    double *geo;              /* per element: Tri3 a0..2 b0..2 c0..2 ; Tet4 a,b,c,d (16) */
    double *size;             /* ne */
    double *side_size;        /* Tet4: ne*4 face areas */
    unsigned char *bndside;   /* ne*nside */
    unsigned char *bndnode;   /* n */
    double *intdd;            /* ne*nn*nn */
    double *intbff;           /* ne*nn*nn */
    int *rowptr, *colidx;     /* CSR pattern */
    int nnz;
} tor_mesh;

static const int TRI_SN[3][2] = {{0, 1}, {1, 2}, {2, 0}};              /* tri3.cc:123-127 */
static const int TET_SN[4][3] = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}}; /* tet4.cc:175-181 */

static double pt_dist(const double *a, const double *b, int dim)
{   /* point.cc:33-41 */
    double d2 = 0.0;
    for (int i = 0; i < dim; i++) d2 += (a[i] - b[i]) * (a[i] - b[i]);
    return sqrt(d2);
}

/* Triangle3::Initialise (tri3.cc:79-88) and Tetrahedron4::Initialise
   (tet4.cc:113-141): geometry coefficients and size. */
static void element_geometry(tor_mesh *m, int e)
{
    const int *nd = m->el + (size_t)e * m->nn;
    double *g = m->geo + (size_t)e * 16;
    if (m->dim == 2) {
        double x0 = m->x[2 * nd[0]], y0 = m->x[2 * nd[0] + 1];
        double x1 = m->x[2 * nd[1]], y1 = m->x[2 * nd[1] + 1];
        double x2 = m->x[2 * nd[2]], y2 = m->x[2 * nd[2] + 1];
        g[0] = x1 * y2 - x2 * y1; g[3] = y1 - y2; g[6] = x2 - x1;
        g[1] = x2 * y0 - x0 * y2; g[4] = y2 - y0; g[7] = x0 - x2;
        g[2] = x0 * y1 - x1 * y0; g[5] = y0 - y1; g[8] = x1 - x0;
        m->size[e] = 0.5 * (g[0] + g[1] + g[2]);  /* tri3.cc:184-189 */
    } else {
        const double *p0 = m->x + 3 * nd[0], *p1 = m->x + 3 * nd[1];
        const double *p2 = m->x + 3 * nd[2], *p3 = m->x + 3 * nd[3];
        double x0 = p0[0], y0 = p0[1], z0 = p0[2], x1 = p1[0], y1 = p1[1], z1 = p1[2];
        double x2 = p2[0], y2 = p2[1], z2 = p2[2], x3 = p3[0], y3 = p3[1], z3 = p3[2];
        double *a = g, *b = g + 4, *c = g + 8, *d = g + 12;
        a[0] = x1*(y2*z3-y3*z2) - x2*(y1*z3-y3*z1) + x3*(y1*z2-y2*z1);
        a[1] = x0*(y3*z2-y2*z3) - x2*(y3*z0-y0*z3) + x3*(y2*z0-y0*z2);
        a[2] = x0*(y1*z3-y3*z1) - x1*(y0*z3-y3*z0) + x3*(y0*z1-y1*z0);
        a[3] = x0*(y2*z1-y1*z2) - x1*(y2*z0-y0*z2) + x2*(y1*z0-y0*z1);
        b[0] = y1*(z3-z2) + y2*(z1-z3) + y3*(z2-z1);
        b[1] = y0*(z2-z3) + y2*(z3-z0) + y3*(z0-z2);
        b[2] = y0*(z3-z1) + y1*(z0-z3) + y3*(z1-z0);
        b[3] = y0*(z1-z2) + y1*(z2-z0) + y2*(z0-z1);
        c[0] = x1*(z2-z3) + x2*(z3-z1) + x3*(z1-z2);
        c[1] = x0*(z3-z2) + x2*(z0-z3) + x3*(z2-z0);
        c[2] = x0*(z1-z3) + x1*(z3-z0) + x3*(z0-z1);
        c[3] = x0*(z2-z1) + x1*(z0-z2) + x2*(z1-z0);
        d[0] = x1*(y3-y2) + x2*(y1-y3) + x3*(y2-y1);
        d[1] = x0*(y2-y3) + x2*(y3-y0) + x3*(y0-y2);
        d[2] = x0*(y3-y1) + x1*(y0-y3) + x3*(y1-y0);
        d[3] = x0*(y1-y2) + x1*(y2-y0) + x2*(y0-y1);
        for (int sd = 0; sd < 4; sd++) {  /* TriangleArea, tet4.cc:15-25 */
            const double *q1 = m->x + 3 * nd[TET_SN[sd][0]];
            const double *q2 = m->x + 3 * nd[TET_SN[sd][1]];
            const double *q3 = m->x + 3 * nd[TET_SN[sd][2]];
            double aa = pt_dist(q1, q2, 3), bb = pt_dist(q2, q3, 3), cc = pt_dist(q3, q1, 3);
            double s = 0.5 * (aa + bb + cc);
            m->side_size[(size_t)e * 4 + sd] = sqrt(s * (s - aa) * (s - bb) * (s - cc));
        }
        m->size[e] = (1.0 / 6.0) * (a[0] + a[1] + a[2] + a[3]);  /* tet4.cc:1010-1013 */
    }
}

typedef struct { int nd[3]; int el, sd; } siderec;

static int side_cmp(const void *a, const void *b)
{
    const siderec *s1 = a, *s2 = b;
    for (int k = 0; k < 3; k++) {
        if (s1->nd[k] < s2->nd[k]) return -1;
        if (s1->nd[k] > s2->nd[k]) return 1;
    }
    return 0;
}

/* Mesh::MarkBoundary (mesh.cc:1614-1705): a side is on the boundary when no
   other element shares it; its nodes become boundary nodes. */
static void mark_boundary(tor_mesh *m)
{
    int nside = m->dim == 2 ? 3 : 4, nsn = m->dim == 2 ? 2 : 3;
    size_t slen = (size_t)m->ne * nside;
    siderec *sd = malloc(slen * sizeof(siderec));
    for (int e = 0; e < m->ne; e++)
        for (int s = 0; s < nside; s++) {
            siderec *r = sd + (size_t)e * nside + s;
            r->el = e; r->sd = s; r->nd[2] = -1;
            for (int k = 0; k < nsn; k++)
                r->nd[k] = m->el[(size_t)e * m->nn + (m->dim == 2 ? TRI_SN[s][k] : TET_SN[s][k])];
            for (int j = 0; j < nsn - 1; j++)
                for (int k = j + 1; k < nsn; k++)
                    if (r->nd[j] > r->nd[k]) { int t = r->nd[j]; r->nd[j] = r->nd[k]; r->nd[k] = t; }
        }
    qsort(sd, slen, sizeof(siderec), side_cmp);
    memset(m->bndnode, 0, m->n);
    memset(m->bndside, 0, slen);
    for (size_t i = 0; i < slen; i++) {
        int isbnd = 1;
        if (i > 0 && side_cmp(sd + i, sd + i - 1) == 0) isbnd = 0;
        if (isbnd && i + 1 < slen && side_cmp(sd + i, sd + i + 1) == 0) isbnd = 0;
        if (isbnd) {
            m->bndside[(size_t)sd[i].el * nside + sd[i].sd] = 1;
            for (int k = 0; k < nsn; k++) m->bndnode[sd[i].nd[k]] = 1;
        }
    }
    free(sd);
}

/* Element_Unstructured::PostInitialisation (element.cc:540-545):
   intdd = ComputeIntDD, intbff = ComputeBndIntFF. */
static void element_tables(tor_mesh *m, int e)
{
    int nn = m->nn;
    double *dd = m->intdd + (size_t)e * nn * nn, *bff = m->intbff + (size_t)e * nn * nn;
    const double *g = m->geo + (size_t)e * 16;
    double sz = m->size[e];
    memset(bff, 0, sizeof(double) * nn * nn);
    if (m->dim == 2) {
        const double *b = g + 3, *c = g + 6;
        double scale = 0.25 / sz;  /* tri3.cc:490-506 */
        for (int i = 0; i < 3; i++)
            for (int j = 0; j <= i; j++)
                dd[i * 3 + j] = dd[j * 3 + i] = scale * (b[i] * b[j] + c[i] * c[j]);
        const int *nd = m->el + (size_t)e * 3;
        for (int s = 0; s < 3; s++) {  /* tri3.cc:561-582 */
            if (!m->bndside[(size_t)e * 3 + s]) continue;
            int n0 = TRI_SN[s][0], n1 = TRI_SN[s][1];
            double dx = m->x[2 * nd[n0]] - m->x[2 * nd[n1]];
            double dy = m->x[2 * nd[n0] + 1] - m->x[2 * nd[n1] + 1];
            double d = hypot(dx, dy);
            for (int i = 0; i < 3; i++) {
                if (i != n0 && i != n1) continue;
                bff[i * 3 + i] += d / 3.0;
                for (int j = 0; j < i; j++)
                    if (j == n0 || j == n1) bff[i * 3 + j] += d / 6.0;
            }
        }
        for (int i = 0; i < 3; i++) for (int j = 0; j < i; j++) bff[j * 3 + i] = bff[i * 3 + j];
    } else {
        const double *b = g + 4, *c = g + 8, *d = g + 12;
        double scale = 1.0 / (36.0 * sz);  /* tet4.cc:1016-1031 */
        for (int i = 0; i < 4; i++)
            for (int j = 0; j <= i; j++)
                dd[i * 4 + j] = dd[j * 4 + i] = scale * (b[j] * b[i] + c[j] * c[i] + d[j] * d[i]);
        /* ComputeBndIntFF (tet4.cc:1109-1122) with sym_bndintff tables (1039-1068) */
        static const int T[4][4][4] = {
            {{2,1,1,0},{1,2,1,0},{1,1,2,0},{0,0,0,0}},
            {{2,1,0,1},{1,2,0,1},{0,0,0,0},{1,1,0,2}},
            {{2,0,1,1},{0,0,0,0},{1,0,2,1},{1,0,1,2}},
            {{0,0,0,0},{0,2,1,1},{0,1,2,1},{0,1,1,2}}};
        for (int s = 0; s < 4; s++) {
            if (!m->bndside[(size_t)e * 4 + s]) continue;
            double ss = m->side_size[(size_t)e * 4 + s];
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++)
                    bff[i * 4 + j] += (T[s][i][j] * (2.0 / 24.0)) * ss;
        }
    }
}

typedef struct { int n1, n2; } ipair;
static int ipair_cmp(const void *a, const void *b)
{
    const ipair *p = a, *q = b;
    if (p->n1 != q->n1) return p->n1 < q->n1 ? -1 : 1;
    if (p->n2 != q->n2) return p->n2 < q->n2 ? -1 : 1;
    return 0;
}

/* Mesh::SparseRowStructure (mesh.cc:422-549): all node pairs that share an
   element, sorted by (row, col) and deduplicated, diagonal included. */
static void csr_pattern(tor_mesh *m)
{
    size_t np = (size_t)m->ne * m->nn * m->nn, p = 0;
    ipair *pr = malloc(np * sizeof(ipair));
    for (int e = 0; e < m->ne; e++)
        for (int i = 0; i < m->nn; i++)
            for (int j = 0; j < m->nn; j++) {
                pr[p].n1 = m->el[(size_t)e * m->nn + i];
                pr[p].n2 = m->el[(size_t)e * m->nn + j];
                p++;
            }
    qsort(pr, np, sizeof(ipair), ipair_cmp);
    size_t nz = 0;
    for (size_t i = 0; i < np; i++)
        if (i == 0 || ipair_cmp(pr + i, pr + nz - 1) != 0) pr[nz++] = pr[i];
    m->nnz = (int)nz;
    m->rowptr = calloc(m->n + 1, sizeof(int));
    m->colidx = malloc(nz * sizeof(int));
    for (size_t i = 0; i < nz; i++) { m->rowptr[pr[i].n1 + 1]++; m->colidx[i] = pr[i].n2; }
    for (int i = 0; i < m->n; i++) m->rowptr[i + 1] += m->rowptr[i];
    free(pr);
}

tor_mesh *tor_mesh_create(int dim, int n, const double *coords, int ne, const int *elnodes)
{
    tor_mesh *m = calloc(1, sizeof(tor_mesh));
    m->dim = dim; m->n = n; m->ne = ne; m->nn = dim == 2 ? 3 : 4;
    int nside = dim == 2 ? 3 : 4;
    m->x = malloc(sizeof(double) * n * dim);
    memcpy(m->x, coords, sizeof(double) * n * dim);
    m->el = malloc(sizeof(int) * ne * m->nn);
    memcpy(m->el, elnodes, sizeof(int) * ne * m->nn);
    m->geo = calloc((size_t)ne * 16, sizeof(double));
    m->size = calloc(ne, sizeof(double));
    m->side_size = calloc((size_t)ne * 4, sizeof(double));
    m->bndside = calloc((size_t)ne * nside, 1);
    m->bndnode = calloc(n, 1);
    m->intdd = calloc((size_t)ne * m->nn * m->nn, sizeof(double));
    m->intbff = calloc((size_t)ne * m->nn * m->nn, sizeof(double));
    for (int e = 0; e < ne; e++) element_geometry(m, e);  /* Mesh::Setup, mesh.cc:96-158 */
    mark_boundary(m);
    for (int e = 0; e < ne; e++) element_tables(m, e);
    csr_pattern(m);
    return m;
}

void tor_mesh_free(tor_mesh *m)
{
    if (!m) return;
    free(m->x); free(m->el); free(m->geo); free(m->size); free(m->side_size);
    free(m->bndside); free(m->bndnode); free(m->intdd); free(m->intbff);
    free(m->rowptr); free(m->colidx); free(m);
}

int tor_mesh_nnz(const tor_mesh *m) { return m->nnz; }
void tor_mesh_csr(const tor_mesh *m, int *rowptr, int *colidx)
{
    memcpy(rowptr, m->rowptr, sizeof(int) * (m->n + 1));
    memcpy(colidx, m->colidx, sizeof(int) * m->nnz);
}
void tor_mesh_bndnodes(const tor_mesh *m, unsigned char *out) { memcpy(out, m->bndnode, m->n); }
void tor_mesh_elsize(const tor_mesh *m, double *out) { memcpy(out, m->size, sizeof(double) * m->ne); }

/* ------------------------------------------------------------------------ */
/* Element integrals                                                          */
/* ------------------------------------------------------------------------ */

/* Triangle3::IntPFF (tri3.cc:325-353) */
static double tri_intpff(const tor_mesh *m, int e, int i, int j, const double *P)
{
    const int *nd = m->el + (size_t)e * 3;
    static const double i30 = 1.0 / 30.0;
    double sz = m->size[e];
    double p0 = P[nd[0]], p1 = P[nd[1]], p2 = P[nd[2]];
    if (i < j) { int t = i; i = j; j = t; }
    switch (i * 3 + j) {
    case 0: return sz * i30 * (3.0 * p0 + p1 + p2);
    case 3: return sz * i30 * (p0 + p1 + 0.5 * p2);
    case 4: return sz * i30 * (p0 + 3.0 * p1 + p2);
    case 6: return sz * i30 * (p0 + 0.5 * p1 + p2);
    case 7: return sz * i30 * (0.5 * p0 + p1 + p2);
    default: return sz * i30 * (p0 + p1 + 3.0 * p2);
    }
}

/* 4x4 planes of the Tet4 IntFFF tensor (tet4.cc:49-77), scaled by 1/120 */
static const int TET_FFF[4][4][4] = {
    {{6,2,2,2},{2,2,1,1},{2,1,2,1},{2,1,1,2}},
    {{2,2,1,1},{2,6,2,2},{1,2,2,1},{1,2,1,2}},
    {{2,1,2,1},{1,2,2,1},{2,2,6,2},{1,1,2,2}},
    {{2,1,1,2},{1,2,1,2},{1,1,2,2},{2,2,2,6}}};

/* Tetrahedron4::IntPFF (tet4.cc:371-378) */
static double tet_intpff(const tor_mesh *m, int e, int i, int j, const double *P)
{
    const int *nd = m->el + (size_t)e * 4;
    return (TET_FFF[0][i][j] / 120.0 * P[nd[0]] + TET_FFF[1][i][j] / 120.0 * P[nd[1]] +
            TET_FFF[2][i][j] / 120.0 * P[nd[2]] + TET_FFF[3][i][j] / 120.0 * P[nd[3]]) * m->size[e];
}

/* Tetrahedron4::IntFDD (tet4.cc:380-412), independent of the first index */
static double tet_intfdd(const tor_mesh *m, int e, int j, int k)
{
    if (j > k) { int t = j; j = k; k = t; }
    const double *g = m->geo + (size_t)e * 16;
    const double *b = g + 4, *c = g + 8, *d = g + 12;
    double scale = 1.0 / (144.0 * m->size[e]);
    return (b[j] * b[k] + c[j] * c[k] + d[j] * d[k]) * scale;
}

/* Element IntPDD: tri3.h:208-209 and tet4.cc:414-419 */
static double el_intpdd(const tor_mesh *m, int e, int i, int j, const double *P)
{
    const int *nd = m->el + (size_t)e * m->nn;
    if (m->dim == 2)
        return m->intdd[(size_t)e * 9 + i * 3 + j] * ((P[nd[0]] + P[nd[1]] + P[nd[2]]) / 3.0);
    double res = 0.0;
    for (int k = 0; k < 4; k++) res += P[nd[k]];
    return res * tet_intfdd(m, e, i, j);
}

/* Element BndIntPFF: tri3.h:217-218 (intbff x nodal mean) and tet4.cc:819-832
   (exact face integral) */
static const int TET_BFFF[4][4][4][4] = {
    { {{6,2,2,0},{2,2,1,0},{2,1,2,0},{0,0,0,0}}, {{2,2,1,0},{2,6,2,0},{1,2,2,0},{0,0,0,0}},
      {{2,1,2,0},{1,2,2,0},{2,2,6,0},{0,0,0,0}}, {{0}} },
    { {{6,2,0,2},{2,2,0,1},{0,0,0,0},{2,1,0,2}}, {{2,2,0,1},{2,6,0,2},{0,0,0,0},{1,2,0,2}},
      {{0}}, {{2,1,0,2},{1,2,0,2},{0,0,0,0},{2,2,0,6}} },
    { {{6,0,2,2},{0,0,0,0},{2,0,2,1},{2,0,1,2}}, {{0}},
      {{2,0,2,1},{0,0,0,0},{2,0,6,2},{1,0,2,2}}, {{2,0,1,2},{0,0,0,0},{1,0,2,2},{2,0,2,6}} },
    { {{0}}, {{0,0,0,0},{0,6,2,2},{0,2,2,1},{0,2,1,2}},
      {{0,0,0,0},{0,2,2,1},{0,2,6,2},{0,1,2,2}}, {{0,0,0,0},{0,2,1,2},{0,1,2,2},{0,2,2,6}} } };

static double el_bndintpff(const tor_mesh *m, int e, int i, int j, const double *P)
{
    const int *nd = m->el + (size_t)e * m->nn;
    if (m->dim == 2)
        return m->intbff[(size_t)e * 9 + i * 3 + j] * ((P[nd[0]] + P[nd[1]] + P[nd[2]]) / 3.0);
    double res = 0.0;
    int any = 0;
    for (int sd = 0; sd < 4; sd++) any |= m->bndside[(size_t)e * 4 + sd];
    if (!any) return 0.0;
    for (int sd = 0; sd < 4; sd++) {
        if (!m->bndside[(size_t)e * 4 + sd]) continue;
        double sres = 0.0;
        for (int k = 0; k < 4; k++) sres += P[nd[k]] * (TET_BFFF[sd][k][i][j] * (2.0 / 120.0));
        res += sres * m->side_size[(size_t)e * 4 + sd];
    }
    return res;
}

/* Element IntFF(i,j): tri3.cc:285-292 (full_intff * size), tet4.cc:348-355 */
static double el_intff(const tor_mesh *m, int e, int i, int j)
{
    if (m->dim == 2) return ((i == j ? 2.0 : 1.0) * (1.0 / 12.0)) * m->size[e];
    return ((i == j ? 2.0 : 1.0) * (1.0 / 20.0)) * m->size[e];
}

/* Element IntFFF(i,j,k): tri3.cc:294-297 (intfff_scale table), tet4.cc:357-361 */
static double el_intfff(const tor_mesh *m, int e, int i, int j, int k)
{
    if (m->dim == 2) {
        static const int idx[3][3][3] = {
            {{2,1,1},{1,1,0},{1,0,1}},{{1,1,0},{1,2,1},{0,1,1}},{{1,0,1},{0,1,1},{1,1,2}}};
        static const double scl[3] = {1.0 / 60.0, 1.0 / 30.0, 1.0 / 10.0};
        return m->size[e] * scl[idx[i][j][k]];
    }
    return TET_FFF[i][j][k] / 120.0 * m->size[e];
}

/* Element IntFDD(i,j,k): tri3.h:196-197 (intdd * 0.3333333333), tet4.cc:380-412 */
static double el_intfdd(const tor_mesh *m, int e, int i, int j, int k)
{
    (void)i;
    if (m->dim == 2) return m->intdd[(size_t)e * 9 + j * 3 + k] * 0.3333333333;
    return tet_intfdd(m, e, j, k);
}

/* ------------------------------------------------------------------------ */
/* Assembly: TFwdSolver::AssembleSystemMatrix (fwdsolver.cc:337-357 real,    */
/* 404-424 complex) via AddToSysMatrix/AddToElMatrix (mesh.cc:1958-2282).    */
/* ------------------------------------------------------------------------ */

static int csr_find(const int *rowptr, const int *colidx, int r, int c)
{
    int lo = rowptr[r], hi = rowptr[r + 1] - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (colidx[mid] == c) return mid;
        if (colidx[mid] < c) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

/* val: nnz doubles (real) or 2*nnz interleaved (complex).  Each nodal term is
   accumulated over all elements into a zeroed temporary and then added into F,
   the order the reference's assembly engine uses with one thread
   (mesh.cc:2135-2167); the i*omega*IntFF term is added directly (2252-2282). */
void tor_assemble(const tor_mesh *m, const double *cmua, const double *ckap, const double *c2a,
                  double omega, int cplx, double *val)
{
    int nnz = m->nnz, nn = m->nn;
    double *tmp = malloc(sizeof(double) * nnz);
    memset(val, 0, sizeof(double) * nnz * (cplx ? 2 : 1));
    for (int mode = 0; mode < 3; mode++) {
        const double *P = mode == 0 ? cmua : mode == 1 ? ckap : c2a;
        memset(tmp, 0, sizeof(double) * nnz);
        for (int e = 0; e < m->ne; e++) {
            const int *nd = m->el + (size_t)e * nn;
            for (int i = 0; i < nn; i++)
                for (int j = 0; j < nn; j++) {
                    double v;
                    if (mode == 0) v = m->dim == 2 ? tri_intpff(m, e, i, j, P) : tet_intpff(m, e, i, j, P);
                    else if (mode == 1) v = el_intpdd(m, e, i, j, P);
                    else v = el_bndintpff(m, e, i, j, P);
                    tmp[csr_find(m->rowptr, m->colidx, nd[i], nd[j])] += v;
                }
        }
        for (int k = 0; k < nnz; k++) val[cplx ? 2 * k : k] += tmp[k];
    }
    if (cplx) {
        for (int e = 0; e < m->ne; e++) {
            const int *nd = m->el + (size_t)e * nn;
            for (int i = 0; i < nn; i++)
                for (int j = 0; j < nn; j++)
                    val[2 * csr_find(m->rowptr, m->colidx, nd[i], nd[j]) + 1] += el_intff(m, e, i, j) * omega;
        }
    }
    free(tmp);
}

/* Element-basis assembly (TFwdSolver::Reset with elbasis, fwdsolver.cc:
   337-357 / 404-424; AddToElMatrix modes ASSEMBLE_PFF_EL / PDD_EL /
   BNDPFF_EL, mesh.cc:1985-1993): entry IntFF(i,j) P[e], IntDD(i,j) P[e],
   BndIntFF(i,j) P[e], each mode accumulated as tor_assemble does. */
void tor_assemble_el(const tor_mesh *m, const double *cmua, const double *ckap, const double *c2a,
                     double omega, int cplx, double *val)
{
    int nnz = m->nnz, nn = m->nn;
    double *tmp = malloc(sizeof(double) * nnz);
    memset(val, 0, sizeof(double) * nnz * (cplx ? 2 : 1));
    for (int mode = 0; mode < 3; mode++) {
        const double *P = mode == 0 ? cmua : mode == 1 ? ckap : c2a;
        memset(tmp, 0, sizeof(double) * nnz);
        for (int e = 0; e < m->ne; e++) {
            const int *nd = m->el + (size_t)e * nn;
            for (int i = 0; i < nn; i++)
                for (int j = 0; j < nn; j++) {
                    double v;
                    if (mode == 0) v = el_intff(m, e, i, j) * P[e];
                    else if (mode == 1) v = m->intdd[((size_t)e * nn + i) * nn + j] * P[e];
                    else v = m->intbff[((size_t)e * nn + i) * nn + j] * P[e];
                    tmp[csr_find(m->rowptr, m->colidx, nd[i], nd[j])] += v;
                }
        }
        for (int k = 0; k < nnz; k++) val[cplx ? 2 * k : k] += tmp[k];
    }
    if (cplx) {
        for (int e = 0; e < m->ne; e++) {
            const int *nd = m->el + (size_t)e * nn;
            for (int i = 0; i < nn; i++)
                for (int j = 0; j < nn; j++)
                    val[2 * csr_find(m->rowptr, m->colidx, nd[i], nd[j]) + 1] += el_intff(m, e, i, j) * omega;
        }
    }
    free(tmp);
}

/* ------------------------------------------------------------------------ */
/* Source and measurement vectors: QVec_Gaussian (source.cc:19-56)           */
/* ------------------------------------------------------------------------ */

void tor_qvec_gaussian(const tor_mesh *m, const double *cnt, double w, int neumann, double *q)
{
    double w2 = w * w;
    double fac1 = 1.0 / (sqrt(2.0 * M_PI) * w);
    if (m->dim == 3) fac1 /= (sqrt(2.0 * M_PI) * w);
    if (!neumann) fac1 /= (sqrt(2.0 * M_PI) * w);
    double fac2 = -0.5 / w2;
    memset(q, 0, sizeof(double) * m->n);
    for (int e = 0; e < m->ne; e++) {
        const int *nd = m->el + (size_t)e * m->nn;
        for (int i = 0; i < m->nn; i++) {
            int is = nd[i];
            if (neumann && !m->bndnode[is]) continue;
            double d = pt_dist(cnt, m->x + (size_t)is * m->dim, m->dim);
            double s = exp(d * d * fac2) * fac1;
            for (int j = 0; j < m->nn; j++) {
                int js = nd[j];
                if (neumann) {
                    if (m->bndnode[js]) q[js] += s * m->intbff[(size_t)e * m->nn * m->nn + i * m->nn + j];
                } else {
                    q[js] += s * el_intff(m, e, i, j);
                }
            }
        }
    }
}

/* Mesh::PullToBoundary (mesh.cc:1052-1111) for P1 elements: project p in the
   local coordinates of the first element around the nearest boundary node
   whose boundary side contains the projection.  Returns 0 on success. */
int tor_pull_to_boundary(const tor_mesh *m, const double *p, double *pshift)
{
    int dim = m->dim, nmin = -1;
    double dmin = 1e10;
    for (int k = 0; k < m->n; k++) {
        if (!m->bndnode[k]) continue;
        double d = pt_dist(p, m->x + (size_t)k * dim, dim);
        if (d < dmin) { dmin = d; nmin = k; }
    }
    /* Triangle3::LNormal (tri3.cc:172-182), Tetrahedron4::LNormal (tet4.cc:254-266) */
    static const double LN2[3][2] = {{0, -1}, {0.7071067814, 0.7071067814}, {-1, 0}};
    static const double LN3[4][3] = {{0, 0, -1}, {0, -1, 0}, {-1, 0, 0},
                                     {0.577350269, 0.577350269, 0.577350269}};
    for (int e = 0; e < m->ne; e++) {
        const int *nd = m->el + (size_t)e * m->nn;
        int has = 0;
        for (int i = 0; i < m->nn; i++) has |= nd[i] == nmin;
        if (!has) continue;
        const double *g = m->geo + (size_t)e * 16;
        double ploc[3], nloc[3];
        int nside = dim == 2 ? 3 : 4;
        for (int sd = 0; sd < nside; sd++) {
            int bnd = 1;  /* Element::BndSideList (element.cc:338-348) */
            for (int k = 0; k < (dim == 2 ? 2 : 3); k++)
                if (!m->bndnode[nd[dim == 2 ? TRI_SN[sd][k] : TET_SN[sd][k]]]) { bnd = 0; break; }
            if (!bnd) continue;
            const double *q0 = m->x + (size_t)nd[dim == 2 ? TRI_SN[sd][0] : TET_SN[sd][0]] * dim;
            if (dim == 2) {  /* Triangle3::Local (tri3.cc:134-144) */
                double scale = 1.0 / (g[0] + g[1] + g[2]);
                ploc[0] = (g[1] + g[4] * p[0] + g[7] * p[1]) * scale;
                ploc[1] = (g[2] + g[5] * p[0] + g[8] * p[1]) * scale;
                nloc[0] = (g[1] + g[4] * q0[0] + g[7] * q0[1]) * scale;
                nloc[1] = (g[2] + g[5] * q0[0] + g[8] * q0[1]) * scale;
                double pd = (ploc[0] - nloc[0]) * LN2[sd][0] + (ploc[1] - nloc[1]) * LN2[sd][1];
                double l0 = ploc[0] - LN2[sd][0] * pd, l1 = ploc[1] - LN2[sd][1] * pd;
                if (l0 + 1e-8 >= 0.0 && l1 + 1e-8 >= 0.0 && l0 + l1 - 1e-8 <= 1.0) {  /* LContains, pad=true (tri3.cc:191-200) */
                    double u[3] = {1.0 - l0 - l1, l0, l1};  /* LocalShapeF + Element::Global */
                    for (int c = 0; c < 2; c++) {
                        pshift[c] = 0.0;
                        for (int j = 0; j < 3; j++) pshift[c] += u[j] * m->x[(size_t)nd[j] * 2 + c];
                    }
                    return 0;
                }
            } else {  /* Tetrahedron4::Local (tet4.cc:186-196) */
                const double *a = g, *b = g + 4, *c = g + 8, *d = g + 12;
                double scale = 1.0 / (a[0] + a[1] + a[2] + a[3]);
                for (int r = 0; r < 3; r++) {
                    ploc[r] = (a[r + 1] + b[r + 1] * p[0] + c[r + 1] * p[1] + d[r + 1] * p[2]) * scale;
                    nloc[r] = (a[r + 1] + b[r + 1] * q0[0] + c[r + 1] * q0[1] + d[r + 1] * q0[2]) * scale;
                }
                double pd = 0.0;
                for (int r = 0; r < 3; r++) pd += (ploc[r] - nloc[r]) * LN3[sd][r];
                double l[3];
                for (int r = 0; r < 3; r++) l[r] = ploc[r] - LN3[sd][r] * pd;
                if (l[0] + 1e-8 >= 0.0 && l[1] + 1e-8 >= 0.0 && l[2] + 1e-8 >= 0.0 &&
                    l[0] + l[1] + l[2] - 1e-8 <= 1.0) {  /* LContains, pad=true (tet4.cc:268-279) */
                    double u[4] = {1.0 - l[0] - l[1] - l[2], l[0], l[1], l[2]};
                    for (int cc = 0; cc < 3; cc++) {
                        pshift[cc] = 0.0;
                        for (int j = 0; j < 4; j++) pshift[cc] += u[j] * m->x[(size_t)nd[j] * 3 + cc];
                    }
                    return 0;
                }
            }
        }
    }
    return 1;  /* the reference falls back to PullToBoundary_old here */
}

/* ------------------------------------------------------------------------ */
/* Preconditioners                                                            */
/* ------------------------------------------------------------------------ */

typedef struct {
    int type;             /* 0 none, 1 diag, 2 ich */
    int n, cplx;
    zd *idiag;            /* diag */
    int *Lrowptr, *Lcolidx;   /* ich: strict lower pattern */
    zd *Lval, *d;
    int *Ccolptr, *Crowidx, *Cvofs;  /* column access of L */
} precon_t;

/* TCompRowMatrix::CalculateIncompleteCholeskyFillin (crmatrix_imp.hpp:2077-2102)
   and IncompleteCholeskyFactorize (2166-2203) with recover=true; complex
   comparisons use squared magnitudes (mathdef.h:128-132). */
static void ic_factor(int n, const int *rowptr, const int *colidx, const zd *A, int cplx, precon_t *P)
{
    const double EPS = 1e-10;
    int nl = 0;
    P->Lrowptr = calloc(n + 1, sizeof(int));
    for (int i = 0; i < n; i++) {
        int nc = 0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; j++) { if (colidx[j] < i) nc++; else break; }
        P->Lrowptr[i + 1] = P->Lrowptr[i] + nc;
    }
    nl = P->Lrowptr[n];
    P->Lcolidx = malloc(sizeof(int) * (nl ? nl : 1));
    for (int i = 0, c = 0; i < n; i++)
        for (int j = rowptr[i]; j < rowptr[i + 1]; j++) { if (colidx[j] < i) P->Lcolidx[c++] = colidx[j]; else break; }
    P->Lval = calloc(nl ? nl : 1, sizeof(zd));
    P->d = calloc(n > 0 ? (size_t)n : 1, sizeof(zd));
    int *Lr = P->Lrowptr, *Lc = P->Lcolidx;
    zd *Lv = P->Lval;
    for (int i = 0; i < n; i++) {
        zd diag = 0;
        int kd = csr_find(rowptr, colidx, i, i);
        if (kd >= 0) diag = A[kd];
        zd x = 0;
        for (int j = Lr[i]; j < Lr[i + 1]; j++) x += Lv[j] * Lv[j];
        int pos;
        if (cplx) {
            double nd = creal(diag) * creal(diag) + cimag(diag) * cimag(diag);
            double nx = creal(x) * creal(x) + cimag(x) * cimag(x);
            pos = nd > nx;
        } else {
            pos = creal(diag) > creal(x);
        }
        if (pos) P->d[i] = cplx ? csqrt(diag - x) : sqrt(creal(diag) - creal(x));
        else P->d[i] = EPS;
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            int j = colidx[k];
            if (j <= i) continue;
            zd Aj = A[k], v;
            if (i) {
                /* row_mult (crmatrix_imp.hpp:1971-2009): sum_{c<i} L(i,c) L(j,c) */
                zd s = 0;
                int i1 = Lr[i], e1 = Lr[i + 1], i2 = Lr[j], e2 = Lr[j + 1];
                while (i1 < e1 && i2 < e2) {
                    int c1 = Lc[i1], c2 = Lc[i2];
                    if (c1 > i - 1 || c2 > i - 1) break;
                    if (c1 < c2) i1++;
                    else if (c1 > c2) i2++;
                    else { s += Lv[i1] * Lv[i2]; i1++; i2++; }
                }
                v = cplx ? (Aj - s) / P->d[i] : (creal(Aj) - creal(s)) / creal(P->d[i]);
            } else {
                v = cplx ? Aj / P->d[i] : creal(Aj) / creal(P->d[i]);
            }
            int kk = csr_find(Lr, Lc, j, i);
            Lv[kk] = v;
        }
    }
    /* SetColAccess: column view, rows ascending within each column */
    P->Ccolptr = calloc(n + 1, sizeof(int));
    P->Crowidx = malloc(sizeof(int) * (nl ? nl : 1));
    P->Cvofs = malloc(sizeof(int) * (nl ? nl : 1));
    for (int k = 0; k < nl; k++) P->Ccolptr[Lc[k] + 1]++;
    for (int i = 0; i < n; i++) P->Ccolptr[i + 1] += P->Ccolptr[i];
    int *fill = calloc(n, sizeof(int));
    for (int r = 0; r < n; r++)
        for (int k = Lr[r]; k < Lr[r + 1]; k++) {
            int c = Lc[k], pos = P->Ccolptr[c] + fill[c]++;
            P->Crowidx[pos] = r; P->Cvofs[pos] = k;
        }
    free(fill);
}

static void precon_setup(int n, const int *rowptr, const int *colidx, const zd *A, int cplx, int type, precon_t *P)
{
    memset(P, 0, sizeof(*P));
    P->type = type; P->n = n; P->cplx = cplx;
    if (type == 1) {  /* TPrecon_Diag::Reset (precon_imp.hpp:56-64) */
        P->idiag = malloc(sizeof(zd) * n);
        for (int i = 0; i < n; i++) {
            int k = csr_find(rowptr, colidx, i, i);
            zd dg = k >= 0 ? A[k] : 0;
            P->idiag[i] = (creal(dg) != 0 || cimag(dg) != 0) ? (cplx ? 1.0 / dg : 1.0 / creal(dg)) : 1.0;
        }
    } else if (type == 2) {
        ic_factor(n, rowptr, colidx, A, cplx, P);
    }
}

static void precon_free(precon_t *P)
{
    free(P->idiag); free(P->Lrowptr); free(P->Lcolidx); free(P->Lval); free(P->d);
    free(P->Ccolptr); free(P->Crowidx); free(P->Cvofs);
}

/* TPrecon_*::Apply; IC apply is CholeskySubst (crmatrix_imp.hpp:2267-2295).
   b and x may alias. */
static void precon_apply(const precon_t *P, const zd *b, zd *x)
{
    int n = P->n;
    if (P->type == 0) { if (x != b) memcpy(x, b, sizeof(zd) * n); return; }
    if (P->type == 1) {
        for (int i = 0; i < n; i++) x[i] = P->cplx ? b[i] * P->idiag[i] : creal(b[i]) * creal(P->idiag[i]);
        return;
    }
    const int *Lr = P->Lrowptr, *Lc = P->Lcolidx;
    const zd *Lv = P->Lval, *d = P->d;
    if (P->cplx) {
        for (int i = 0; i < n; i++) {
            zd s = b[i];
            for (int k = Lr[i]; k < Lr[i + 1]; k++) s -= Lv[k] * x[Lc[k]];
            x[i] = s / d[i];
        }
        for (int i = n - 1; i >= 0; i--) {
            zd s = x[i];
            for (int k = P->Ccolptr[i + 1] - 1; k >= P->Ccolptr[i]; k--) s -= Lv[P->Cvofs[k]] * x[P->Crowidx[k]];
            x[i] = s / d[i];
        }
    } else {
        for (int i = 0; i < n; i++) {
            double s = creal(b[i]);
            for (int k = Lr[i]; k < Lr[i + 1]; k++) s -= creal(Lv[k]) * creal(x[Lc[k]]);
            x[i] = s / creal(d[i]);
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = creal(x[i]);
            for (int k = P->Ccolptr[i + 1] - 1; k >= P->Ccolptr[i]; k--)
                s -= creal(Lv[P->Cvofs[k]]) * creal(x[P->Crowidx[k]]);
            x[i] = s / creal(d[i]);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Krylov solvers                                                             */
/* ------------------------------------------------------------------------ */

typedef struct { int n; const int *rowptr, *colidx; const zd *val; int cplx; } spmat;

/* TCompRowMatrix::Ax (crmatrix_imp.hpp:1172-1189) */
static void spmv(const spmat *A, const zd *x, zd *y)
{
    for (int r = 0; r < A->n; r++) {
        zd s = 0;
        if (A->cplx) for (int k = A->rowptr[r]; k < A->rowptr[r + 1]; k++) s += A->val[k] * x[A->colidx[k]];
        else {
            double sr = 0;
            for (int k = A->rowptr[r]; k < A->rowptr[r + 1]; k++) sr += creal(A->val[k]) * creal(x[A->colidx[k]]);
            s = sr;
        }
        y[r] = s;
    }
}

/* l2norm (vector_imp.hpp:1116-1120, 1290-1298): sqrt(sum |v_i|^2) with |.| = abs */
static double l2norm(const zd *v, int n)
{
    double s = 0.0;
    for (int i = 0; i < n; i++) { double t = cabs(v[i]); s += t * t; }
    return sqrt(s);
}

/* PCG (matrix_imp.hpp:93-154), real */
static int pcg_real(const spmat *A, const zd *bz, zd *xz, double *tol, const precon_t *P, int maxit)
{
    int n = A->n, niter;
    double dnew, dold, alpha, beta, err = 0, bnorm;
    if (!maxit) maxit = n + 1;
    zd *r = malloc(sizeof(zd) * n), *d = malloc(sizeof(zd) * n), *q = malloc(sizeof(zd) * n);
    spmv(A, xz, r);
    for (int i = 0; i < n; i++) r[i] = creal(bz[i]) - creal(r[i]);
    if (P->type) precon_apply(P, r, d); else memcpy(d, r, sizeof(zd) * n);
    dnew = 0; for (int i = 0; i < n; i++) dnew += creal(r[i]) * creal(d[i]);
    bnorm = l2norm(bz, n);
    for (niter = 0; niter < maxit; niter++) {
        spmv(A, d, q);
        double dq = 0; for (int i = 0; i < n; i++) dq += creal(d[i]) * creal(q[i]);
        alpha = dnew / dq;
        if (!alpha || isnan(alpha)) break;
        for (int i = 0; i < n; i++) xz[i] = creal(xz[i]) + creal(d[i]) * alpha;
        for (int i = 0; i < n; i++) r[i] = creal(r[i]) - creal(q[i]) * alpha;
        dold = dnew;
        if (P->type) {
            precon_apply(P, r, q);
            dnew = 0; for (int i = 0; i < n; i++) dnew += creal(r[i]) * creal(q[i]);
            beta = dnew / dold;
            for (int i = 0; i < n; i++) { double t = creal(d[i]) * beta; d[i] = t + creal(q[i]); }
        } else {
            dnew = 0; for (int i = 0; i < n; i++) dnew += creal(r[i]) * creal(r[i]);
            beta = dnew / dold;
            for (int i = 0; i < n; i++) { double t = creal(d[i]) * beta; d[i] = t + creal(r[i]); }
        }
        if (!beta || isnan(beta)) break;
        err = l2norm(r, n);
        if (err <= *tol * bnorm) break;
    }
    *tol = err / bnorm;
    free(r); free(d); free(q);
    return niter;
}

/* Re(conj(a) b) summed, the scalar the reference's complex BiCGSTAB uses */
static double redot(const zd *a, const zd *b, int n)
{
    double s = 0.0;
    for (int i = 0; i < n; i++) s += creal(a[i]) * creal(b[i]) + cimag(a[i]) * cimag(b[i]);
    return s;
}

/* BiCGSTAB, complex specialisation with real scalars (matrix_imp.hpp:350-413) */
static int bicgstab_cplx(const spmat *A, const zd *b, zd *x, double *tol, const precon_t *P, int maxit, int *fail)
{
    int n = A->n, niter;
    double err = 0, bnorm, rho = 0, rhop, alpha = 0, beta, omega = 0, aden, onum, oden;
    if (!maxit) maxit = n + 1;
    zd *r = malloc(sizeof(zd) * n), *rd = malloc(sizeof(zd) * n), *p = malloc(sizeof(zd) * n);
    zd *pd = malloc(sizeof(zd) * n), *v = malloc(sizeof(zd) * n), *s = malloc(sizeof(zd) * n);
    zd *sd = malloc(sizeof(zd) * n), *t = malloc(sizeof(zd) * n);
    spmv(A, x, r);
    for (int i = 0; i < n; i++) rd[i] = r[i] = b[i] - r[i];
    bnorm = l2norm(b, n);
    *fail = 0;
    for (niter = 0; niter < maxit; niter++) {
        rhop = rho;
        rho = redot(rd, r, n);
        if (rho == 0.0) { *fail = 1; break; }  /* xASSERT in the reference */
        if (!niter) memcpy(p, r, sizeof(zd) * n);
        else {
            beta = (rho * alpha) / (rhop * omega);
            for (int i = 0; i < n; i++) p[i] = r[i] + (p[i] - v[i] * omega) * beta;
        }
        precon_apply(P, p, pd);
        spmv(A, pd, v);
        aden = redot(rd, v, n);
        alpha = rho / aden;
        for (int i = 0; i < n; i++) s[i] = r[i] - v[i] * alpha;
        precon_apply(P, s, sd);
        spmv(A, sd, t);
        onum = redot(t, s, n);
        oden = redot(t, t, n);
        omega = onum / oden;
        for (int i = 0; i < n; i++) {
            x[i] += pd[i] * alpha + sd[i] * omega;
            r[i] = s[i] - t[i] * omega;
        }
        err = l2norm(r, n);
        if (err <= *tol * bnorm) break;
        if (omega == 0.0) break;
    }
    *tol = err / bnorm;
    free(r); free(rd); free(p); free(pd); free(v); free(s); free(sd); free(t);
    return niter;
}

/* BiCGSTAB, generic (real) version (matrix_imp.hpp:479-547) */
static int bicgstab_real(const spmat *A, const zd *bz, zd *xz, double *tol, const precon_t *P, int maxit)
{
    int n = A->n, niter;
    double rho = 0, alpha = 0, aden, beta, bden, omega = 0, err = 0, bnorm;
    if (!maxit) maxit = n + 1;
    double *r = malloc(8 * n), *rd = malloc(8 * n), *p = malloc(8 * n), *s = malloc(8 * n), *t = malloc(8 * n), *v = malloc(8 * n);
    zd *pd = malloc(sizeof(zd) * n), *sd = malloc(sizeof(zd) * n), *tz = malloc(sizeof(zd) * n);
    spmv(A, xz, tz);
    for (int i = 0; i < n; i++) rd[i] = r[i] = creal(bz[i]) - creal(tz[i]);
    bnorm = l2norm(bz, n);
    for (niter = 0; niter < maxit; niter++) {
        bden = rho;
        rho = 0; for (int i = 0; i < n; i++) rho += rd[i] * r[i];
        if (!rho) break;
        if (!niter) memcpy(p, r, 8 * n);
        else {
            beta = (rho * alpha) / (bden * omega);
            for (int i = 0; i < n; i++) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        }
        for (int i = 0; i < n; i++) tz[i] = p[i];
        precon_apply(P, tz, pd);
        spmv(A, pd, tz);
        for (int i = 0; i < n; i++) v[i] = creal(tz[i]);
        aden = 0; for (int i = 0; i < n; i++) aden += rd[i] * v[i];
        alpha = rho / aden;
        for (int i = 0; i < n; i++) s[i] = r[i] - alpha * v[i];
        err = 0; for (int i = 0; i < n; i++) err += fabs(s[i]) * fabs(s[i]);
        err = sqrt(err);
        if (err < *tol * bnorm) {
            for (int i = 0; i < n; i++) xz[i] = creal(xz[i]) + alpha * creal(pd[i]);
            break;
        }
        for (int i = 0; i < n; i++) tz[i] = s[i];
        precon_apply(P, tz, sd);
        spmv(A, sd, tz);
        for (int i = 0; i < n; i++) t[i] = creal(tz[i]);
        double ts = 0, tt = 0;
        for (int i = 0; i < n; i++) ts += t[i] * s[i];
        for (int i = 0; i < n; i++) tt += t[i] * t[i];
        omega = ts / tt;
        for (int i = 0; i < n; i++) {
            xz[i] = creal(xz[i]) + (alpha * creal(pd[i]) + omega * creal(sd[i]));
            r[i] = s[i] - omega * t[i];
        }
        err = 0; for (int i = 0; i < n; i++) err += fabs(r[i]) * fabs(r[i]);
        err = sqrt(err);
        if (err <= *tol * bnorm) break;
        if (omega == 0.0) break;
    }
    *tol = err / bnorm;
    free(r); free(rd); free(p); free(s); free(t); free(v); free(pd); free(sd); free(tz);
    return niter;
}

/* gmres (gmres_imp.hpp:39-230), restart 20 (gsmatrix_imp.hpp:539).  Complex
   arithmetic throughout; for a real system every imaginary part stays zero. */
static int gmres_z(const spmat *A, const zd *b, zd *x, double *elim, const precon_t *P, int restart, int maxit)
{
    int N = A->n, M = restart, MAXC = maxit ? maxit : N + 1;
    int j, k, l, cycle;
    double norm_b, norm_v, norm_x, tmp;
    zd *y = calloc(M, sizeof(zd)), *s = calloc(M + 1, sizeof(zd));
    zd *c1 = calloc(M, sizeof(zd)), *c2 = calloc(M, sizeof(zd));
    zd *H = calloc((size_t)M * (M + 1), sizeof(zd));
#define HH(a, b) H[(a) * (M + 1) + (b)]
    zd **v = malloc(sizeof(zd *) * (M + 1));
    for (j = 0; j <= M; j++) v[j] = calloc(N, sizeof(zd));
    zd *Mb = malloc(sizeof(zd) * N), *w = malloc(sizeof(zd) * N);
    memcpy(Mb, b, sizeof(zd) * N);
    precon_apply(P, Mb, Mb);
    norm_b = l2norm(Mb, N);
    norm_x = l2norm(x, N);
    cycle = j = 0;
    if (norm_x < *elim * N) memcpy(v[0], Mb, sizeof(zd) * N);
    else {
        spmv(A, x, v[0]);
        precon_apply(P, v[0], v[0]);
        for (int i = 0; i < N; i++) v[0][i] = Mb[i] - v[0][i];
    }
    while (((norm_v = l2norm(v[0], N)) > *elim * norm_b) && (cycle < MAXC)) {
        s[0] = norm_v;
        for (int i = 0; i < N; i++) v[0][i] = v[0][i] / s[0];
        j = -1;
        cycle++;
        while ((norm_x = cabs(s[j + 1])) > *elim * norm_b && (j < M - 1) && (cycle < MAXC)) {
            j++;
            zd *vj1 = v[j + 1];
            spmv(A, v[j], w);
            precon_apply(P, w, vj1);
            for (k = 0; k <= j; k++) {
                zd *vk = v[k], sum = 0;
                for (int i = 0; i < N; i++) sum += vj1[i] * conj(vk[i]);
                HH(j, k) = sum;
                for (int i = 0; i < N; i++) vj1[i] -= sum * vk[i];
            }
            tmp = l2norm(vj1, N);
            HH(j, j + 1) = tmp;
            tmp = 1.0 / tmp;
            for (int i = 0; i < N; i++) vj1[i] *= tmp;
            for (k = 0; k < j; k++) {
                zd h1 = c1[k] * HH(j, k) + c2[k] * HH(j, k + 1);
                zd h2 = -c2[k] * HH(j, k) + c1[k] * HH(j, k + 1);
                HH(j, k) = h1;
                HH(j, k + 1) = h2;
            }
            zd r = csqrt(HH(j, j) * HH(j, j) + HH(j, j + 1) * HH(j, j + 1));
            c1[j] = HH(j, j) / r;
            c2[j] = HH(j, j + 1) / r;
            HH(j, j) = r;
            HH(j, j + 1) = 0.0;
            s[j + 1] = -c2[j] * s[j];
            s[j] = s[j] * c1[j];
        }
        for (l = j; l >= 0; l--) {
            y[l] = s[l] / HH(l, l);
            for (k = l - 1; k >= 0; k--) s[k] = s[k] - HH(l, k) * y[l];
        }
        for (l = j; l >= 0; l--)
            for (int i = 0; i < N; i++) x[i] = x[i] + y[l] * v[l][i];
        spmv(A, x, v[0]);
        precon_apply(P, v[0], v[0]);
        for (int i = 0; i < N; i++) v[0][i] = Mb[i] - v[0][i];
    }
#undef HH
    *elim = norm_v / norm_b;
    for (j = 0; j <= M; j++) free(v[j]);
    free(v); free(y); free(s); free(c1); free(c2); free(H); free(Mb); free(w);
    return cycle;
}

/* ------------------------------------------------------------------------ */
/* Multi-source solve: TFwdSolver::CalcFields (fwdsolver.cc:653-750), sources */
/* split over threads in contiguous ranges like CalcFields_engine (618-643).  */
/* ------------------------------------------------------------------------ */

typedef struct {
    const spmat *A; const precon_t *P;
    int method, maxit, nrhs, q0, q1;
    double tol;
    const double *B; double *X; int *its; double *errs; int *fails;
} solve_job;

static void *solve_worker(void *arg)
{
    solve_job *J = arg;
    int n = J->A->n;
    zd *b = malloc(sizeof(zd) * n), *x = malloc(sizeof(zd) * n);
    for (int q = J->q0; q < J->q1; q++) {
        for (int i = 0; i < n; i++) {
            if (J->A->cplx) { b[i] = J->B[2 * ((size_t)q * n + i)] + I * J->B[2 * ((size_t)q * n + i) + 1];
                              x[i] = J->X[2 * ((size_t)q * n + i)] + I * J->X[2 * ((size_t)q * n + i) + 1]; }
            else { b[i] = J->B[(size_t)q * n + i]; x[i] = J->X[(size_t)q * n + i]; }
        }
        double tol = J->tol;
        int it = -1, fail = 0;
        if (J->method == 0 && !J->A->cplx) it = pcg_real(J->A, b, x, &tol, J->P, J->maxit);
        else if (J->method == 1 && J->A->cplx) it = bicgstab_cplx(J->A, b, x, &tol, J->P, J->maxit, &fail);
        else if (J->method == 1) it = bicgstab_real(J->A, b, x, &tol, J->P, J->maxit);
        else if (J->method == 2) it = gmres_z(J->A, b, x, &tol, J->P, 20, J->maxit);
        else fail = 2;
        for (int i = 0; i < n; i++) {
            if (J->A->cplx) { J->X[2 * ((size_t)q * n + i)] = creal(x[i]); J->X[2 * ((size_t)q * n + i) + 1] = cimag(x[i]); }
            else J->X[(size_t)q * n + i] = creal(x[i]);
        }
        J->its[q] = it; J->errs[q] = tol; J->fails[q] = fail;
    }
    free(b); free(x);
    return NULL;
}

/* method: 0 CG (real), 1 BiCGSTAB, 2 GMRES(20).  precon: 0 none,
   1 diag, 2 IC(0).  B, X: nrhs x n (complex interleaved when cplx); X holds
   the initial guess on entry.  Returns 0, or the number of failed solves. */
int tor_solve(int n, const int *rowptr, const int *colidx, const double *val, int cplx,
              int method, int precon, double tol, int maxit, int nrhs,
              const double *B, double *X, int *its, double *errs, int nthreads)
{
    int nnz = rowptr[n];
    zd *A = malloc(sizeof(zd) * (nnz ? nnz : 1));
    for (int k = 0; k < nnz; k++) A[k] = cplx ? val[2 * k] + I * val[2 * k + 1] : val[k];
    spmat S = {n, rowptr, colidx, A, cplx};
    precon_t P;
    precon_setup(n, rowptr, colidx, A, cplx, precon, &P);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > nrhs) nthreads = nrhs > 0 ? nrhs : 1;
    int *fails = calloc(nrhs > 0 ? nrhs : 1, sizeof(int));
    solve_job *jobs = malloc(sizeof(solve_job) * nthreads);
    pthread_t *th = malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; t++) {
        solve_job j = {&S, &P, method, maxit, nrhs, (t * nrhs) / nthreads, ((t + 1) * nrhs) / nthreads,
                       tol, B, X, its, errs, fails};
        jobs[t] = j;
        if (nthreads > 1) pthread_create(&th[t], NULL, solve_worker, &jobs[t]);
        else solve_worker(&jobs[t]);
    }
    if (nthreads > 1) for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    int nf = 0;
    for (int q = 0; q < nrhs; q++) nf += fails[q] != 0;
    free(fails); free(jobs); free(th); free(A);
    precon_free(&P);
    return nf;
}

/* IC(0) factor as a standalone entry point (for kernel-level parity tests).
   Lrowptr: n+1, Lcolidx/Lval: nnz_L (Lval complex interleaved when cplx), d: n. */
int tor_ic_factor(int n, const int *rowptr, const int *colidx, const double *val, int cplx,
                  int *Lrowptr, int *Lcolidx, double *Lval, double *d)
{
    int nnz = rowptr[n];
    zd *A = malloc(sizeof(zd) * (nnz ? nnz : 1));
    for (int k = 0; k < nnz; k++) A[k] = cplx ? val[2 * k] + I * val[2 * k + 1] : val[k];
    precon_t P;
    precon_setup(n, rowptr, colidx, A, cplx, 2, &P);
    int nl = P.Lrowptr[n];
    memcpy(Lrowptr, P.Lrowptr, sizeof(int) * (n + 1));
    memcpy(Lcolidx, P.Lcolidx, sizeof(int) * nl);
    for (int k = 0; k < nl; k++) {
        if (cplx) { Lval[2 * k] = creal(P.Lval[k]); Lval[2 * k + 1] = cimag(P.Lval[k]); }
        else Lval[k] = creal(P.Lval[k]);
    }
    for (int i = 0; i < n; i++) {
        if (cplx) { d[2 * i] = creal(P.d[i]); d[2 * i + 1] = cimag(P.d[i]); }
        else d[i] = creal(P.d[i]);
    }
    precon_free(&P);
    free(A);
    return nl;
}

/* ------------------------------------------------------------------------ */
/* ProjectAll (fwdsolver.cc:1415-1447): y_qm = dot(phi_q, mvec_m), non-       */
/* conjugating, over the linked detectors in link order; LOG gives log(y).   */
/* ------------------------------------------------------------------------ */

void tor_project(int n, int nq, const double *phi, const double *mvec_dense, const int *link_ofs,
                 const int *link_m, int cplx, int logscale, double *proj)
{
    for (int q = 0; q < nq; q++)
        for (int l = link_ofs[q]; l < link_ofs[q + 1]; l++) {
            int m = link_m[l];
            if (cplx) {
                zd s = 0;
                for (int i = 0; i < n; i++) {
                    zd a = phi[2 * ((size_t)q * n + i)] + I * phi[2 * ((size_t)q * n + i) + 1];
                    zd b = mvec_dense[2 * ((size_t)m * n + i)] + I * mvec_dense[2 * ((size_t)m * n + i) + 1];
                    s += a * b;
                }
                if (logscale) s = clog(s);
                proj[2 * l] = creal(s); proj[2 * l + 1] = cimag(s);
            } else {
                double s = 0;
                for (int i = 0; i < n; i++) s += phi[(size_t)q * n + i] * mvec_dense[(size_t)m * n + i];
                proj[l] = logscale ? log(s) : s;
            }
        }
}

/* ------------------------------------------------------------------------ */
/* Nodal Jacobian: GenerateJacobian_mesh (jacobian.cc:441-497) for complex    */
/* fields and GenerateJacobian_cw_mesh (738-802) + RowScale (160-177) for CW. */
/* IntFG (806-835) and IntGradFGradG (839-872) are restated element by        */
/* element with the same summation order.                                     */
/* ------------------------------------------------------------------------ */

static void intfg_pair(const tor_mesh *m, const zd *f, const zd *g, int kap, zd *tmp)
{
    memset(tmp, 0, sizeof(zd) * m->n);
    for (int e = 0; e < m->ne; e++) {
        const int *nd = m->el + (size_t)e * m->nn;
        for (int i = 0; i < m->nn; i++) {
            int bs = nd[i];
            for (int j = 0; j < m->nn; j++) {
                int nj = nd[j];
                zd sum = (f[nj] * g[nj]) * (kap ? el_intfdd(m, e, i, j, j) : el_intfff(m, e, i, j, j));
                for (int k = 0; k < j; k++) {
                    int nk = nd[k];
                    sum += (f[nj] * g[nk] + f[nk] * g[nj]) * (kap ? el_intfdd(m, e, i, j, k) : el_intfff(m, e, i, j, k));
                }
                tmp[bs] += sum;
            }
        }
    }
}

static void intfg_pair_real(const tor_mesh *m, const double *f, const double *g, int kap, double *tmp)
{
    memset(tmp, 0, sizeof(double) * m->n);
    for (int e = 0; e < m->ne; e++) {
        const int *nd = m->el + (size_t)e * m->nn;
        for (int i = 0; i < m->nn; i++) {
            int bs = nd[i];
            for (int j = 0; j < m->nn; j++) {
                int nj = nd[j];
                double sum = (f[nj] * g[nj]) * (kap ? el_intfdd(m, e, i, j, j) : el_intfff(m, e, i, j, j));
                for (int k = 0; k < j; k++) {
                    int nk = nd[k];
                    sum += (f[nj] * g[nk] + f[nk] * g[nj]) * (kap ? el_intfdd(m, e, i, j, k) : el_intfff(m, e, i, j, k));
                }
                tmp[bs] += sum;
            }
        }
    }
}

typedef struct {
    const tor_mesh *m; int nq, nm, cplx, logscale, l0, l1;
    const double *dphi, *aphi, *proj; const int *link_ofs, *link_m; double *J; int nqm;
} jac_job;

/* the source of link l (link_ofs ascending) */
static int link_source(const int *link_ofs, int nq, int l)
{
    int a = 0, b = nq;  /* link_ofs[a] <= l < link_ofs[b] */
    while (b - a > 1) {
        int c = (a + b) / 2;
        if (link_ofs[c] <= l) a = c;
        else b = c;
    }
    return a;
}

/* a range of links [l0, l1): the same per-link sums as jacobian.cc:441-497
   (complex) and 738-802 (CW) whatever the split, so the result does not
   depend on the thread count */
static void *jac_worker(void *arg)
{
    jac_job *jb = arg;
    const tor_mesh *m = jb->m;
    int n = m->n, nqm = jb->nqm;
    if (jb->cplx) {
        zd *f = malloc(sizeof(zd) * n), *g = malloc(sizeof(zd) * n);
        zd *pm = malloc(sizeof(zd) * n), *pk = malloc(sizeof(zd) * n);
        int qf = -1;
        for (int l = jb->l0; l < jb->l1; l++) {
            int q = link_source(jb->link_ofs, jb->nq, l);
            if (q != qf) {
                for (int i = 0; i < n; i++) f[i] = jb->dphi[2 * ((size_t)q * n + i)] + I * jb->dphi[2 * ((size_t)q * n + i) + 1];
                qf = q;
            }
            int mm = jb->link_m[l];
            for (int i = 0; i < n; i++) g[i] = jb->aphi[2 * ((size_t)mm * n + i)] + I * jb->aphi[2 * ((size_t)mm * n + i) + 1];
            intfg_pair(m, f, g, 0, pm);
            intfg_pair(m, f, g, 1, pk);
            if (jb->logscale) {
                zd y = jb->proj[2 * l] + I * jb->proj[2 * l + 1];
                for (int k = 0; k < n; k++) { pm[k] = pm[k] / y; pk[k] = pk[k] / y; }
            }
            double *r0 = jb->J + (size_t)l * 2 * n, *r1 = jb->J + (size_t)(l + nqm) * 2 * n;
            for (int k = 0; k < n; k++) {
                r0[k] = -creal(pm[k]); r1[k] = -cimag(pm[k]);
                r0[k + n] = -creal(pk[k]); r1[k + n] = -cimag(pk[k]);
            }
        }
        free(f); free(g); free(pm); free(pk);
    } else {
        double *pm = malloc(sizeof(double) * n), *pk = malloc(sizeof(double) * n);
        for (int l = jb->l0; l < jb->l1; l++) {
            int q = link_source(jb->link_ofs, jb->nq, l);
            const double *f = jb->dphi + (size_t)q * n;
            const double *g = jb->aphi + (size_t)jb->link_m[l] * n;
            intfg_pair_real(m, f, g, 0, pm);
            intfg_pair_real(m, f, g, 1, pk);
            double sc = jb->logscale ? 1.0 / jb->proj[l] : 1.0;
            double *rm = jb->J + (size_t)l * n, *rk = jb->J + (size_t)(nqm + l) * n;
            for (int k = 0; k < n; k++) {
                rm[k] = -pm[k];
                rk[k] = -pk[k];
                if (jb->logscale) { rm[k] *= sc; rk[k] *= sc; }
            }
        }
        free(pm); free(pk);
    }
    return NULL;
}

/* Complex: J is (2 nQM) x (2 n) row-major, rows [Re; Im], columns [mua | kappa].
   Real (CW): J holds Jmua (nQM x n) followed by Jkap (nQM x n).
   proj: the linear projections (complex interleaved or real) used for LOG.
   nthreads host threads share the links (the reference forms J serially,
   jacobian.cc:380-497; every link's row is the same sum either way). */
void tor_jacobian(const tor_mesh *m, int nq, int nm, const double *dphi, const double *aphi,
                  const double *proj, const int *link_ofs, const int *link_m, int cplx, int logscale,
                  double *J, int nthreads)
{
    int nqm = link_ofs[nq];
    (void)nm;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > nqm) nthreads = nqm > 0 ? nqm : 1;
    jac_job *jobs = malloc(sizeof(jac_job) * nthreads);
    pthread_t *th = malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; t++) {
        jac_job jb = {m, nq, nm, cplx, logscale, (int)(((long long)t * nqm) / nthreads),
                      (int)(((long long)(t + 1) * nqm) / nthreads), dphi, aphi, proj, link_ofs, link_m, J, nqm};
        jobs[t] = jb;
        if (nthreads > 1) pthread_create(&th[t], NULL, jac_worker, &jobs[t]);
        else jac_worker(&jobs[t]);
    }
    if (nthreads > 1) for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(jobs); free(th);
}

/* ------------------------------------------------------------------------ */
/* Pixel raster and the grid-basis Jacobian                                  */
/* ------------------------------------------------------------------------ */

/* Element_Unstructured::GContains (element.cc:553-563): the element's
   bounding box widened by 1e-8, then Element::GContains (element.cc:178-182):
   LContains(Local(p)) with the padded test (pad = true, tri3.cc:191-200,
   tet4.cc:268-279); Local per tri3.cc:134-144, tet4.cc:186-196. */
static int el_gcontains(const tor_mesh *m, int e, const double *p)
{
    const int dim = m->dim, nn = m->nn;
    const int *nd = m->el + (size_t)e * nn;
    for (int d = 0; d < dim; d++) {  /* Element_Unstructured::Initialise (element.cc:528-536) */
        double lo = 1e10, hi = -1e10;
        for (int i = 0; i < nn; i++) {
            double v = m->x[(size_t)nd[i] * dim + d];
            if (v < lo) lo = v;
            if (v > hi) hi = v;
        }
        if (p[d] < lo - 1e-8 || p[d] > hi + 1e-8) return 0;
    }
    const double *g = m->geo + (size_t)e * 16;
    const double EPS = 1e-8;
    if (dim == 2) {
        double scale = 1.0 / (g[0] + g[1] + g[2]);
        double l0 = (g[1] + g[4] * p[0] + g[7] * p[1]) * scale;
        double l1 = (g[2] + g[5] * p[0] + g[8] * p[1]) * scale;
        return l0 + EPS >= 0.0 && l1 + EPS >= 0.0 && l0 + l1 - EPS <= 1.0;
    }
    const double *a = g, *b = g + 4, *c = g + 8, *dd = g + 12;
    double scale = 1.0 / (a[0] + a[1] + a[2] + a[3]);
    double l[3];
    for (int r = 0; r < 3; r++) l[r] = (a[r + 1] + b[r + 1] * p[0] + c[r + 1] * p[1] + dd[r + 1] * p[2]) * scale;
    return l[0] + EPS >= 0.0 && l[1] + EPS >= 0.0 && l[2] + EPS >= 0.0 && l[0] + l[1] + l[2] - EPS <= 1.0;
}

/* Whether any element contains p (Mesh::ElFind, mesh.cc:248-290, searches
   from the last element found; whether one is found does not depend on the
   search order) */
int tor_el_found(const tor_mesh *m, const double *p)
{
    for (int e = 0; e < m->ne; e++)
        if (el_gcontains(m, e, p)) return 1;
    return 0;
}

/* Triangle3::Intersection (tri3.cc:698-780) with add_endpoints false and
   boundary_only true, in the element's local frame.  The reference tests the
   flag of side 1 against the edge x = 0 and the flag of side 2 against the
   edge x + y = 1, although side 1 joins nodes 1-2 (x + y = 1) and side 2
   nodes 2-0 (x = 0) (tri3.cc:121-127); the same pairing is kept.  The points
   found are then kept only where they lie on the segment p1-p2. */
static int tri_bnd_intersect(const unsigned char *bs, const double *p1, const double *p2, double s[4][3])
{
    const double EPS = 1e-12;
    int k = 0;
    if (bs[0] && p1[1] * p2[1] < 0.0) {
        double xs = p1[0] - p1[1] / (p2[1] - p1[1]) * (p2[0] - p1[0]);
        if (xs > -EPS && xs < 1.0 + EPS) { s[k][0] = xs; s[k][1] = 0.0; k++; }
    }
    if (bs[1] && p1[0] * p2[0] < 0.0) {
        double ys = p1[1] - p1[0] / (p2[0] - p1[0]) * (p2[1] - p1[1]);
        if (ys > -EPS && ys < 1.0 + EPS) { s[k][0] = 0.0; s[k][1] = ys; k++; }
    }
    if (bs[2]) {
        double xs;
        if (fabs(p1[0] - p2[0]) > EPS) {
            double a = (p1[1] - p2[1]) / (p1[0] - p2[0]);
            double c = p1[1] - a * p1[0];
            xs = (1.0 - c) / (a + 1.0);
        } else {
            xs = p1[0];
        }
        if (xs > -EPS && xs < 1.0 + EPS) { s[k][0] = xs; s[k][1] = 1.0 - xs; k++; }
    }
    if (k) {
        int d = 0, j = 0;
        double dp = p2[0] - p1[0];
        if (fabs(dp) < EPS) { d = 1; dp = p2[1] - p1[1]; }
        for (int i = 0; i < k; i++) {
            double a = (s[i][d] - p1[d]) / dp;
            if (a < -EPS || a > 1.0 + EPS) continue;
            s[j][0] = s[i][0]; s[j][1] = s[i][1]; j++;
        }
        k = j;
    }
    return k;
}

/* Tetrahedron4::Intersection (tet4.cc:1222-1283) with boundary_only true: the
   line through p1 and p2 (not only the segment) against the planes of the
   boundary faces, each point kept where it lies in the face's triangle. */
static int tet_bnd_intersect(const unsigned char *bs, const double *p1, const double *p2, double s[4][3])
{
    int n = 0;
    double a, rx, ry, rz;
    double sx = p1[0], sy = p1[1], sz = p1[2];
    double dx = p2[0] - p1[0], dy = p2[1] - p1[1], dz = p2[2] - p1[2];
    if (bs[0] && dz != 0.0) {
        a = -sz / dz; rx = sx + a * dx; ry = sy + a * dy;
        if (rx >= 0 && ry >= 0 && rx + ry <= 1) { s[n][0] = rx; s[n][1] = ry; s[n][2] = 0.0; n++; }
    }
    if (bs[1] && dy != 0.0) {
        a = -sy / dy; rx = sx + a * dx; rz = sz + a * dz;
        if (rx >= 0 && rz >= 0 && rx + rz <= 1) { s[n][0] = rx; s[n][1] = 0.0; s[n][2] = rz; n++; }
    }
    if (bs[2] && dx != 0.0) {
        a = -sx / dx; ry = sy + a * dy; rz = sz + a * dz;
        if (ry >= 0 && rz >= 0 && ry + rz <= 1) { s[n][0] = 0.0; s[n][1] = ry; s[n][2] = rz; n++; }
    }
    if (bs[3] && (dx + dy + dz) != 0.0) {
        a = (1 - sx - sy - sz) / (dx + dy + dz);
        rx = sx + a * dx; ry = sy + a * dy; rz = sz + a * dz;
        if (rx >= 0 && ry >= 0 && rx + ry <= 1) { s[n][0] = rx; s[n][1] = ry; s[n][2] = rz; n++; }
    }
    return n;
}

/* Mesh::BndIntersect (mesh.cc:1369-1453): in 3D the line must first cross
   the mesh's bounding box (Mesh::BoundingBox, mesh.cc:1341-1360); then every
   element with a boundary side intersects the line in its local frame
   (Element::GlobalIntersection, element.cc:505-511), each point is mapped
   back (Element::Global, element.cc:164-176) and the one nearest pt1 (the
   first of equal distance) is the result.  Returns 0, or 1 when nothing is
   found (the reference then returns an empty point). */
int tor_bnd_intersect(const tor_mesh *m, const double *pt1, const double *pt2, double *out)
{
    const int dim = m->dim, nn = m->nn, nside = dim == 2 ? 3 : 4;
    if (dim > 2) {
        const double EPS = 1e-12;
        double lo[3] = {1e6, 1e6, 1e6}, hi[3] = {-1e6, -1e6, -1e6};
        for (int k = 0; k < m->n; k++)
            for (int d = 0; d < 3; d++) {
                double v = m->x[(size_t)k * 3 + d];
                if (v < lo[d]) lo[d] = v;
                if (v > hi[d]) hi[d] = v;
            }
        double d[3] = {pt2[0] - pt1[0], pt2[1] - pt1[1], pt2[2] - pt1[2]};
        int hit = 0;
        /* the faces z = const, then y = const, then x = const; u, v are the
           two other axes */
        static const int AX[3][3] = {{2, 0, 1}, {1, 0, 2}, {0, 1, 2}};
        for (int f = 0; f < 3 && !hit; f++) {
            int w = AX[f][0], u = AX[f][1], v = AX[f][2];
            if (d[w] == 0.0) continue;
            for (int side = 0; side < 2 && !hit; side++) {
                double a = ((side ? hi[w] : lo[w]) - pt1[w]) / d[w];
                double ru = pt1[u] + a * d[u], rv = pt1[v] + a * d[v];
                if (ru > lo[u] - EPS && ru < hi[u] + EPS && rv > lo[v] - EPS && rv < hi[v] + EPS) hit = 1;
            }
        }
        if (!hit) return 1;
    }
    double dstmin = 1e10;
    int found = 0;
    for (int e = 0; e < m->ne; e++) {
        const unsigned char *bs = m->bndside + (size_t)e * nside;
        int any = 0;
        for (int s = 0; s < nside; s++) any |= bs[s];
        if (!any) continue;
        const int *nd = m->el + (size_t)e * nn;
        const double *g = m->geo + (size_t)e * 16;
        double l1[3], l2[3], s[4][3];
        if (dim == 2) {  /* Triangle3::Local (tri3.cc:134-144) */
            double scale = 1.0 / (g[0] + g[1] + g[2]);
            l1[0] = (g[1] + g[4] * pt1[0] + g[7] * pt1[1]) * scale;
            l1[1] = (g[2] + g[5] * pt1[0] + g[8] * pt1[1]) * scale;
            l2[0] = (g[1] + g[4] * pt2[0] + g[7] * pt2[1]) * scale;
            l2[1] = (g[2] + g[5] * pt2[0] + g[8] * pt2[1]) * scale;
        } else {  /* Tetrahedron4::Local (tet4.cc:186-196) */
            const double *a = g, *b = g + 4, *c = g + 8, *dd = g + 12;
            double scale = 1.0 / (a[0] + a[1] + a[2] + a[3]);
            for (int r = 0; r < 3; r++) {
                l1[r] = (a[r + 1] + b[r + 1] * pt1[0] + c[r + 1] * pt1[1] + dd[r + 1] * pt1[2]) * scale;
                l2[r] = (a[r + 1] + b[r + 1] * pt2[0] + c[r + 1] * pt2[1] + dd[r + 1] * pt2[2]) * scale;
            }
        }
        int k = dim == 2 ? tri_bnd_intersect(bs, l1, l2, s) : tet_bnd_intersect(bs, l1, l2, s);
        for (int j = 0; j < k; j++) {
            double u[4], glob[3];
            if (dim == 2) { u[0] = 1.0 - s[j][0] - s[j][1]; u[1] = s[j][0]; u[2] = s[j][1]; }
            else { u[0] = 1.0 - s[j][0] - s[j][1] - s[j][2]; u[1] = s[j][0]; u[2] = s[j][1]; u[3] = s[j][2]; }
            for (int c = 0; c < dim; c++) {
                glob[c] = 0.0;
                for (int i = 0; i < nn; i++) glob[c] += u[i] * m->x[(size_t)nd[i] * dim + c];
            }
            double dst = pt_dist(pt1, glob, dim);
            if (dst < dstmin) {
                dstmin = dst;
                for (int c = 0; c < dim; c++) out[c] = glob[c];
                found = 1;
            }
        }
    }
    return found ? 0 : 1;
}

/* An "external" source position of QMMesh::LoadQM (qmmesh.cc:378-391): the
   unit direction n (the normal read with the position, or -q when the list
   says "default"; TVector::operator/= multiplies by the reciprocal,
   vector_imp.hpp:672-677; l2norm is the plain root of the sum of squares,
   vector_imp.hpp:1117-1120, 1290-1298) and the boundary point that
   BndIntersect finds from q + |q| n towards q.  nrm NULL: default normals.
   Returns 0, 2 for a zero normal, 1 when no boundary point is found. */
int tor_external_source(const tor_mesh *m, const double *q, const double *nrm, double *out)
{
    const int dim = m->dim;
    double n[3], s = 0.0, sq = 0.0, p1[3];
    for (int c = 0; c < dim; c++) n[c] = nrm ? nrm[c] : -q[c];
    for (int c = 0; c < dim; c++) s += fabs(n[c]) * fabs(n[c]);
    if (nrm && !(sqrt(s) > 0.0)) return 2;
    double inv = 1.0 / sqrt(s);
    for (int c = 0; c < dim; c++) n[c] *= inv;
    for (int c = 0; c < dim; c++) sq += fabs(q[c]) * fabs(q[c]);
    double len = sqrt(sq);
    for (int c = 0; c < dim; c++) p1[c] = q[c] + len * n[c];
    return tor_bnd_intersect(m, p1, q, out);
}

/* GenerateElementPixelRef (mesh.cc:2944-3014) on a grid of bdim points over
   the box [bbmin, bbmax]: elements in order, each claims the unclaimed grid
   points of its widened bounding box that it contains; -1 elsewhere */
static void pixel_elref(const tor_mesh *m, const int *bdim, const double *bbmin, const double *bbmax, int *elref)
{
    const int dim = m->dim, nn = m->nn;
    const int nx = bdim[0], ny = bdim[1], nz = dim > 2 ? bdim[2] : 1;
    const int glen = nx * ny * nz;
    double dW[3];
    for (int d = 0; d < dim; d++) dW[d] = (bbmax[d] - bbmin[d]) / (double)(bdim[d] - 1);
    for (int i = 0; i < glen; i++) elref[i] = -1;
    for (int e = 0; e < m->ne; e++) {
        const int *nd = m->el + (size_t)e * nn;
        double lo[3], hi[3];
        for (int d = 0; d < dim; d++) { lo[d] = 1e10; hi[d] = -1e10; }
        for (int i = 0; i < nn; i++)
            for (int d = 0; d < dim; d++) {
                double v = m->x[(size_t)nd[i] * dim + d];
                if (v < lo[d]) lo[d] = v;
                if (v > hi[d]) hi[d] = v;
            }
        int rmin[3] = {0, 0, 0}, rmax[3] = {1, 1, 1}, skip = 0;
        for (int d = 0; d < dim; d++) {
            lo[d] -= 1e-6;
            hi[d] += 1e-6;
            if (lo[d] > bbmax[d] || hi[d] < bbmin[d]) { skip = 1; break; }
            int a = (int)ceil((lo[d] - bbmin[d]) / dW[d]);
            int b = (int)floor((hi[d] - bbmin[d]) / dW[d]) + 1;
            rmin[d] = a > 0 ? a : 0;
            rmax[d] = b < bdim[d] ? b : bdim[d];
        }
        if (skip) continue;
        double p[3] = {0.0, 0.0, 0.0};
        for (int iz = rmin[2]; iz < rmax[2]; iz++) {
            if (dim > 2) p[2] = iz * dW[2] + bbmin[2];
            for (int iy = rmin[1]; iy < rmax[1]; iy++) {
                p[1] = iy * dW[1] + bbmin[1];
                for (int ix = rmin[0]; ix < rmax[0]; ix++) {
                    int idx = ix + nx * (iy + ny * iz);
                    if (elref[idx] >= 0) continue;
                    p[0] = ix * dW[0] + bbmin[0];
                    if (el_gcontains(m, e, p)) elref[idx] = e;
                }
            }
        }
    }
}

/* Raster_Pixel with the grid equal to the basis (raster.cc:18-83,
   raster_px.cc:10-48, the case bdim == gdim):
   - bounding box: Mesh::BoundingBox (mesh.cc:1341-1360), no padding;
   - elref: GenerateElementPixelRef (mesh.cc:2944-3014), the first element
     (in element order) containing each grid point, -1 outside;
   - B: GridMapMatrix (mesh.cc:2486-2554), row g = the containing element's
     global shape functions at the grid point (tri3.cc:231-240,
     tet4.cc:302-313), in the element's node order.
   Returns glen.  browptr: glen+1, bcol / bval: glen*nn (room for every row). */
int tor_raster_pixel(const tor_mesh *m, const int *bdim, double *bbmin, double *bbmax, int *elref,
                     int *browptr, int *bcol, double *bval)
{
    const int dim = m->dim, nn = m->nn;
    for (int d = 0; d < dim; d++) { bbmin[d] = 1e6; bbmax[d] = -1e6; }
    for (int k = 0; k < m->n; k++)
        for (int d = 0; d < dim; d++) {
            double v = m->x[(size_t)k * dim + d];
            if (v < bbmin[d]) bbmin[d] = v;
            if (v > bbmax[d]) bbmax[d] = v;
        }
    pixel_elref(m, bdim, bbmin, bbmax, elref);
    const int nx = bdim[0], ny = bdim[1], nz = dim > 2 ? bdim[2] : 1;
    const int glen = nx * ny * nz;
    double dW[3];
    for (int d = 0; d < dim; d++) dW[d] = (bbmax[d] - bbmin[d]) / (double)(bdim[d] - 1);
    int k = 0;
    browptr[0] = 0;
    for (int iz = 0, i = 0; iz < nz; iz++) {
        double p[3] = {0.0, 0.0, 0.0};
        if (dim > 2) p[2] = iz * dW[2] + bbmin[2];
        for (int iy = 0; iy < ny; iy++) {
            p[1] = iy * dW[1] + bbmin[1];
            for (int ix = 0; ix < nx; ix++, i++) {
                int e = elref[i];
                if (e >= 0) {
                    p[0] = ix * dW[0] + bbmin[0];
                    const int *nd = m->el + (size_t)e * nn;
                    const double *g = m->geo + (size_t)e * 16;
                    if (dim == 2) {
                        double scale = 1.0 / (2.0 * m->size[e]);
                        for (int j = 0; j < 3; j++) {
                            bcol[k] = nd[j];
                            bval[k++] = scale * (g[j] + g[3 + j] * p[0] + g[6 + j] * p[1]);
                        }
                    } else {
                        double scale = 1.0 / (6.0 * m->size[e]);
                        for (int j = 0; j < 4; j++) {
                            bcol[k] = nd[j];
                            bval[k++] = scale * (g[j] + g[4 + j] * p[0] + g[8 + j] * p[1] + g[12 + j] * p[2]);
                        }
                    }
                }
                browptr[i + 1] = k;
            }
        }
    }
    return glen;
}

/* NodeMapMatrix (mesh.cc:2695-2852): per mesh node, the bilinear /
   trilinear weights of the grid points around it, only those inside the
   mesh (elref >= 0), renormalised when some are missing (equal weights when
   their sum is below 1e-8); a node outside the box has no entries.  Zero
   weights are dropped (Shrink).  browptr: n+1, bcol / bval: n*2^dim. */
void tor_node_map(const tor_mesh *m, const int *bdim, const double *bbmin, const double *bbmax, const int *elref,
                  int *browptr, int *bcol, double *bval)
{
    const int dim = m->dim, nx = bdim[0], ny = bdim[1];
    double dW[3];
    for (int d = 0; d < dim; d++) dW[d] = (bbmax[d] - bbmin[d]) / (double)(bdim[d] - 1);
    int idx = 0;
    browptr[0] = 0;
    for (int k = 0; k < m->n; k++) {
        const double *p = m->x + (size_t)k * dim;
        int i0[3] = {0, 0, 0}, inside = 1;
        double d0[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) {
            if (!(p[d] >= bbmin[d] && p[d] <= bbmax[d])) { inside = 0; break; }
            i0[d] = (int)((p[d] - bbmin[d]) / dW[d]);
            if (i0[d] < 0) i0[d] = 0;
            else if (i0[d] >= bdim[d] - 1) i0[d] = bdim[d] - 2;
            d0[d] = (p[d] - (i0[d] * dW[d] + bbmin[d])) / dW[d];
            if (d0[d] < 0.0) d0[d] = 0.0;
            else if (d0[d] > 1.0) d0[d] = 1.0;
        }
        if (inside) {
            const int idx0 = idx, ncorner = dim == 2 ? 4 : 8;
            for (int c = 0; c < ncorner; c++) {
                const int cx = c & 1, cy = (c >> 1) & 1, cz = (c >> 2) & 1;
                const int pix = (i0[0] + cx) + nx * ((i0[1] + cy) + ny * (dim > 2 ? i0[2] + cz : 0));
                if (elref[pix] < 0) continue;
                double w = (cx ? d0[0] : 1.0 - d0[0]) * (cy ? d0[1] : 1.0 - d0[1]);
                if (dim > 2) w *= cz ? d0[2] : 1.0 - d0[2];
                bcol[idx] = pix;
                bval[idx++] = w;
            }
            if (idx > idx0 && idx - idx0 < ncorner) {
                double wsum = 0.0;
                for (int i = idx0; i < idx; i++) wsum += bval[i];
                if (wsum > 1e-8)
                    for (int i = idx0; i < idx; i++) bval[i] /= wsum;
                else
                    for (int i = idx0; i < idx; i++) bval[i] = 1.0 / (double)(idx - idx0);
            }
            /* Shrink: drop zero weights, keeping the order */
            int o = idx0;
            for (int i = idx0; i < idx; i++)
                if (bval[i] != 0.0) { bcol[o] = bcol[i]; bval[o++] = bval[i]; }
            idx = o;
        }
        browptr[k + 1] = idx;
    }
}

/* ImageGradient (jacobian.cc:944-1060): central differences where both
   neighbours are in the mask, one-sided where one is, 0 outside the mask;
   spacing gsize/n (sic: n, not n-1).  mask NULL: every point counts as
   inside.  grad: dim planes of glen values. */
static void image_gradient(int dim, const int *gdim, const double *gsize, const zd *im, zd *grad, const int *mask)
{
    const int nx = gdim[0], ny = gdim[1], nz = dim >= 3 ? gdim[2] : 1, n = nx * ny * nz;
    const int stride[3] = {1, nx, nx * ny}, len[3] = {nx, ny, nz};
    for (int d = 0; d < dim; d++) {
        double h = gsize[d] / len[d], ih = 1.0 / h, i2h = 0.5 * ih;
        zd *gr = grad + (size_t)d * n;
        for (int z = 0, idx = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++, idx++) {
                    int c = d == 0 ? x : (d == 1 ? y : z);
                    int st = stride[d];
                    int bcnt = !mask || mask[idx] >= 0;
                    int blo = c > 0 && (!mask || mask[idx - st] >= 0);
                    int bhi = c < len[d] - 1 && (!mask || mask[idx + st] >= 0);
                    zd v;
                    if (blo && bhi) v = (im[idx + st] - im[idx - st]) * i2h;
                    else if (!bcnt) v = 0.0;
                    else if (blo) v = (im[idx] - im[idx - st]) * ih;
                    else if (bhi) v = (im[idx + st] - im[idx]) * ih;
                    else v = 0.0;
                    gr[idx] = v;
                }
    }
}

/* Map_MeshToGrid (raster.cc:188-199; RCompRowMatrix::Ax_cplx,
   crmatrix_imp.hpp:1302-1327): g = B f, row by row in entry order */
static void grid_map(int glen, const int *browptr, const int *bcol, const double *bval, const zd *f, zd *g)
{
    for (int r = 0; r < glen; r++) {
        double re = 0.0, im = 0.0;
        for (int j = browptr[r]; j < browptr[r + 1]; j++) {
            re += creal(f[bcol[j]]) * bval[j];
            im += cimag(f[bcol[j]]) * bval[j];
        }
        g[r] = re + I * im;
    }
}

/* ------------------------------------------------------------------------ */
/* Raster_Pixel with an intermediate grid (gdim != bdim)                      */
/* ------------------------------------------------------------------------ */

/* The basis-point / grid-point pairs of the linear pixel basis, in the loop
   order of Grid2LinPixMatrix (mesh.cc:3138-3320), LinPix2GridMatrix
   (3540-3640) and SubsampleLinPixel (3047-3136): basis points b in grid
   order (x fastest); for each, the fine grid points of its window
   [floor(x0 (g-1)), ceil(x1 (g-1))] per axis (z, then y, then x), kept where
   the distance to the basis point in basis spacings is below 1 along every
   axis and (elref given) the point lies in the mesh, with the weight
   t = (1 - dx)(1 - dy)(1 - dz).  Window points past the grid's last index
   (a window end rounded up from 1 + ulp) are skipped: the reference skips
   them too, by the distance test.  fn(ctx, b, g, t) per pair. */
typedef void (*linpix_fn)(void *ctx, int b, int g, double t);

static void linpix_pairs(int dim, const int *gdim, const int *bdim, const int *elref, linpix_fn fn, void *ctx)
{
    const int gx = gdim[0], gy = gdim[1], gz = dim > 2 ? gdim[2] : 1;
    const int bx = bdim[0], by = bdim[1], bz = dim > 2 ? bdim[2] : 1;
    const double nbx = bx - 1.0, nby = by - 1.0, nbz = bz - 1.0;
    const double dbx = 1.0 / nbx, dby = 1.0 / nby, dgx = 1.0 / (gx - 1.0), dgy = 1.0 / (gy - 1.0);
    double dbz = 0.0, dgz = 0.0, z = 0.0;
    if (bz > 1) { dbz = 1.0 / nbz; dgz = 1.0 / (gz - 1.0); }
    int gz0 = 0, gz1 = 0;
    for (int iz = 0; iz < bz; iz++) {
        if (bz > 1) {
            z = (double)iz * dbz;
            double z0 = iz ? (iz - 1) * dbz : 0.0, z1 = iz < bz - 1 ? (iz + 1) * dbz : 1.0;
            gz0 = (int)floor(z0 * (gz - 1));
            gz1 = (int)ceil(z1 * (gz - 1));
        }
        for (int iy = 0; iy < by; iy++) {
            double y = (double)iy * dby;
            double y0 = iy ? (iy - 1) * dby : 0.0, y1 = iy < by - 1 ? (iy + 1) * dby : 1.0;
            int gy0 = (int)floor(y0 * (gy - 1)), gy1 = (int)ceil(y1 * (gy - 1));
            for (int ix = 0; ix < bx; ix++) {
                double x = ix * dbx;
                double x0 = ix ? (ix - 1) * dbx : 0.0, x1 = ix < bx - 1 ? (ix + 1) * dbx : 1.0;
                int gx0 = (int)floor(x0 * (gx - 1)), gx1 = (int)ceil(x1 * (gx - 1));
                const int b = ix + (iy + iz * by) * bx;
                if (bz == 1) {
                    for (int yy = gy0; yy <= gy1 && yy < gy; yy++) {
                        double dy = fabs(yy * dgy - y) * nby;
                        if (dy >= 1.0) continue;
                        double idy = 1.0 - dy;
                        for (int xx = gx0; xx <= gx1 && xx < gx; xx++) {
                            int gidx = xx + yy * gx;
                            if (elref && elref[gidx] < 0) continue;
                            double dx = fabs(xx * dgx - x) * nbx;
                            if (dx >= 1.0) continue;
                            fn(ctx, b, gidx, (1.0 - dx) * idy);
                        }
                    }
                } else {
                    for (int zz = gz0; zz <= gz1 && zz < gz; zz++) {
                        double dz = fabs(zz * dgz - z) * nbz;
                        if (dz >= 1.0) continue;
                        double idz = 1.0 - dz;
                        for (int yy = gy0; yy <= gy1 && yy < gy; yy++) {
                            double dy = fabs(yy * dgy - y) * nby;
                            if (dy >= 1.0) continue;
                            double idyz = (1.0 - dy) * idz;
                            for (int xx = gx0; xx <= gx1 && xx < gx; xx++) {
                                int gidx = xx + (yy + zz * gy) * gx;
                                if (elref && elref[gidx] < 0) continue;
                                double dx = fabs(xx * dgx - x) * nbx;
                                if (dx >= 1.0) continue;
                                fn(ctx, b, gidx, (1.0 - dx) * idyz);
                            }
                        }
                    }
                }
            }
        }
    }
}

typedef struct { int *cnt, *rowptr, *col; double *val; int by_grid; } linpix_csr;

static void linpix_count(void *c, int b, int g, double t)
{
    linpix_csr *L = c;
    (void)t;
    L->cnt[L->by_grid ? g : b]++;
}

static void linpix_fill(void *c, int b, int g, double t)
{
    linpix_csr *L = c;
    const int r = L->by_grid ? g : b;
    const int i = L->rowptr[r] + L->cnt[r]++;
    L->col[i] = L->by_grid ? b : g;
    L->val[i] = t;
}

/* TCompRowMatrix::Shrink (crmatrix_imp.hpp:1774-1804): zero entries
   dropped, order kept.  Returns the new entry count. */
static int csr_shrink(int rows, int *rowptr, int *col, double *val)
{
    int o = 0, r0 = 0;
    for (int r = 0; r < rows; r++) {
        const int r1 = rowptr[r + 1];
        for (int i = r0; i < r1; i++)
            if (val[i] != 0.0) { col[o] = col[i]; val[o++] = val[i]; }
        r0 = r1;
        rowptr[r + 1] = o;
    }
    return o;
}

/* Grid2LinPixMatrix (mesh.cc:3138-3320), shrunk (raster_px.cc:24-25): the
   blen x glen map grid -> basis, row b the pairs of basis point b with their
   weights divided by the row's weight sum (0 when it is 0); by_grid: the
   LinPix2GridMatrix (mesh.cc:3540-3640, raster_px.cc:26-27), glen x blen,
   row g the weights t of the basis points that take grid point g, basis
   points ascending, not normalised.  col / val NULL: count only.  Returns
   the entry count. */
int tor_linpix_map(int dim, const int *gdim, const int *bdim, const int *elref, int by_grid, int *rowptr, int *col,
                   double *val)
{
    int glen = 1, blen = 1;
    for (int d = 0; d < dim; d++) { glen *= gdim[d]; blen *= bdim[d]; }
    const int rows = by_grid ? glen : blen;
    linpix_csr L = {calloc(rows, sizeof(int)), rowptr, col, val, by_grid};
    linpix_pairs(dim, gdim, bdim, elref, linpix_count, &L);
    rowptr[0] = 0;
    for (int r = 0; r < rows; r++) rowptr[r + 1] = rowptr[r] + L.cnt[r];
    if (!col) { free(L.cnt); return rowptr[rows]; }
    memset(L.cnt, 0, sizeof(int) * rows);
    linpix_pairs(dim, gdim, bdim, elref, linpix_fill, &L);
    free(L.cnt);
    if (!by_grid)
        for (int r = 0; r < rows; r++) {
            double wgt = 0.0;
            for (int i = rowptr[r]; i < rowptr[r + 1]; i++) wgt += val[i];
            for (int i = rowptr[r]; i < rowptr[r + 1]; i++) val[i] = wgt != 0.0 ? val[i] / wgt : 0.0;
        }
    return csr_shrink(rows, rowptr, col, val);
}

typedef struct { const double *gf; double *sum, *wgt; } subsample_ctx;

static void subsample_acc(void *c, int b, int g, double t)
{
    subsample_ctx *S = c;
    S->wgt[b] += t;
    S->sum[b] += t * S->gf[g];
}

/* SubsampleLinPixel (mesh.cc:3047-3136) without a mask, as the raster calls
   it for its support (raster.cc:58-64): bf[b] = sum t gf[g] / sum t over
   the pairs of basis point b (0 when the weights sum to 0) */
void tor_subsample_linpixel(int dim, const int *gdim, const int *bdim, const double *gf, double *bf)
{
    int blen = 1;
    for (int d = 0; d < dim; d++) blen *= bdim[d];
    double *wgt = calloc(blen, sizeof(double));
    memset(bf, 0, sizeof(double) * blen);
    subsample_ctx S = {gf, bf, wgt};
    linpix_pairs(dim, gdim, bdim, NULL, subsample_acc, &S);
    for (int b = 0; b < blen; b++) bf[b] = wgt[b] != 0.0 ? bf[b] / wgt[b] : 0.0;
    free(wgt);
}

/* TCompRowMatrix::AB (crmatrix_imp.hpp:1453-1541) then Shrink: C = A B, each
   row's entries in the order their columns first appear (A's row in order,
   then B's rows), each the sum of the products a b in that order.  ccol /
   cval hold at least the returned count (call once with ccol NULL for the
   count before shrinking, an upper bound).  Returns the entry count. */
int tor_csr_ab(int nr, int nc, const int *arp, const int *acol, const double *aval, const int *brp, const int *bcol,
               const double *bval, int *crp, int *ccol, double *cval)
{
    int *pos = malloc(sizeof(int) * (nc > 0 ? nc : 1));
    for (int j = 0; j < nc; j++) pos[j] = -1;
    int nz = 0;
    crp[0] = 0;
    for (int i = 0; i < nr; i++) {
        const int r0 = nz;
        for (int ra = arp[i]; ra < arp[i + 1]; ra++) {
            const int k = acol[ra];
            for (int rb = brp[k]; rb < brp[k + 1]; rb++) {
                const int j = bcol[rb];
                if (pos[j] >= 0) {
                    if (ccol) cval[pos[j]] += aval[ra] * bval[rb];
                } else {
                    pos[j] = nz;
                    if (ccol) { ccol[nz] = j; cval[nz] = aval[ra] * bval[rb]; }
                    nz++;
                }
            }
        }
        if (ccol)
            for (int t = r0; t < nz; t++) pos[ccol[t]] = -1;
        else  /* count pass: clear the marks by walking the row again */
            for (int ra = arp[i]; ra < arp[i + 1]; ra++)
                for (int rb = brp[acol[ra]]; rb < brp[acol[ra] + 1]; rb++) pos[bcol[rb]] = -1;
        crp[i + 1] = nz;
    }
    free(pos);
    return ccol ? csr_shrink(nr, crp, ccol, cval) : nz;
}

/* The basis side of Raster_Pixel(bdim, gdim) (raster.cc:18-83,
   raster_px.cc:10-48): support s = 1 at grid points in the mesh, bsupport =
   SubsampleLinPixel(s), solution points = basis points with bsupport > 0 in
   basis order.  sol2basis: room for blen.  Returns slen. */
int tor_basis_support(int dim, const int *gdim, const int *bdim, const int *elref, int *sol2basis)
{
    int glen = 1, blen = 1;
    for (int d = 0; d < dim; d++) { glen *= gdim[d]; blen *= bdim[d]; }
    double *s = malloc(sizeof(double) * glen), *bs = malloc(sizeof(double) * blen);
    for (int g = 0; g < glen; g++) s[g] = elref[g] >= 0 ? 1.0 : 0.0;
    tor_subsample_linpixel(dim, gdim, bdim, s, bs);
    int slen = 0;
    for (int b = 0; b < blen; b++)
        if (bs[b] > 0.0) sol2basis[slen++] = b;
    free(s); free(bs);
    return slen;
}

/* ------------------------------------------------------------------------ */
/* Raster_CubicPixel (raster_cp.cc): the cubic B-spline basis                */
/* ------------------------------------------------------------------------ */

/* The cubic B-spline weight at distance dr (in basis spacings), in the
   reference's form (raster_cp.cc:57-62, 204-209) */
static double cubic_weight(double dr)
{
    double dm2 = dr - 2.0, dm1 = dr - 1.0, dp1 = dr + 1.0, dp2 = dr + 2.0;
    return (fabs(dm2 * dm2 * dm2) - 4.0 * fabs(dm1 * dm1 * dm1) + 6.0 * fabs(dr * dr * dr) -
            4.0 * fabs(dp1 * dp1 * dp1) + fabs(dp2 * dp2 * dp2)) / 12.0;
}

/* The maps of Raster_CubicPixel(bdim, gdim) (raster_cp.cc:10-186).
   by_grid 0: G, blen x glen: row b holds the grid points inside the mesh
   (elref >= 0) in the axis-wise support window of b with a positive
   product of the axis weights (dr = |b_k - (j / iggrid) ibgrid|, < 2), in
   grid order, each divided by the row's sum.  by_grid 1: GI, glen x blen:
   row g (grid points inside the mesh only) holds Raster_CubicPixel::Value
   (raster_cp.cc:189-214) of every basis point at the grid point, nonzero
   ones in basis order.  ibgrid = (bdim - 1) / bbsize, iggrid = (gdim - 1) /
   bbsize.  col / val NULL: count only.  Returns the entry count. */
int tor_cubic_map(int dim, const int *gdim, const int *bdim, const double *bbmin, const double *bbmax,
                  const int *elref, int by_grid, int *rowptr, int *col, double *val)
{
    int glen = 1, blen = 1;
    for (int d = 0; d < dim; d++) { glen *= gdim[d]; blen *= bdim[d]; }
    double ib[3], ig[3];
    for (int d = 0; d < dim; d++) {
        ib[d] = (bdim[d] - 1) / (bbmax[d] - bbmin[d]);
        ig[d] = (gdim[d] - 1) / (bbmax[d] - bbmin[d]);
    }
    int nz = 0;
    rowptr[0] = 0;
    if (!by_grid) {
        double *sw[3], *grow = calloc(glen, sizeof(double));
        for (int d = 0; d < dim; d++) sw[d] = calloc(gdim[d], sizeof(double));
        for (int i = 0; i < blen; i++) {
            int bg[3] = {0, 0, 0}, r = i;
            if (dim == 3) { bg[2] = r / (bdim[0] * bdim[1]); r -= bg[2] * bdim[0] * bdim[1]; }
            bg[0] = r % bdim[0];
            bg[1] = r / bdim[0];
            int imin[3] = {100000, 100000, 0}, imax[3] = {-1, -1, 0};
            for (int k = 0; k < dim; k++) {
                imin[k] = 100000; imax[k] = -1;
                for (int j = 0; j < gdim[k]; j++) {
                    double dr = fabs(bg[k] - (j / ig[k]) * ib[k]);
                    if (fabs(dr) < 2.0) {
                        sw[k][j] = cubic_weight(dr);
                        if (j < imin[k]) imin[k] = j;
                        if (j > imax[k]) imax[k] = j;
                    }
                }
            }
            double gsum = 0.0;
            for (int jz = imin[2]; jz <= imax[2]; jz++)
                for (int jy = imin[1]; jy <= imax[1]; jy++)
                    for (int jx = imin[0]; jx <= imax[0]; jx++) {
                        int j = gdim[0] * gdim[1] * jz + jy * gdim[0] + jx, gr[3] = {jx, jy, jz};
                        if (elref[j] < 0) continue;
                        double v = 1.0;
                        for (int k = 0; k < dim; k++) v *= sw[k][gr[k]];
                        if (v > 0) { grow[j] = v; gsum += v; }
                    }
            for (int jz = imin[2]; jz <= imax[2]; jz++)
                for (int jy = imin[1]; jy <= imax[1]; jy++)
                    for (int jx = imin[0]; jx <= imax[0]; jx++) {
                        int j = gdim[0] * gdim[1] * jz + jy * gdim[0] + jx;
                        if (grow[j] != 0.0) {
                            if (col) { col[nz] = j; val[nz] = grow[j] / gsum; }
                            nz++;
                            grow[j] = 0.0;
                        }
                    }
            rowptr[i + 1] = nz;
        }
        for (int d = 0; d < dim; d++) free(sw[d]);
        free(grow);
    } else {
        for (int j = 0; j < glen; j++) {
            if (elref[j] >= 0) {
                int gg[3] = {0, 0, 0}, r = j;
                if (dim == 3) { gg[2] = r / (gdim[0] * gdim[1]); r -= gg[2] * gdim[0] * gdim[1]; }
                gg[0] = r % gdim[0];
                gg[1] = r / gdim[0];
                double p[3];
                for (int k = 0; k < dim; k++) p[k] = bbmin[k] + gg[k] / ig[k];
                for (int i = 0; i < blen; i++) {
                    int bg[3] = {0, 0, 0}, t = i;
                    if (dim == 3) { bg[2] = t / (bdim[0] * bdim[1]); t -= bg[2] * bdim[0] * bdim[1]; }
                    bg[0] = t % bdim[0];
                    bg[1] = t / bdim[0];
                    double v = 1.0;
                    for (int k = 0; k < dim; k++) {
                        double dr = fabs(bg[k] + (bbmin[k] - p[k]) * ib[k]);
                        if (dr >= 2.0) { v = 0.0; break; }
                        v *= cubic_weight(dr);
                    }
                    if (v != 0.0) {
                        if (col) { col[nz] = i; val[nz] = v; }
                        nz++;
                    }
                }
            }
            rowptr[j + 1] = nz;
        }
    }
    return nz;
}

/* ------------------------------------------------------------------------ */
/* The blob bases (Raster_Blob, raster_bl.cc, and its subclasses)            */
/* ------------------------------------------------------------------------ */

/* A blob raster (raster_bl.cc:9-75): the basis grid of bdim points over the
   mesh's bounding box, padded by npad = ceil(sup - 1e-6) layers on every
   side (igrid = (bdim - 1) / bbsize from the unpadded size); the element
   per padded grid point over the padded box; the solution points are the
   basis points within sup (in grid spacings) of a mesh node, in basis
   order.  Blob values (Value_nomask) at a point p for basis point b:
   r = (b - npad) + (bbmin - p) igrid,
   kind 1 Gaussian (raster_gb.cc): scale exp(-|r|^2 / sigma^2), |r|^2 < sup^2;
   kind 2 Hanning (raster_hb.cc): scale (1 + cos(pi |r| / sup)), |r| < sup;
   kind 3 ramp (raster_rb.cc): scale (1 - |r| / sup);
   kind 4 spline (raster_sb.cc): scale 4 sum over the knots xi_k = (k - 2)
   sup / 2 left of -|r| (the first two) of (-|r| - xi_k)^3 omega_k, omega_k
   = 1 / prod_{j != k} (xi_k - xi_j).  The scale: the subclass's start value
   (1, or 0.5 for Hanning) times 1 / mean over the nodes of the sum of the
   blob values there (ComputeBasisScale, raster_bl.cc:353-361).  nodevals:
   per node the nonzero blob values of the solution points, in their order
   (ComputeNodeValues, 82-114). */
typedef struct {
    int dim, kind, npad, pdim[3], blen, slen, n;
    double sup, sigma, scale, a2, isigma2, fac, isup, xi[5], iomega[5];
    double bbmin[3], bbmax[3], igrid[3], bbmin_pad[3], bbmax_pad[3];
    int *elref, *basis2sol, *sol2basis;
    int *nrp, *ncol;
    double *nval;
} tor_blob;

static double blob_value(const tor_blob *B, const double *p, int j)
{
    int ib = B->sol2basis[j], bg[3] = {0, 0, 0};
    if (B->dim == 3) { bg[2] = ib / (B->pdim[0] * B->pdim[1]); ib -= bg[2] * B->pdim[0] * B->pdim[1]; }
    bg[0] = ib % B->pdim[0];
    bg[1] = ib / B->pdim[0];
    double r2 = 0.0;
    for (int d = 0; d < B->dim; d++) {
        double r = (bg[d] - B->npad) + (B->bbmin[d] - p[d]) * B->igrid[d];
        r2 += fabs(r) * fabs(r);
    }
    if (B->kind == 1) {
        if (r2 >= B->a2) return 0.0;
        return B->scale * exp(-r2 * B->isigma2);
    }
    double rad = sqrt(r2);
    if (rad >= B->sup) return 0.0;
    if (B->kind == 2) return B->scale * (1.0 + cos(B->fac * rad));
    if (B->kind == 3) return B->scale * (1.0 - rad * B->isup);
    double x = -rad, dx = x - B->xi[0], d3 = dx * dx * dx, sum = d3 * B->iomega[0];
    if (x > B->xi[1]) {
        dx = x - B->xi[1];
        d3 = dx * dx * dx;
        sum += d3 * B->iomega[1];
    }
    sum *= 4.0;
    return B->scale * sum;
}

tor_blob *tor_blob_create(const tor_mesh *m, int kind, double sigma, double sup, const int *bdim)
{
    const double eps = 1e-6, PI = 3.14159265358979323846;
    const int dim = m->dim, n = m->n;
    tor_blob *B = calloc(1, sizeof(tor_blob));
    B->dim = dim; B->kind = kind; B->sup = sup; B->sigma = sigma; B->n = n;
    for (int d = 0; d < dim; d++) { B->bbmin[d] = 1e6; B->bbmax[d] = -1e6; }
    for (int k = 0; k < n; k++)
        for (int d = 0; d < dim; d++) {
            double v = m->x[(size_t)k * dim + d];
            if (v < B->bbmin[d]) B->bbmin[d] = v;
            if (v > B->bbmax[d]) B->bbmax[d] = v;
        }
    for (int d = 0; d < dim; d++) B->igrid[d] = (bdim[d] - 1.0) / (B->bbmax[d] - B->bbmin[d]);
    B->npad = (int)ceil(sup - eps);
    B->blen = 1;
    for (int d = 0; d < 3; d++) B->pdim[d] = 1;
    for (int d = 0; d < dim; d++) B->blen *= (B->pdim[d] = bdim[d] + 2 * B->npad);
    for (int d = 0; d < dim; d++) {
        B->bbmin_pad[d] = B->bbmin[d] - B->npad / B->igrid[d];
        B->bbmax_pad[d] = B->bbmax[d] + B->npad / B->igrid[d];
    }
    B->elref = malloc(sizeof(int) * B->blen);
    pixel_elref(m, B->pdim, B->bbmin_pad, B->bbmax_pad, B->elref);
    /* solution points */
    B->basis2sol = malloc(sizeof(int) * B->blen);
    B->sol2basis = malloc(sizeof(int) * B->blen);
    const double sup2 = sup * sup;
    const int nx = B->pdim[0], ny = B->pdim[1], nz = dim > 2 ? B->pdim[2] : 1;
    int idx = 0;
    B->slen = 0;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++, idx++) {
                double r[3] = {(double)i, (double)j, (double)k};
                B->basis2sol[idx] = -1;
                for (int nd = 0; nd < n; nd++) {
                    double rad2 = 0.0;
                    for (int d = 0; d < dim; d++) {
                        double dx = (m->x[(size_t)nd * dim + d] - B->bbmin[d]) * B->igrid[d] + B->npad - r[d];
                        rad2 += dx * dx;
                    }
                    if (rad2 < sup2) { B->basis2sol[idx] = B->slen++; break; }
                }
                if (B->basis2sol[idx] >= 0) B->sol2basis[B->basis2sol[idx]] = idx;
            }
    /* the subclass's constants and start scale */
    B->a2 = sup * sup;
    B->scale = 1.0;
    if (kind == 1) B->isigma2 = 1.0 / (sigma * sigma);
    if (kind == 2) { B->fac = PI / sup; B->scale = 0.5; }
    if (kind == 3) B->isup = 1.0 / sup;
    if (kind == 4) {
        for (int i = 0; i <= 4; i++) B->xi[i] = (i - 2) * 0.5 * sup;
        for (int i = 0; i <= 4; i++) {
            B->iomega[i] = 1.0;
            for (int j = 0; j <= 4; j++)
                if (i != j) B->iomega[i] /= B->xi[i] - B->xi[j];
        }
    }
    /* ComputeBasisScale: 1 / mean over the nodes of the sum of the values */
    double tot = 0.0;
    for (int nd = 0; nd < n; nd++) {
        double sum = 0.0;
        for (int j = 0; j < B->slen; j++) sum += 1.0 * blob_value(B, m->x + (size_t)nd * dim, j);
        tot += sum;
    }
    double cbs = 1.0 / (tot / n);
    B->scale = kind == 1 ? cbs : B->scale * cbs;
    /* ComputeNodeValues */
    B->nrp = malloc(sizeof(int) * (n + 1));
    size_t cap = 64, nz2 = 0;
    B->ncol = malloc(sizeof(int) * cap);
    B->nval = malloc(sizeof(double) * cap);
    B->nrp[0] = 0;
    for (int nd = 0; nd < n; nd++) {
        for (int j = 0; j < B->slen; j++) {
            double v = blob_value(B, m->x + (size_t)nd * dim, j);
            if (v != 0.0) {
                if (nz2 == cap) {
                    cap *= 2;
                    B->ncol = realloc(B->ncol, sizeof(int) * cap);
                    B->nval = realloc(B->nval, sizeof(double) * cap);
                }
                B->ncol[nz2] = j;
                B->nval[nz2++] = v;
            }
        }
        B->nrp[nd + 1] = (int)nz2;
    }
    return B;
}

void tor_blob_info(const tor_blob *B, int *pdim, int *slen, int *nnz, double *scale, double *bbmin, double *bbmax)
{
    for (int d = 0; d < B->dim; d++) {
        pdim[d] = B->pdim[d];
        bbmin[d] = B->bbmin[d];
        bbmax[d] = B->bbmax[d];
    }
    *slen = B->slen;
    *nnz = B->nrp[B->n];
    *scale = B->scale;
}

void tor_blob_arrays(const tor_blob *B, int *elref, int *sol2basis, int *nrp, int *ncol, double *nval)
{
    memcpy(elref, B->elref, sizeof(int) * B->blen);
    memcpy(sol2basis, B->sol2basis, sizeof(int) * B->slen);
    memcpy(nrp, B->nrp, sizeof(int) * (B->n + 1));
    memcpy(ncol, B->ncol, sizeof(int) * B->nrp[B->n]);
    memcpy(nval, B->nval, sizeof(double) * B->nrp[B->n]);
}

void tor_blob_free(tor_blob *B)
{
    if (!B) return;
    free(B->elref); free(B->basis2sol); free(B->sol2basis); free(B->nrp); free(B->ncol); free(B->nval); free(B);
}

/* Raster_Blob::Map_MeshToBasis (raster_bl.cc:170-204): per solution point
   the node-value-weighted sum of the field over the nodes, in node order,
   divided by the sum of the weights (0 where that is 0); other basis
   points 0.  Complex fields component by component. */
static void blob_mesh_to_basis(const tor_blob *B, const zd *f, int cplx, zd *b)
{
    double *fr = calloc(B->slen, sizeof(double)), *fi = calloc(B->slen, sizeof(double));
    double *sum = calloc(B->slen, sizeof(double));
    for (int nd = 0; nd < B->n; nd++)
        for (int t = B->nrp[nd]; t < B->nrp[nd + 1]; t++) {
            const int j = B->ncol[t];
            const double v = B->nval[t];
            if (cplx) { fr[j] += creal(f[nd]) * v; fi[j] += cimag(f[nd]) * v; }
            else fr[j] += v * creal(f[nd]);
            sum[j] += v;
        }
    for (int i = 0; i < B->blen; i++) {
        const int j = B->basis2sol[i];
        if (j >= 0 && sum[j] != 0.0) b[i] = fr[j] / sum[j] + I * (fi[j] / sum[j]);
        else b[i] = 0.0;
    }
    free(fr); free(fi); free(sum);
}

/* Grid-basis Jacobian with a blob raster (GenerateJacobian_grid and
   GenerateJacobian_cw_grid as for the pixel raster): the fields mapped by
   Map_MeshToGrid = Map_MeshToBasis, image gradients on the padded grid with
   spacing bbsize / pdim (ImageGradient with the raster's GSize, the
   unpadded size), masked as for the pixel raster, Map_GridToSol = the
   solution points' values, J times prod bbsize / (pdim - 1). */
int tor_jacobian_blob(const tor_mesh *m, const tor_blob *B, int nq, int nm, const double *dphi, const double *aphi,
                      const double *proj, const int *link_ofs, const int *link_m, int cplx, int logscale, double *J)
{
    const int dim = m->dim, n = m->n, glen = B->blen, slen = B->slen, nqm = link_ofs[nq];
    double gsize[3];
    for (int d = 0; d < dim; d++) gsize[d] = B->bbmax[d] - B->bbmin[d];
    zd *fin = malloc(sizeof(zd) * n);
    zd *ag = malloc(sizeof(zd) * (size_t)nm * glen), *agr = malloc(sizeof(zd) * (size_t)nm * dim * glen);
    zd *dg = malloc(sizeof(zd) * glen), *dgr = malloc(sizeof(zd) * (size_t)dim * glen);
    zd *pm = malloc(sizeof(zd) * glen), *pk = malloc(sizeof(zd) * glen);
    for (int j = 0; j < nm; j++) {
        for (int i = 0; i < n; i++)
            fin[i] = cplx ? aphi[2 * ((size_t)j * n + i)] + I * aphi[2 * ((size_t)j * n + i) + 1] : aphi[(size_t)j * n + i];
        blob_mesh_to_basis(B, fin, cplx, ag + (size_t)j * glen);
        image_gradient(dim, B->pdim, gsize, ag + (size_t)j * glen, agr + (size_t)j * dim * glen, cplx ? B->elref : NULL);
    }
    double sz = 1.0;
    for (int d = 0; d < dim; d++) sz *= gsize[d] / (B->pdim[d] - 1.0);
    const size_t cols = cplx ? 2 * (size_t)slen : (size_t)slen;
    for (int q = 0; q < nq; q++) {
        for (int i = 0; i < n; i++)
            fin[i] = cplx ? dphi[2 * ((size_t)q * n + i)] + I * dphi[2 * ((size_t)q * n + i) + 1] : dphi[(size_t)q * n + i];
        blob_mesh_to_basis(B, fin, cplx, dg);
        image_gradient(dim, B->pdim, gsize, dg, dgr, B->elref);
        for (int l = link_ofs[q]; l < link_ofs[q + 1]; l++) {
            const int j = link_m[l];
            const zd *a = ag + (size_t)j * glen, *agj = agr + (size_t)j * dim * glen;
            zd y = cplx ? proj[2 * l] + I * proj[2 * l + 1] : proj[l];
            double *r0 = J + (size_t)l * cols, *r1 = J + (size_t)(l + nqm) * cols;
            for (int s = 0; s < slen; s++) {
                const int g = B->sol2basis[s];
                zd vm = -(dg[g] * a[g]), vk = 0.0;
                for (int d = 0; d < dim; d++) vk -= dgr[(size_t)d * glen + g] * agj[(size_t)d * glen + g];
                if (cplx) {
                    if (logscale) { vm = vm / y; vk = vk / y; }
                    r0[s] = creal(vm) * sz; r1[s] = cimag(vm) * sz;
                    r0[slen + s] = creal(vk) * sz; r1[slen + s] = cimag(vk) * sz;
                } else {
                    double wm = creal(vm) * sz, wk = creal(vk) * sz, iy = 1.0 / creal(y);
                    r0[s] = logscale ? wm * iy : wm;
                    r1[s] = logscale ? wk * iy : wk;
                }
            }
        }
    }
    free(fin); free(ag); free(agr); free(dg); free(dgr); free(pm); free(pk);
    return slen;
}

/* The data gradient's grid part with a blob raster (tor_gradient_grid with
   the blob's field map and solution points) */
void tor_gradient_blob(const tor_mesh *m, const tor_blob *B, int nq, const double *dphi, const double *wphi,
                       double *grad)
{
    const int dim = m->dim, n = m->n, glen = B->blen, slen = B->slen;
    double gsize[3];
    for (int d = 0; d < dim; d++) gsize[d] = B->bbmax[d] - B->bbmin[d];
    zd *df = malloc(sizeof(zd) * glen), *af = malloc(sizeof(zd) * glen);
    zd *dg = malloc(sizeof(zd) * (size_t)dim * glen), *ag = malloc(sizeof(zd) * (size_t)dim * glen);
    for (int q = 0; q < nq; q++) {
        blob_mesh_to_basis(B, (const zd *)(dphi + 2 * (size_t)q * n), 1, df);
        image_gradient(dim, B->pdim, gsize, df, dg, B->elref);
        blob_mesh_to_basis(B, (const zd *)(wphi + 2 * (size_t)q * n), 1, af);
        image_gradient(dim, B->pdim, gsize, af, ag, B->elref);
        for (int s = 0; s < slen; s++) {
            const int g = B->sol2basis[s];
            grad[s] -= creal(df[g] * af[g]);
        }
        for (int s = 0; s < slen; s++) {
            const int g = B->sol2basis[s];
            zd gk = 0.0;
            for (int d = 0; d < dim; d++) gk += dg[(size_t)d * glen + g] * ag[(size_t)d * glen + g];
            grad[slen + s] -= creal(gk);
        }
    }
    free(df); free(af); free(dg); free(ag);
}

/* The grid -> solution map of a Raster_Pixel (Map_GridToSol, raster.cc:
   374-390): with an intermediate grid, G (Grid2LinPixMatrix) applied to the
   grid vector (RCompRowMatrix::Ax / Ax_cplx, crmatrix_imp.hpp:1173-1190,
   1302-1327: sums in entry order of val x), then the solution points'
   basis values; without (G NULL) the grid values at the solution points.
   The real path's selection is D->Ax (raster_px.cc:147-150), 0 + 1 x. */
typedef struct {
    int slen, blen, kind;
    const int *sol;                   /* grid index (G NULL) or basis index per solution point */
    const int *grp, *gcol;            /* G: blen x glen, or NULL */
    const double *gval;
    zd *tmp;                          /* blen */
} grid2sol_t;

static void grid_to_sol(const grid2sol_t *M, const zd *x, int cplx, zd *out)
{
    const zd *b = x;
    if (M->grp) {
        for (int r = 0; r < M->blen; r++) {
            double re = 0.0, im = 0.0;
            for (int j = M->grp[r]; j < M->grp[r + 1]; j++) {
                if (cplx) {
                    re += creal(x[M->gcol[j]]) * M->gval[j];
                    im += cimag(x[M->gcol[j]]) * M->gval[j];
                } else {
                    re += M->gval[j] * creal(x[M->gcol[j]]);
                }
            }
            M->tmp[r] = re + I * im;
        }
        b = M->tmp;
    }
    /* the pixel raster's real map is D->Ax; the cubic raster's the base
       class's copy (raster.cc:292-303) */
    for (int k = 0; k < M->slen; k++)
        out[k] = (cplx || M->kind) ? b[M->sol[k]] : 0.0 + 1.0 * creal(b[M->sol[k]]);
}

/* the raster's grid -> solution map for basis bdim on grid gdim: kind 0
   Raster_Pixel (no G when the grids are equal; else the linear pixel map
   and the subsampled support), kind 1 Raster_CubicPixel (its G; the
   solution points are the basis points whose row of G is not empty,
   raster_cp.cc:170-178).  Allocates into M (free with grid2sol_free). */
static void grid2sol_init(int dim, int kind, const int *bdim, const int *gdim, const double *bbmin,
                          const double *bbmax, const int *elref, grid2sol_t *M)
{
    int glen = 1, blen = 1, same = 1;
    for (int d = 0; d < dim; d++) { glen *= gdim[d]; blen *= bdim[d]; same &= gdim[d] == bdim[d]; }
    int *sol = malloc(sizeof(int) * (same ? glen : blen) + sizeof(int) * blen);
    M->blen = blen;
    M->grp = M->gcol = NULL;
    M->gval = NULL;
    M->tmp = NULL;
    if (same && kind == 0) {
        M->slen = 0;
        for (int g = 0; g < glen; g++) if (elref[g] >= 0) sol[M->slen++] = g;
    } else {
        int *rp = malloc(sizeof(int) * (blen + 1));
        int nz = kind ? tor_cubic_map(dim, gdim, bdim, bbmin, bbmax, elref, 0, rp, NULL, NULL)
                      : tor_linpix_map(dim, gdim, bdim, elref, 0, rp, NULL, NULL);
        int *col = malloc(sizeof(int) * (nz > 0 ? nz : 1));
        double *val = malloc(sizeof(double) * (nz > 0 ? nz : 1));
        if (kind) tor_cubic_map(dim, gdim, bdim, bbmin, bbmax, elref, 0, rp, col, val);
        else tor_linpix_map(dim, gdim, bdim, elref, 0, rp, col, val);
        M->grp = rp; M->gcol = col; M->gval = val;
        M->tmp = malloc(sizeof(zd) * blen);
        if (kind) {
            M->slen = 0;
            for (int b = 0; b < blen; b++) if (rp[b + 1] > rp[b]) sol[M->slen++] = b;
        } else {
            M->slen = tor_basis_support(dim, gdim, bdim, elref, sol);
        }
    }
    M->kind = kind;
    M->sol = sol;
}

static void grid2sol_free(grid2sol_t *M)
{
    free((void *)M->sol); free((void *)M->grp); free((void *)M->gcol); free((void *)M->gval); free(M->tmp);
}

/* Grid-basis Jacobian for Raster_Pixel(bdim, gdim) (kind 0) or
   Raster_CubicPixel(bdim, gdim) (kind 1): the fields mapped on the
   grid gdim (Map_MeshToGrid), their image gradients on it, the PMDFs per
   grid point, then Map_GridToSol into the solution basis.
   Complex (GenerateJacobian_grid with projections, jacobian.cc:289-373):
   PMDF_mua = -(f a), PMDF_kap = -sum_d grad_d f grad_d a (jacobian.cc:58-72),
   both gradients masked by elref; LOG divides by y (PMDF_log, 76-79) before
   the map; J(l, s) = Re, J(l+nQM, s) = Im, kappa at column slen + s; then
   J *= prod gsize/(bdim-1).
   Real (GenerateJacobian_cw_grid, jacobian.cc:516-712, the threaded engine):
   the adjoint gradient is NOT masked; Jmua = PMDF_mua, Jkap = PMDF_kap (rows
   nQM + l) mapped, times the voxel scale, then, for LOG data, each row times
   1/y (GenerateJacobian_cw, 178-193).
   J: complex (2 nQM) x (2 slen), real (2 nQM) x slen.  Returns slen. */
int tor_jacobian_grid(const tor_mesh *m, int kind, const int *bdim, const int *gdim, int nq, int nm,
                      const double *dphi, const double *aphi, const double *proj, const int *link_ofs,
                      const int *link_m, int cplx, int logscale, double *J)
{
    const int dim = m->dim, nn = m->nn, n = m->n;
    int glen = 1;
    for (int d = 0; d < dim; d++) glen *= gdim[d];
    double bbmin[3], bbmax[3], gsize[3];
    int *elref = malloc(sizeof(int) * glen), *browptr = malloc(sizeof(int) * (glen + 1));
    int *bcol = malloc(sizeof(int) * (size_t)glen * nn);
    double *bval = malloc(sizeof(double) * (size_t)glen * nn);
    tor_raster_pixel(m, gdim, bbmin, bbmax, elref, browptr, bcol, bval);
    for (int d = 0; d < dim; d++) gsize[d] = bbmax[d] - bbmin[d];
    grid2sol_t M;
    grid2sol_init(dim, kind, bdim, gdim, bbmin, bbmax, elref, &M);
    const int slen = M.slen;
    const int nqm = link_ofs[nq];
    zd *fin = malloc(sizeof(zd) * n);
    zd *ag = malloc(sizeof(zd) * (size_t)nm * glen), *agr = malloc(sizeof(zd) * (size_t)nm * dim * glen);
    zd *dg = malloc(sizeof(zd) * glen), *dgr = malloc(sizeof(zd) * (size_t)dim * glen);
    zd *pm = malloc(sizeof(zd) * glen), *pk = malloc(sizeof(zd) * glen);
    zd *sm = malloc(sizeof(zd) * (slen > 0 ? slen : 1)), *sk = malloc(sizeof(zd) * (slen > 0 ? slen : 1));
    for (int j = 0; j < nm; j++) {
        for (int i = 0; i < n; i++)
            fin[i] = cplx ? aphi[2 * ((size_t)j * n + i)] + I * aphi[2 * ((size_t)j * n + i) + 1] : aphi[(size_t)j * n + i];
        grid_map(glen, browptr, bcol, bval, fin, ag + (size_t)j * glen);
        image_gradient(dim, gdim, gsize, ag + (size_t)j * glen, agr + (size_t)j * dim * glen, cplx ? elref : NULL);
    }
    double sz = 1.0;
    for (int d = 0; d < dim; d++) sz *= gsize[d] / (bdim[d] - 1.0);
    const size_t cols = cplx ? 2 * (size_t)slen : (size_t)slen;
    for (int q = 0; q < nq; q++) {
        for (int i = 0; i < n; i++)
            fin[i] = cplx ? dphi[2 * ((size_t)q * n + i)] + I * dphi[2 * ((size_t)q * n + i) + 1] : dphi[(size_t)q * n + i];
        grid_map(glen, browptr, bcol, bval, fin, dg);
        image_gradient(dim, gdim, gsize, dg, dgr, elref);
        for (int l = link_ofs[q]; l < link_ofs[q + 1]; l++) {
            const int j = link_m[l];
            const zd *a = ag + (size_t)j * glen, *agj = agr + (size_t)j * dim * glen;
            zd y = cplx ? proj[2 * l] + I * proj[2 * l + 1] : proj[l];
            for (int g = 0; g < glen; g++) {
                pm[g] = -(dg[g] * a[g]);
                zd kk = 0.0;
                for (int d = 0; d < dim; d++) kk -= dgr[(size_t)d * glen + g] * agj[(size_t)d * glen + g];
                pk[g] = kk;
                if (cplx && logscale) { pm[g] = pm[g] / y; pk[g] = pk[g] / y; }
            }
            grid_to_sol(&M, pm, cplx, sm);
            grid_to_sol(&M, pk, cplx, sk);
            double *r0 = J + (size_t)l * cols, *r1 = J + (size_t)(l + nqm) * cols;
            if (cplx) {
                for (int s = 0; s < slen; s++) {
                    r0[s] = creal(sm[s]) * sz; r1[s] = cimag(sm[s]) * sz;
                    r0[slen + s] = creal(sk[s]) * sz; r1[slen + s] = cimag(sk[s]) * sz;
                }
            } else {
                double iy = 1.0 / creal(y);
                for (int s = 0; s < slen; s++) {
                    double vm = creal(sm[s]) * sz, vk = creal(sk[s]) * sz;
                    r0[s] = logscale ? vm * iy : vm;
                    r1[s] = logscale ? vk * iy : vk;
                }
            }
        }
    }
    grid2sol_free(&M);
    free(elref); free(browptr); free(bcol); free(bval); free(fin);
    free(ag); free(agr); free(dg); free(dgr); free(pm); free(pk); free(sm); free(sk);
    return slen;
}

/* Element-basis Jacobian (GenerateJacobian_mesh with elbasis, jacobian.cc:
   441-497, complex, projections given; GenerateJacobian_cw_mesh 738-802 and
   the LOG row scaling of GenerateJacobian_cw 178-193, real), with IntFG_el /
   IntGradFGradG_el (jacobian.cc:884-939): per element sum_ij (f_i g_j)
   IntFF(i,j) and (f_i g_j) IntDD(i,j).  J: complex (2 nQM) x (2 ne) rows
   -Re / -Im, kappa at column ne + e; real (2 nQM) x ne [mua ; kappa]. */
void tor_jacobian_el(const tor_mesh *m, int nq, int nm, const double *dphi, const double *aphi,
                     const double *proj, const int *link_ofs, const int *link_m, int cplx, int logscale, double *J)
{
    const int n = m->n, ne = m->ne, nn = m->nn, nqm = link_ofs[nq];
    (void)nm;
    const size_t cols = cplx ? 2 * (size_t)ne : (size_t)ne;
    for (int q = 0; q < nq; q++)
        for (int l = link_ofs[q]; l < link_ofs[q + 1]; l++) {
            const int j = link_m[l];
            double *r0 = J + (size_t)l * cols, *r1 = J + (size_t)(l + nqm) * cols;
            for (int e = 0; e < ne; e++) {
                const int *nd = m->el + (size_t)e * nn;
                if (cplx) {
                    zd sm = 0.0, sk = 0.0;
                    for (int a = 0; a < nn; a++)
                        for (int b = 0; b < nn; b++) {
                            zd f = dphi[2 * ((size_t)q * n + nd[a])] + I * dphi[2 * ((size_t)q * n + nd[a]) + 1];
                            zd g = aphi[2 * ((size_t)j * n + nd[b])] + I * aphi[2 * ((size_t)j * n + nd[b]) + 1];
                            sm += (f * g) * el_intff(m, e, a, b);
                            sk += (f * g) * m->intdd[((size_t)e * nn + a) * nn + b];
                        }
                    zd pm = 0.0 + sm, pk = 0.0 + sk;
                    if (logscale) {
                        zd y = proj[2 * l] + I * proj[2 * l + 1];
                        pm = pm / y;
                        pk = pk / y;
                    }
                    r0[e] = -creal(pm); r1[e] = -cimag(pm);
                    r0[ne + e] = -creal(pk); r1[ne + e] = -cimag(pk);
                } else {
                    double sm = 0.0, sk = 0.0;
                    for (int a = 0; a < nn; a++)
                        for (int b = 0; b < nn; b++) {
                            double fg = dphi[(size_t)q * n + nd[a]] * aphi[(size_t)j * n + nd[b]];
                            sm += fg * el_intff(m, e, a, b);
                            sk += fg * m->intdd[((size_t)e * nn + a) * nn + b];
                        }
                    double vm = -(0.0 + sm), vk = -(0.0 + sk);
                    if (logscale) {
                        double iy = 1.0 / proj[l];
                        vm *= iy;
                        vk *= iy;
                    }
                    r0[e] = vm;
                    r1[e] = vk;
                }
            }
        }
}

/* The data gradient of toast's Gradient (GetGradient / AddDataGradient,
   src/python/toastmodule.cc:1745-1887), in two parts around the adjoint
   solves.  Weights: for source q, w_q = sum over its links (in order) of
   mvec_m * (a r dn, -a i dn) and then mvec_m * (-p i dn, -p r dn), with
   y = r + i i the linear projection, dn = 1/|y|^2, a = -2 b_mod / sd_mod,
   p = -2 b_arg / sd_arg, b = (data - model) / sd, model = (ln|y|, arg y).
   data, sd: 2 nQM (log amplitude block, then phase block).  W: nq x n. */
void tor_gradient_weights(int nq, int n, const double *mvec, const double *ylin, const double *ylog,
                          const double *data, const double *sd, const int *link_ofs, const int *link_m, double *W)
{
    const int nqm = link_ofs[nq];
    for (int q = 0; q < nq; q++) {
        zd *w = (zd *)(W + 2 * (size_t)q * n);
        for (int i = 0; i < n; i++) w[i] = 0.0;
        for (int l = link_ofs[q]; l < link_ofs[q + 1]; l++) {
            const zd *row = (const zd *)(mvec + 2 * (size_t)link_m[l] * n);
            const double rp = ylin[2 * l], ip = ylin[2 * l + 1], dn = 1.0 / (rp * rp + ip * ip);
            const double bm = (data[l] - ylog[2 * l]) / sd[l];
            const double ba = (data[nqm + l] - ylog[2 * l + 1]) / sd[nqm + l];
            double t = -2.0 * bm / (1.0 * sd[l]);
            const zd c1 = t * rp * dn + I * (-t * ip * dn);
            for (int i = 0; i < n; i++) w[i] += row[i] * c1;
            t = -2.0 * ba / (1.0 * sd[nqm + l]);
            const zd c2 = -t * ip * dn + I * (-t * rp * dn);
            for (int i = 0; i < n; i++) w[i] += row[i] * c2;
        }
    }
}

/* Grid part: per source, both fields resampled on the Raster_Pixel grid
   gdim, their masked image gradients, then grad_mua -= Re(Map_GridToSol(f a))
   and grad_kappa -= Re(Map_GridToSol(sum_d grad_d f grad_d a)) (no voxel
   scaling).  dphi, wphi: nq x n complex; grad: 2 slen, in/out. */
void tor_gradient_grid(const tor_mesh *m, int kind, const int *bdim, const int *gdim, int nq, const double *dphi,
                       const double *wphi, double *grad)
{
    const int dim = m->dim, nn = m->nn, n = m->n;
    int glen = 1;
    for (int d = 0; d < dim; d++) glen *= gdim[d];
    double bbmin[3], bbmax[3], gsize[3];
    int *elref = malloc(sizeof(int) * glen), *browptr = malloc(sizeof(int) * (glen + 1));
    int *bcol = malloc(sizeof(int) * (size_t)glen * nn);
    double *bval = malloc(sizeof(double) * (size_t)glen * nn);
    tor_raster_pixel(m, gdim, bbmin, bbmax, elref, browptr, bcol, bval);
    for (int d = 0; d < dim; d++) gsize[d] = bbmax[d] - bbmin[d];
    grid2sol_t M;
    grid2sol_init(dim, kind, bdim, gdim, bbmin, bbmax, elref, &M);
    const int slen = M.slen;
    zd *df = malloc(sizeof(zd) * glen), *af = malloc(sizeof(zd) * glen), *pr = malloc(sizeof(zd) * glen);
    zd *dg = malloc(sizeof(zd) * (size_t)dim * glen), *ag = malloc(sizeof(zd) * (size_t)dim * glen);
    zd *sv = malloc(sizeof(zd) * (slen > 0 ? slen : 1));
    for (int q = 0; q < nq; q++) {
        grid_map(glen, browptr, bcol, bval, (const zd *)(dphi + 2 * (size_t)q * n), df);
        image_gradient(dim, gdim, gsize, df, dg, elref);
        grid_map(glen, browptr, bcol, bval, (const zd *)(wphi + 2 * (size_t)q * n), af);
        image_gradient(dim, gdim, gsize, af, ag, elref);
        for (int g = 0; g < glen; g++) pr[g] = df[g] * af[g];
        grid_to_sol(&M, pr, 1, sv);
        for (int s = 0; s < slen; s++) grad[s] -= creal(sv[s]);
        for (int g = 0; g < glen; g++) {
            zd gk = 0.0;
            for (int d = 0; d < dim; d++) gk += dg[(size_t)d * glen + g] * ag[(size_t)d * glen + g];
            pr[g] = gk;
        }
        grid_to_sol(&M, pr, 1, sv);
        for (int s = 0; s < slen; s++) grad[slen + s] -= creal(sv[s]);
    }
    grid2sol_free(&M);
    free(elref); free(browptr); free(bcol); free(bval); free(df); free(af); free(pr); free(dg); free(ag); free(sv);
}

/* A_Keijzer (param.cc:24-32) */
double tor_a_keijzer(double n)
{
    double th = asin(1.0 / n);
    double costh = fabs(cos(th));
    double R0 = ((n - 1.0) * (n - 1.0)) / ((n + 1.0) * (n + 1.0));
    return (2.0 / (1.0 - R0) - 1.0 + costh * costh * costh) / (1.0 - costh * costh);
}

/* ------------------------------------------------------------------------ */
/* Direct solver (LSOLVER_DIRECT)                                            */
/* ------------------------------------------------------------------------ */
/* The reference's direct path for real systems: SymbolicCholeskyFactorize
   (src/libmath/crmatrix_imp.hpp:2067-2073 -> symbolic_cholesky_factor,
   src/libmath/cr_cholesky.cc:76-233: the row set of each column merged into
   its elimination-tree parent), CholeskyFactorize (crmatrix_imp.hpp:2104-2164:
   left-looking columns, d_c = sqrt of the pivot, recover mode sets 1e-10) and
   CholeskySubst (crmatrix_imp.hpp:2267-2295).  Complex systems go through
   SuperLU in the reference (src/libstoast/fwdsolver_zslu.cc: zgssvx, natural
   column order, no equilibration, no refinement); here they take the same
   Cholesky code in complex-symmetric arithmetic (F = L L^T, principal square
   roots, no pivoting), which solves the same system to round-off for these
   matrices (a dominant positive definite real part), and the tests check it
   against SuperLU itself.
   The reference factors in the mesh's own node order; perm (optional,
   perm[new] = old) applies a symmetric reordering first, which changes the
   fill and the rounding but not the solution. */
typedef struct {
    int n;
    int *cptr, *crow;   /* strictly lower factor by columns, rows ascending */
    zd *cval, *d;
    int *perm;          /* perm[new] = old */
} tor_direct;

static int int_cmp(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* Reverse Cuthill-McKee: breadth-first from a low-degree node of each
   component, neighbours by ascending degree, the order reversed. */
void tor_rcm(int n, const int *rowptr, const int *colidx, int *perm)
{
    int *deg = malloc(sizeof(int) * (n ? n : 1)), *seen = calloc(n ? n : 1, sizeof(int));
    int *q = malloc(sizeof(int) * (n ? n : 1)), *nb = malloc(sizeof(int) * (n ? n : 1));
    for (int i = 0; i < n; i++) deg[i] = rowptr[i + 1] - rowptr[i];
    int head = 0, tail = 0;
    for (;;) {
        int s = -1;
        for (int i = 0; i < n; i++)
            if (!seen[i] && (s < 0 || deg[i] < deg[s])) s = i;
        if (s < 0) break;
        seen[s] = 1;
        q[tail++] = s;
        while (head < tail) {
            int v = q[head++], cnt = 0;
            for (int e = rowptr[v]; e < rowptr[v + 1]; e++) {
                int w = colidx[e];
                if (!seen[w]) { seen[w] = 1; nb[cnt++] = w; }
            }
            /* insertion sort by degree, then index */
            for (int a = 1; a < cnt; a++) {
                int w = nb[a], b = a - 1;
                while (b >= 0 && (deg[nb[b]] > deg[w] || (deg[nb[b]] == deg[w] && nb[b] > w))) { nb[b + 1] = nb[b]; b--; }
                nb[b + 1] = w;
            }
            for (int a = 0; a < cnt; a++) q[tail++] = nb[a];
        }
    }
    for (int i = 0; i < n; i++) perm[i] = q[n - 1 - i];
    free(deg); free(seen); free(q); free(nb);
}

/* Factor F (CSR, sorted columns) after the reordering perm (NULL: natural).
   Returns NULL on allocation failure. */
tor_direct *tor_direct_factor(int n, const int *rowptr, const int *colidx, const double *val, int cplx,
                              const int *perm)
{
    tor_direct *D = calloc(1, sizeof(tor_direct));
    D->n = n;
    D->perm = malloc(sizeof(int) * (n ? n : 1));
    int *iperm = malloc(sizeof(int) * (n ? n : 1));
    for (int i = 0; i < n; i++) D->perm[i] = perm ? perm[i] : i;
    for (int i = 0; i < n; i++) iperm[D->perm[i]] = i;
    /* the permuted lower pattern by columns: column j holds rows i > j */
    int *cnt = calloc((size_t)(n > 0 ? n : 0) + 1, sizeof(int));
    for (int i = 0; i < n; i++) {
        int oi = D->perm[i];
        for (int e = rowptr[oi]; e < rowptr[oi + 1]; e++) {
            int j = iperm[colidx[e]];
            if (j < i) cnt[j]++;
        }
    }
    int **col = malloc(sizeof(int *) * (size_t)(n > 0 ? n : 1));
    int *len = calloc(n ? n : 1, sizeof(int)), *cap = malloc(sizeof(int) * (n ? n : 1));
    for (int j = 0; j < n; j++) { cap[j] = cnt[j] + 4; col[j] = malloc(sizeof(int) * cap[j]); }
    for (int i = 0; i < n; i++) {
        int oi = D->perm[i];
        for (int e = rowptr[oi]; e < rowptr[oi + 1]; e++) {
            int j = iperm[colidx[e]];
            if (j < i) col[j][len[j]++] = i;
        }
    }
    /* symbolic factorisation: ascending columns, each sorted column's rows
       (minus its parent, the smallest) merged into the parent's */
    int *buf = NULL, bcap = 0;
    for (int j = 0; j < n; j++) {
        qsort(col[j], len[j], sizeof(int), int_cmp);
        if (len[j] == 0) continue;
        int p = col[j][0];
        int need = len[j] - 1 + len[p];
        if (need > bcap) { bcap = need * 2; buf = realloc(buf, sizeof(int) * bcap); }
        int a = 1, b = 0, m = 0;
        qsort(col[p], len[p], sizeof(int), int_cmp);
        while (a < len[j] && b < len[p]) {
            if (col[j][a] < col[p][b]) buf[m++] = col[j][a++];
            else if (col[j][a] > col[p][b]) buf[m++] = col[p][b++];
            else { buf[m++] = col[j][a++]; b++; }
        }
        while (a < len[j]) buf[m++] = col[j][a++];
        while (b < len[p]) buf[m++] = col[p][b++];
        if (m > cap[p]) { cap[p] = m; col[p] = realloc(col[p], sizeof(int) * m); }
        memcpy(col[p], buf, sizeof(int) * m);
        len[p] = m;
    }
    free(buf);
    D->cptr = malloc(sizeof(int) * (n + 1));
    D->cptr[0] = 0;
    for (int j = 0; j < n; j++) D->cptr[j + 1] = D->cptr[j] + len[j];
    size_t nl = (size_t)D->cptr[n];
    D->crow = malloc(sizeof(int) * (nl ? nl : 1));
    D->cval = calloc(nl ? nl : 1, sizeof(zd));
    D->d = malloc(sizeof(zd) * (n ? n : 1));
    for (int j = 0; j < n; j++) { memcpy(D->crow + D->cptr[j], col[j], sizeof(int) * len[j]); free(col[j]); }
    free(col); free(len); free(cap); free(cnt);
    /* row view of L (the columns cc < c with L(c, cc) != 0, ascending) */
    int *rptr = calloc(n + 1, sizeof(int)), *rcol = malloc(sizeof(int) * (nl ? nl : 1));
    for (size_t q = 0; q < nl; q++) rptr[D->crow[q] + 1]++;
    for (int i = 0; i < n; i++) rptr[i + 1] += rptr[i];
    int *fillp = malloc(sizeof(int) * (n ? n : 1));
    for (int i = 0; i < n; i++) fillp[i] = rptr[i];
    for (int j = 0; j < n; j++)
        for (int q = D->cptr[j]; q < D->cptr[j + 1]; q++) rcol[fillp[D->crow[q]]++] = j;
    /* numeric factorisation (CholeskyFactorize): column c gathers A(c:n, c),
       subtracts L(r, cc) L(c, cc) for every left column cc of row c, takes the
       pivot's square root (recover: 1e-10) and scales the column */
    zd *full = calloc(n ? n : 1, sizeof(zd));
    int *next = malloc(sizeof(int) * (n ? n : 1));  /* per column: first entry with row >= current c */
    for (int j = 0; j < n; j++) next[j] = D->cptr[j];
    const double EPS = 1e-10;
    for (int c = 0; c < n; c++) {
        int oc = D->perm[c];
        for (int e = rowptr[oc]; e < rowptr[oc + 1]; e++) {
            int r = iperm[colidx[e]];
            if (r >= c) full[r] = cplx ? val[2 * e] + I * val[2 * e + 1] : val[e];
        }
        for (int t = rptr[c]; t < rptr[c + 1]; t++) {
            int cc = rcol[t];
            int q = next[cc];  /* the entry (c, cc) */
            zd ajk = D->cval[q];
            for (; q < D->cptr[cc + 1]; q++) full[D->crow[q]] -= ajk * D->cval[q];
            next[cc]++;
        }
        zd piv = full[c];
        int ok = cplx ? cabs(piv) > 0.0 : creal(piv) > 0.0;
        D->d[c] = ok ? csqrt(piv) : EPS;
        zd idiag = 1.0 / D->d[c];
        full[c] = 0.0;
        for (int q = D->cptr[c]; q < D->cptr[c + 1]; q++) {
            int r = D->crow[q];
            D->cval[q] = full[r] * idiag;
            full[r] = 0.0;
        }
    }
    free(full); free(next); free(rptr); free(rcol); free(fillp); free(iperm);
    return D;
}

int tor_direct_nnz(const tor_direct *D) { return D->cptr[D->n]; }

void tor_direct_free(tor_direct *D)
{
    if (!D) return;
    free(D->cptr); free(D->crow); free(D->cval); free(D->d); free(D->perm);
    free(D);
}

/* CholeskySubst on nrhs right-hand sides (nrhs x n, complex interleaved when
   cplx): forward sweep over rows of L, backward sweep over its columns; host
   threads share the right-hand sides. */
typedef struct { const tor_direct *D; int cplx, q0, q1; const double *B; double *X; } dsolve_job;

static void *dsolve_worker(void *arg)
{
    dsolve_job *jb = arg;
    const tor_direct *D = jb->D;
    int n = D->n, cplx = jb->cplx;
    zd *y = malloc(sizeof(zd) * (size_t)(n > 0 ? n : 1));
    for (int q = jb->q0; q < jb->q1; q++) {
        const double *b = jb->B + (size_t)q * n * (cplx ? 2 : 1);
        for (int i = 0; i < n; i++) {
            int o = D->perm[i];
            y[i] = cplx ? b[2 * o] + I * b[2 * o + 1] : b[o];
        }
        /* forward: L y = b by columns (same sums as the row form) */
        for (int j = 0; j < n; j++) {
            y[j] /= D->d[j];
            for (int t = D->cptr[j]; t < D->cptr[j + 1]; t++) y[D->crow[t]] -= D->cval[t] * y[j];
        }
        /* backward: L^T x = y */
        for (int j = n - 1; j >= 0; j--) {
            zd s = y[j];
            for (int t = D->cptr[j + 1] - 1; t >= D->cptr[j]; t--) s -= D->cval[t] * y[D->crow[t]];
            y[j] = s / D->d[j];
        }
        double *x = jb->X + (size_t)q * n * (cplx ? 2 : 1);
        for (int i = 0; i < n; i++) {
            int o = D->perm[i];
            if (cplx) { x[2 * o] = creal(y[i]); x[2 * o + 1] = cimag(y[i]); }
            else x[o] = creal(y[i]);
        }
    }
    free(y);
    return NULL;
}

void tor_direct_solve(const tor_direct *D, int cplx, int nrhs, const double *B, double *X, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > nrhs) nthreads = nrhs > 0 ? nrhs : 1;
    dsolve_job *jobs = malloc(sizeof(dsolve_job) * nthreads);
    pthread_t *th = malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; t++) {
        dsolve_job jb = {D, cplx, (t * nrhs) / nthreads, ((t + 1) * nrhs) / nthreads, B, X};
        jobs[t] = jb;
        if (nthreads > 1) pthread_create(&th[t], NULL, dsolve_worker, &jobs[t]);
        else dsolve_worker(&jobs[t]);
    }
    if (nthreads > 1) for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(jobs); free(th);
}

/* Nested dissection by coordinates (an ordering for the direct factor that
   only reduces its fill): a node set is split at the median of its longest
   bounding-box axis, the nodes of the upper half adjacent to the lower half
   form the separator, and the order is lower half, upper half, separator,
   recursively down to sets of 64 nodes. */
static const double *nd_x;
static int nd_dim, nd_axis;
static int nd_cmp(const void *a, const void *b)
{
    double u = nd_x[(size_t)(*(const int *)a) * nd_dim + nd_axis], v = nd_x[(size_t)(*(const int *)b) * nd_dim + nd_axis];
    if (u != v) return (u > v) - (u < v);
    return (*(const int *)a > *(const int *)b) - (*(const int *)a < *(const int *)b);
}

static void nd_rec(const int *rowptr, const int *colidx, int *idx, int m, int *mark, int *stamp, int *out, int *pos,
                   int *tmp)
{
    if (m <= 64) {
        for (int i = 0; i < m; i++) out[(*pos)++] = idx[i];
        return;
    }
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < m; i++)
        for (int d = 0; d < nd_dim; d++) {
            double v = nd_x[(size_t)idx[i] * nd_dim + d];
            if (v < lo[d]) lo[d] = v;
            if (v > hi[d]) hi[d] = v;
        }
    nd_axis = 0;
    for (int d = 1; d < nd_dim; d++)
        if (hi[d] - lo[d] > hi[nd_axis] - lo[nd_axis]) nd_axis = d;
    qsort(idx, m, sizeof(int), nd_cmp);
    int half = m / 2;
    int lid = ++(*stamp);
    for (int i = 0; i < half; i++) mark[idx[i]] = lid;
    /* upper half: separator nodes (adjacent to the lower half) go last */
    int nu = 0, ns = 0;
    for (int i = half; i < m; i++) {
        int v = idx[i], sep = 0;
        for (int e = rowptr[v]; e < rowptr[v + 1]; e++)
            if (mark[colidx[e]] == lid) { sep = 1; break; }
        if (sep) tmp[ns++] = v;
        else idx[half + nu++] = v;
    }
    memcpy(idx + half + nu, tmp, sizeof(int) * ns);
    int *sepcopy = malloc(sizeof(int) * (ns ? ns : 1));
    memcpy(sepcopy, tmp, sizeof(int) * ns);
    nd_rec(rowptr, colidx, idx, half, mark, stamp, out, pos, tmp);
    nd_rec(rowptr, colidx, idx + half, nu, mark, stamp, out, pos, tmp);
    for (int i = 0; i < ns; i++) out[(*pos)++] = sepcopy[i];
    free(sepcopy);
}

void tor_nd_order(int n, const int *rowptr, const int *colidx, const double *coords, int dim, int *perm)
{
    int *idx = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1)), *mark = calloc((size_t)(n > 0 ? n : 1), sizeof(int));
    int *tmp = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) idx[i] = i;
    nd_x = coords;
    nd_dim = dim;
    int stamp = 0, pos = 0;
    nd_rec(rowptr, colidx, idx, n, mark, &stamp, perm, &pos, tmp);
    free(idx); free(mark); free(tmp);
}
