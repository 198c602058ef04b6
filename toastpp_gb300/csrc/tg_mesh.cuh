// tg_mesh.cuh -- per-mesh structure: element geometry, CSR pattern, IC(0)
// pattern and level schedule, assembly gather map, node->element map.
// Built once per mesh on the host (the equivalent of Mesh::Setup), uploaded
// once; every per-request step runs on the GPU.
#pragma once
#include <vector>
#include "tg_common.cuh"

namespace tg {

// Per-element record, 32 doubles (256 B):
//  [0]      size (signed, as the reference)
//  [1..9]   intdd (Tri3) or IntFDD(0,i,j) (Tet4) -- 3x3 or first 9 of 4x4? see below
// Layout used:
//  Tri3: [0] size, [1..9] intdd 3x3, [10..18] intbff 3x3
//  Tet4: [0] size, [1..16] IntFDD(0,i,j) 4x4, [17..20] side areas, [21] bnd side mask,
//        [22..31] unused
constexpr int EL_REC = 32;

// IC(0) pattern for one elimination ordering, in layout positions.  key[p] =
// rank of layout row p in the ordering; L row p = its neighbours of smaller
// rank in ascending rank (the factorisation's merge order), U = column view,
// levels = depth in the dependency graph (rows of a level in layout order),
// ELL copies of each level's entries for the sweep kernels.
struct ICHost {
    std::vector<int> key, Lrowptr, Lcolidx, Lapos, Lkey, Ucolptr, Urow, Umap;
    std::vector<int> fwd_lev_ptr, fwd_lev_rows, bwd_lev_ptr, bwd_lev_rows;
    std::vector<int> fwd_ell_w, fwd_ell_off, fwd_ell_col, fwd_ell_src;
    std::vector<int> bwd_ell_w, bwd_ell_off, bwd_ell_col, bwd_ell_src;
};

struct ICDev {
    int nnzL, nlev_fwd, nlev_bwd, nell_fwd, nell_bwd;
    int *key, *Lrowptr, *Lcolidx, *Lapos, *Lkey, *Ucolptr, *Urow, *Umap;
    int *fwd_lev_rows, *bwd_lev_rows;
    int *fwd_ell_col, *fwd_ell_src, *bwd_ell_col, *bwd_ell_src;
    // per level: first row (nlev + 1 entries), ELL width and ELL offset, for
    // the persistent sweep kernel
    int *fwd_lev_ptr, *bwd_lev_ptr, *fwd_ell_w, *bwd_ell_w, *fwd_ell_off, *bwd_ell_off;
};

struct MeshHost {
    int dim = 0, n = 0, ne = 0, nn = 0;
    std::vector<double> coords;       // n*dim
    std::vector<int> el;              // ne*nn
    std::vector<double> geo;          // ne*16 geometry coefficients a,b,c(,d)
    std::vector<double> rec;          // ne*EL_REC element record
    std::vector<unsigned char> bndside, bndnode;
    std::vector<double> intbff;       // ne*nn*nn (source vectors)
    // CSR pattern of F in the natural (reference) numbering; the host API reports it
    std::vector<int> rowptr, colidx, diagpos;
    // device layout: nodes stored in a spatially coherent (Morton) order.
    // perm[natural] = layout position, iperm[layout] = natural node.  Layout
    // rows keep their entries in natural column order, so every row sum is
    // the reference's; lay2nat[e] = natural CSR entry of layout entry e.
    std::vector<int> perm, iperm, lrowptr, lcolidx, ldiagpos, lay2nat, Lkey, jcolidx;
    // per ROW_TILE-row layout tile: the distinct columns its rows reference
    // (ascending), and for every layout entry the column's index in that list
    std::vector<int> halo_ptr, halo_col;
    std::vector<unsigned short> lcol;
    int halo_max = 0;
    // IC(0) structures: [0] the natural (reference) ordering, [1] a colour-major
    // ordering (greedy colouring, colour classes are independent sets) used by
    // the FP32 inner preconditioner of the mixed path
    ICHost ic[2];
    int ncolors = 0;
    // assembly gather map: for F entry k, contributions (el*16 + i*4 + j) in element order
    std::vector<int> asm_ptr, asm_list;
    // node -> (element*4 + local index), element order
    std::vector<int> nel_ptr, nel_list;
    std::vector<unsigned> nel_pos;
};

struct MeshDev {
    int dim, n, ne, nn, nnz;
    double* rec;
    int* el;                   // element nodes, natural numbering
    int *rowptr, *colidx, *diagpos;   // layout CSR (rows and columns in layout positions)
    int *perm, *iperm;         // natural -> layout, layout -> natural
    int *jrowptr, *jcolidx;    // natural-row CSR with layout column ids (Jacobian tiles over natural nodes)
    int *halo_ptr, *halo_col;  // distinct columns per ROW_TILE-row layout tile
    unsigned short* lcol;      // per layout entry: index of its column in the tile's halo
    int halo_max;
    unsigned *nel_pos;         // per node-element slot: positions of the element nodes in the node's CSR row (4 x uint8)
    int *asm_ptr, *asm_list;
    int *nel_ptr, *nel_list;
    unsigned char* bndnode;
    double* intbff;            // ne*nn*nn boundary integrals BndIntFF (element basis, source vectors)
    ICDev ic[2];
};

struct Mesh {
    MeshHost h;
    MeshDev d{};
    int device = 0;
    long long uid = 0;  // unique per mesh built in this process
    ~Mesh();
};

Mesh* mesh_build(int dim, int n, const double* coords, int ne, const int* el);
// The complete Cholesky pattern of F for the direct solver: a nested-
// dissection ordering of the nodes by their coordinates and the symbolic
// factor (fill included, Lapos -1 where A has no entry), with the column
// view, levels and ELL layouts of ICHost.  Throws TG_ERR_UNSUPPORTED past
// max_nnz factor entries.
void direct_pattern(const MeshHost& m, ICHost& c, long long max_nnz);
void qvec_gaussian_host(const MeshHost& m, const double* cnt, double w, bool neumann, double* q);
// Element_Unstructured::GContains for element e (padded bounding box, then
// the padded local test)
bool el_gcontains(const MeshHost& m, int e, const double* p);
// QMMesh::InitM's placement of a detector read from a QM file (fixed: kept,
// or nudged into an element; else pulled to the boundary); false if a fixed
// position lies in no element
bool qm_place_detector(const MeshHost& m, bool fixed, double* p);
// QMMesh::LoadQM's "external" source position: the boundary point that
// Mesh::BndIntersect finds from q + |q| n towards q, n the unit normal read
// with the position (nrm) or the unit vector along -q (nrm NULL).  Returns
// 0, 2 for a zero normal, 1 when no boundary point is found.
int qm_external_source(const MeshHost& m, const double* q, const double* nrm, double* out);

}  // namespace tg
