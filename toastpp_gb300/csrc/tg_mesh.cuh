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

struct MeshHost {
    int dim = 0, n = 0, ne = 0, nn = 0;
    std::vector<double> coords;       // n*dim
    std::vector<int> el;              // ne*nn
    std::vector<double> geo;          // ne*16 geometry coefficients a,b,c(,d)
    std::vector<double> rec;          // ne*EL_REC element record
    std::vector<unsigned char> bndside, bndnode;
    std::vector<double> intbff;       // ne*nn*nn (source vectors)
    // CSR pattern of F
    std::vector<int> rowptr, colidx, diagpos;
    // IC(0): strict lower pattern L (rows), its column view U (for the back
    // sweep and the factorisation), A positions of each L/U entry
    std::vector<int> Lrowptr, Lcolidx, Lapos;       // Lapos: index of a_ij in F for L(i,j)
    std::vector<int> Ucolptr, Urow, Umap;           // column i of L: rows r>i, index into L
    std::vector<int> fwd_lev_ptr, fwd_lev_rows, bwd_lev_ptr, bwd_lev_rows;
    // assembly gather map: for F entry k, contributions (el*16 + i*4 + j) in element order
    std::vector<int> asm_ptr, asm_list;
    // node -> (element*4 + local index), element order
    std::vector<int> nel_ptr, nel_list;
};

struct MeshDev {
    int dim, n, ne, nn, nnz, nnzL, nlev_fwd, nlev_bwd;
    double* rec;
    int* el;
    int *rowptr, *colidx, *diagpos;
    int *Lrowptr, *Lcolidx, *Lapos;
    int *Ucolptr, *Urow, *Umap;
    int *fwd_lev_rows, *bwd_lev_rows;
    int *asm_ptr, *asm_list;
    int *nel_ptr, *nel_list;
    unsigned char* bndnode;
};

struct Mesh {
    MeshHost h;
    MeshDev d{};
    std::vector<int> fwd_lev_ptr_h, bwd_lev_ptr_h;
    int device = 0;
    ~Mesh();
};

Mesh* mesh_build(int dim, int n, const double* coords, int ne, const int* el);
void qvec_gaussian_host(const MeshHost& m, const double* cnt, double w, bool neumann, double* q);

}  // namespace tg
