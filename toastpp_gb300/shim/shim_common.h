// shim_common.h -- what the two shim translation units share: the GPU mesh
// and solver of a QMMesh (built once per mesh, for the free functions of
// the reference's interface) and its link list.
#ifndef TOASTGPU_SHIM_COMMON_H
#define TOASTGPU_SHIM_COMMON_H

#include <vector>

#include "toastgpu.h"

class QMMesh;

namespace tgshim {
// xERROR with the library's message when rc is not TG_OK
void check(int rc, const char* what);
// the GPU mesh of a QMMesh (3-noded triangles or 4-noded tetrahedra)
tg_mesh make_mesh(const QMMesh* mesh);
// a GPU solver of the mesh (real or complex), built at first use and kept;
// *m (optional) receives the mesh handle
tg_solver mesh_solver(const QMMesh* mesh, bool cplx, tg_mesh* m);
// QMMesh's Qofs / QMref as offsets and detector indices (qmmesh.h:24-36)
void links_of(const QMMesh* mesh, std::vector<int>& ofs, std::vector<int>& lm);
}  // namespace tgshim

#endif
