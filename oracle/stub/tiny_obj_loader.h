// Link stub for the un-vendored tinyobj dependency of the Jet reference.
//
// Only TriangleMesh3::readObj (src/jet/triangle_mesh3.cpp) includes this
// header. The pressure-projection path never loads OBJ files, so the stub
// declares just the types that file names and a LoadObj that always fails.
// It exists so the reference library links for the oracle build; it is test
// infrastructure, not part of the product.
#ifndef ORACLE_STUB_TINY_OBJ_LOADER_H_
#define ORACLE_STUB_TINY_OBJ_LOADER_H_

#include <istream>
#include <string>
#include <vector>

namespace tinyobj {

typedef float real_t;

struct index_t {
    int vertex_index = -1;
    int normal_index = -1;
    int texcoord_index = -1;
};

struct mesh_t {
    std::vector<index_t> indices;
    std::vector<unsigned char> num_face_vertices;
};

struct shape_t {
    std::string name;
    mesh_t mesh;
};

struct material_t {
    std::string name;
};

struct attrib_t {
    std::vector<real_t> vertices;
    std::vector<real_t> normals;
    std::vector<real_t> texcoords;
};

inline bool LoadObj(attrib_t*, std::vector<shape_t>*, std::vector<material_t>*,
                    std::string* err, std::istream*) {
    if (err) err->clear();
    return false;
}

}  // namespace tinyobj

#endif  // ORACLE_STUB_TINY_OBJ_LOADER_H_
