// Declarations standing in for tinygltf, an un-vendored submodule of the reference, so that
// corelib/src/resource.cpp compiles for its Wavefront OBJ loader (wavefront_obj::load_geometry,
// resource.cpp:137-255). The glTF half of resource.cpp is never called by the oracle; every glTF
// load here fails. Found through the oracle's existing -I qt_stub as
// qt_stub/../thirdparty/tinygltf/tiny_gltf.h.
#pragma once

#include <cstddef>
#include <map>
#include <string>
#include <vector>

namespace tinygltf {

struct Buffer {
    std::vector<unsigned char> data;
};
struct BufferView {
    int buffer = -1;
    size_t byteOffset = 0;
};
struct Accessor {
    int bufferView = -1;
    size_t byteOffset = 0;
    size_t count = 0;
    int ByteStride(BufferView const &) const { return 0; }
};
struct Primitive {
    std::map<std::string, int> attributes;
    int indices = -1;
};
struct Mesh {
    std::string name;
    std::vector<Primitive> primitives;
};
struct PerspectiveCamera {
    double aspectRatio = 0, yfov = 0, zfar = 0, znear = 0;
};
struct Camera {
    std::string type, name;
    PerspectiveCamera perspective;
};
struct Parameter {
    std::vector<double> number_array;
};
struct Material {
    std::string name;
    std::map<std::string, Parameter> values;
};
struct Node {
    int camera = -1, mesh = -1;
    std::string name;
    std::vector<int> children;
    std::vector<double> matrix;
};
struct Scene {
    std::vector<int> nodes;
};
struct Model {
    std::vector<Accessor> accessors;
    std::vector<BufferView> bufferViews;
    std::vector<Buffer> buffers;
    std::vector<Camera> cameras;
    std::vector<Material> materials;
    std::vector<Mesh> meshes;
    std::vector<Node> nodes;
    std::vector<Scene> scenes;
};
class TinyGLTF {
  public:
    bool LoadASCIIFromFile(Model *, std::string *err, std::string *, std::string const &) { return refuse(err); }
    bool LoadBinaryFromFile(Model *, std::string *err, std::string *, std::string const &) { return refuse(err); }

  private:
    static bool refuse(std::string *err) {
        if (err)
            *err = "glTF loading is not part of the oracle build";
        return false;
    }
};

} // namespace tinygltf
