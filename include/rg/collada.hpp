// collada.hpp -- scene ingest of the C++ facade: Collada (.dae) models and .rgmat.json materials.
//
// Replaces what Raygun does through assimp and its resource manager:
//   Entity(name, path, loadMaterials)   raygun/entity.cpp:86-122 (with loadMesh / collapseMeshes,
//                                       entity.cpp:32-80, and Mesh::merge, render/mesh.cpp:52-62)
//   Material(name, path)                raygun/material.cpp:59-108 (defaults: gpu_material.def)
//   ResourceManager::loadMaterial       raygun/resource_manager.cpp:60-64 (materials/<name>.rgmat.json)
//   utils::toTransform + Transform(mat4) raygun/utils/assimp_utils.hpp, raygun/transform.hpp:31-36
//
// The import semantics are those of assimp's Collada importer with aiProcess_Triangulate, restated:
//   * the children of the visual scene's root become the entity's children, in document order; each
//     child's transform is its node's <matrix> (or translate / rotate / scale sequence); the importer's
//     up-axis and unit corrections live on the root node, which the reference does not use;
//   * each <triangles> / <polylist> / <polygons> block of an instanced geometry is one mesh; its
//     vertices are the face corners in <p> order (no sharing), faces are (0,1,2), (3,4,5), ...;
//     polygons with more than three corners are split as a fan around their first corner;
//   * a child's model mesh is its node's meshes followed by those of its descendants, merged
//     (descendant transforms are not applied, as in collapseMeshes);
//   * materials are the file's <library_materials> in order of their ids (the importer keeps them
//     in a map keyed by id); a vertex's matIndex is its mesh's material's position in that list;
//     each material is loaded by its name attribute from <materialsDir>/<name>.rgmat.json, and a
//     missing file gives the default material, as the resource manager does.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "raygun.hpp"

namespace rg {

struct ColladaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// glm::decompose semantics for an affine matrix without shear: translation, per-axis scale (negative
// on all axes for a mirrored basis) and the rotation of the normalised basis
Transform transformFromMat4(const mat4& m);

// material.cpp:59-108: a Material from a .rgmat.json file ("basedOn" resolved in the same folder);
// throws ColladaError on unreadable or malformed files
std::shared_ptr<Material> loadMaterialFile(const std::string& path);

struct ColladaInfo {
    std::vector<std::string> materialIds;    // import order
    std::vector<std::string> materialNames;  // the names materials are loaded by
    std::string upAxis;                      // "Y_UP" / "Z_UP" / ...
};

// Entity(name, path, loadMaterials): materialsDir empty = loadMaterials false (models get no
// materials).  Throws ColladaError on files it cannot import.
std::shared_ptr<Entity> loadColladaEntity(const std::string& name, const std::string& daePath, const std::string& materialsDir,
                                          ColladaInfo* info = nullptr);

}  // namespace rg
