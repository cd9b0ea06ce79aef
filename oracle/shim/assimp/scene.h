// Oracle test infrastructure -- not part of the shipped library.
// Declaration-only stand-in for the assimp scene header (include/model.h:5).
#pragma once
#include "material.h"
struct aiVector3D { float x, y, z; };
struct aiFace { unsigned mNumIndices; unsigned* mIndices; };
struct aiMesh {
  unsigned mNumVertices = 0, mNumFaces = 0, mMaterialIndex = 0;
  aiVector3D* mVertices = nullptr;
  aiVector3D* mNormals = nullptr;
  aiVector3D* mTextureCoords[8] = {};
  aiFace* mFaces = nullptr;
};
struct aiNode {};
#define AI_SCENE_FLAGS_INCOMPLETE 0x1
struct aiScene {
  unsigned mFlags = 0, mNumMeshes = 0, mNumMaterials = 0;
  aiMesh** mMeshes = nullptr;
  aiMaterial** mMaterials = nullptr;
  aiNode* mRootNode = nullptr;
};
