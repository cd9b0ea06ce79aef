// Oracle test infrastructure -- not part of the shipped library.
// Stand-in for the assimp material header that the reference includes
// (include/material.h:5). Scenes reach the compiled reference through the
// oracle harness, never through assimp, so only the names the reference
// mentions are declared.
#pragma once
#include <string>
typedef float ai_real;
enum aiReturn { AI_SUCCESS = 0, AI_FAILURE = -1 };
enum aiTextureType {
  aiTextureType_NONE = 0, aiTextureType_DIFFUSE = 1, aiTextureType_SPECULAR = 2,
  aiTextureType_AMBIENT = 3, aiTextureType_EMISSIVE = 4, aiTextureType_HEIGHT = 5,
  aiTextureType_NORMALS = 6, aiTextureType_SHININESS = 7, aiTextureType_OPACITY = 8,
  aiTextureType_UNKNOWN = 9
};
#define AI_TEXTURE_TYPE_MAX 10
struct aiString {
  std::string s;
  const char* C_Str() const { return s.c_str(); }
};
#define AI_MATKEY_NAME "?mat.name", 0, 0
#define AI_MATKEY_OPACITY "$mat.opacity", 0, 0
// The oracle harness may set a name and an opacity, which Get then returns
// under AI_MATKEY_NAME / AI_MATKEY_OPACITY (to run the reference's
// Material::loadMaterialProperties); everything else reports no value.
struct aiMaterial {
  bool has_name = false, has_opacity = false;
  std::string name;
  ai_real opacity = 1.0f;
  aiReturn Get(const char* key, unsigned, unsigned, aiString& out) const {
    if (!has_name || std::string(key) != "?mat.name") return AI_FAILURE;
    out.s = name;
    return AI_SUCCESS;
  }
  aiReturn Get(const char* key, unsigned, unsigned, ai_real& out) const {
    if (!has_opacity || std::string(key) != "$mat.opacity") return AI_FAILURE;
    out = opacity;
    return AI_SUCCESS;
  }
  unsigned GetTextureCount(aiTextureType) const { return 0; }
  aiReturn GetTexture(aiTextureType, unsigned, aiString*) const { return AI_FAILURE; }
};
