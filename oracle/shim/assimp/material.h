// Oracle test infrastructure -- not part of the shipped library.
// Declaration-only stand-in for the assimp material header that the
// reference includes (include/material.h:5). Scenes reach the compiled
// reference through the oracle harness, never through assimp, so only the
// names the reference mentions are declared; none of them does any work.
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
struct aiMaterial {
  aiReturn Get(const char*, unsigned, unsigned, aiString&) const { return AI_FAILURE; }
  aiReturn Get(const char*, unsigned, unsigned, ai_real&) const { return AI_FAILURE; }
  unsigned GetTextureCount(aiTextureType) const { return 0; }
  aiReturn GetTexture(aiTextureType, unsigned, aiString*) const { return AI_FAILURE; }
};
