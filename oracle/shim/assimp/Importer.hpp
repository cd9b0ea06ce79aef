// Oracle test infrastructure -- not part of the shipped library.
// Stand-in for the assimp importer (include/model.h:4): ReadFile loads
// nothing, so Model's file constructor reports an error and returns; the
// oracle harness fills Model's public members directly instead.
#pragma once
#include "scene.h"
#define AI_CONFIG_PP_PTV_KEEP_HIERARCHY "PP_PTV_KEEP_HIERARCHY"
namespace Assimp {
class Importer {
 public:
  void SetPropertyInteger(const char*, int) {}
  const aiScene* ReadFile(const char*, unsigned) { return nullptr; }
  const char* GetErrorString() const { return "asset import is not available in the oracle build"; }
  void FreeScene() {}
};
}  // namespace Assimp
