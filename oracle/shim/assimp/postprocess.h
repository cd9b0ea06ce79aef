// Oracle test infrastructure -- not part of the shipped library.
// Declaration-only stand-in for the assimp post-process flags (include/model.h:6).
#pragma once
enum aiPostProcessSteps {
  aiProcess_Triangulate = 0x8, aiProcess_PreTransformVertices = 0x100,
  aiProcess_SortByPType = 0x8000, aiProcess_FixInfacingNormals = 0x2000
};
