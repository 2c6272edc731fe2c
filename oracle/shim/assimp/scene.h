// Test-infrastructure shim: scene-graph types that the reference's
// lib/output.h prints. Only their field names matter; nothing is imported.
#pragma once

#include "camera.h"
#include "types.h"

struct aiFace {
    unsigned int mNumIndices = 0;
    unsigned int* mIndices = nullptr;
};

struct aiMesh {
    unsigned int mNumFaces = 0;
    aiFace* mFaces = nullptr;
    aiVector3D* mVertices = nullptr;
};

struct aiNode {
    aiString mName;
    unsigned int mNumChildren = 0;
    aiNode** mChildren = nullptr;
};
