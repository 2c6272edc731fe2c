// Test-infrastructure shim: the aiCamera fields the reference's Camera class
// reads (lib/types.h:92-105). Defaults follow the assimp convention for a
// camera in its node's local space: at the origin, up +y, looking down -z.
#pragma once

#include "types.h"

struct aiCamera {
    aiString mName;
    aiVector3D mPosition{0, 0, 0};
    aiVector3D mUp{0, 1, 0};
    aiVector3D mLookAt{0, 0, -1};
    float mHorizontalFOV = 0.25f * 3.14159265358979f;
    float mClipPlaneNear = 0.1f;
    float mClipPlaneFar = 1000.f;
    float mAspect = 0.f;
};
