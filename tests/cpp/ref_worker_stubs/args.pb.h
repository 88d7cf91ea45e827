// Stand-in for the protobuf-generated args.pb.h that the reference's
// gpuWorker.cpp includes but does not use (the PS messages are handled by
// streamWorker). TEST INFRASTRUCTURE ONLY.
#pragma once
