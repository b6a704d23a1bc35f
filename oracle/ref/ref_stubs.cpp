// Link stubs for compiling the reference's BVH/Ray/AABB/job-system sources into
// the checker library (oracle/_ref/libaeref.so).  TEST INFRASTRUCTURE ONLY.
//
// The compiled reference sources reference two engine facilities that the hot
// path does not need: the in-memory log (src/engine/Log.h:10-78) and the SDL
// performance counter constructed, and never read, in BVH::BVH
// (src/engine/volume/BVH.cpp:16).  Both are given empty bodies here.
#include "Log.h"
#include "tools/PerformanceCounter.h"

namespace Atlas {

    std::vector<Log::Entry> Log::entries;
    std::mutex Log::mutex;

    void Log::Message(const std::string&, int32_t) {}
    void Log::Warning(const std::string&, int32_t) {}
    void Log::Error(const std::string&, int32_t) {}

    namespace Tools {
        PerformanceCounter::PerformanceCounter() {}
    }

}
