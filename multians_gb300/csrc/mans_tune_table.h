// Measured planner table, written by multians_gb300/tune.py from decodes
// timed on GB300; read by mans_plan (mans_decode.cu).  Do not edit by hand:
// run the tool again.
//   command: python -m multians_gb300.tune --sizes 16,256 --L 1024,2048,4096,8192 --lam 0.005,0.05,0.2,1.0,2.0
//   measured: 2026-12-04 17:00 UTC, 40 entries
// Each entry: the stream it was measured on (L, bits per symbol, size
// class: 1 = 256 MiB of symbols, 0 = 16 MiB) and the fastest plan found
// (units per block, shortest region in mean merge distances, capture), with
// its decoded GB/s and the model's plan's on the same stream.
#pragma once

#include <cstdint>

namespace mans {

struct TuneEntry {
    uint32_t L;            // table size the entry was measured at
    float bps;             // bits per symbol of the swept stream
    uint32_t large;        // 1: measured on 256 MiB of symbols, 0: on 16 MiB
    uint32_t block_units;  // units per block
    float meet_mult;       // shortest region, in mean meeting distances
    uint32_t capture;      // symbol capture on
    float gbps;            // decoded GB/s of this choice in the sweep
    float model_gbps;      // decoded GB/s of the model's own plan there
};

constexpr TuneEntry kTuneTable[] = {
    {1024, 0.672f, 0, 8, 2.0f, 0, 29.4f, 24.6f},
    {1024, 1.523f, 0, 16, 4.0f, 0, 15.0f, 13.3f},
    {1024, 3.838f, 0, 16, 3.0f, 0, 23.2f, 20.2f},
    {1024, 6.002f, 0, 16, 3.0f, 1, 52.5f, 52.3f},
    {1024, 8.570f, 0, 16, 1.5f, 0, 97.7f, 95.0f},
    {2048, 0.670f, 0, 8, 3.0f, 0, 17.8f, 10.6f},
    {2048, 1.520f, 0, 16, 1.5f, 0, 9.5f, 8.0f},
    {2048, 3.830f, 0, 16, 3.0f, 0, 14.8f, 12.8f},
    {2048, 5.956f, 0, 16, 2.0f, 0, 32.4f, 26.1f},
    {2048, 8.660f, 0, 16, 4.0f, 0, 80.0f, 76.8f},
    {4096, 0.669f, 0, 8, 2.0f, 0, 10.4f, 9.2f},
    {4096, 1.518f, 0, 16, 1.5f, 0, 5.5f, 4.2f},
    {4096, 3.830f, 0, 16, 3.0f, 0, 7.2f, 7.0f},
    {4096, 5.960f, 0, 16, 2.0f, 0, 18.9f, 18.9f},
    {4096, 8.639f, 0, 16, 1.5f, 0, 52.5f, 52.4f},
    {8192, 0.668f, 0, 8, 2.0f, 0, 6.4f, 5.5f},
    {8192, 1.518f, 0, 8, 1.5f, 0, 2.2f, 1.4f},
    {8192, 3.831f, 0, 8, 2.0f, 0, 4.2f, 3.9f},
    {8192, 5.958f, 0, 16, 1.5f, 0, 10.8f, 8.9f},
    {8192, 8.633f, 0, 16, 2.0f, 0, 33.6f, 30.7f},
    {1024, 0.672f, 1, 4, 3.0f, 0, 266.4f, 264.5f},
    {1024, 1.526f, 1, 16, 3.0f, 0, 150.1f, 126.7f},
    {1024, 3.858f, 1, 16, 4.0f, 1, 244.5f, 195.5f},
    {1024, 6.001f, 1, 16, 1.5f, 1, 374.5f, 373.6f},
    {1024, 8.570f, 1, 16, 1.5f, 1, 436.5f, 433.4f},
    {2048, 0.669f, 1, 8, 3.0f, 0, 185.1f, 160.0f},
    {2048, 1.523f, 1, 16, 2.0f, 0, 103.1f, 78.7f},
    {2048, 3.844f, 1, 16, 3.0f, 1, 147.3f, 136.5f},
    {2048, 5.956f, 1, 16, 1.5f, 1, 278.0f, 280.8f},
    {2048, 8.659f, 1, 16, 1.5f, 1, 386.6f, 385.5f},
    {4096, 0.668f, 1, 8, 2.0f, 0, 117.4f, 102.1f},
    {4096, 1.522f, 1, 16, 4.0f, 0, 54.7f, 46.2f},
    {4096, 3.846f, 1, 16, 3.0f, 1, 93.8f, 77.1f},
    {4096, 5.961f, 1, 16, 4.0f, 1, 193.2f, 185.9f},
    {4096, 8.639f, 1, 16, 1.5f, 1, 296.7f, 293.8f},
    {8192, 0.668f, 1, 4, 2.0f, 0, 58.4f, 49.9f},
    {8192, 1.521f, 1, 8, 2.0f, 0, 30.8f, 28.8f},
    {8192, 3.847f, 1, 16, 2.0f, 0, 52.1f, 40.2f},
    {8192, 5.960f, 1, 16, 3.0f, 0, 104.9f, 101.6f},
    {8192, 8.633f, 1, 16, 1.5f, 0, 178.8f, 176.1f},
};
constexpr uint32_t kTuneCount = sizeof(kTuneTable) / sizeof(kTuneTable[0]);

}  // namespace mans
