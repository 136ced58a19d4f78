// Tuning table: the kernel variant of each (kernel group, dimension, degree, Gauss points) key,
// chosen by timing the variants on a problem (Context::autotune, autotune.cu) and kept for the whole
// process; saved to and loaded from a text file. Only variants that form the same sums in the same
// order are tuned, so a tuned context gives the same bits as an untuned one.
#pragma once

namespace gsgpu {

// 3D stiffness stage 1 (axis 0): interior rows in shared-memory tiles, or rows with 4 / 2 output
// fields per launch
enum : int { kStage31Tiles = 0, kStage31RowsNh4 = 1, kStage31RowsNh2 = 2 };
// 3D stiffness stage 2 (axis 1): rows with 4 / 2 output fields per launch
enum : int { kStage32RowsNh4 = 0, kStage32RowsNh2 = 1 };
// inner FP32 product of the mixed solve on the half-diagonal operator: load-based with one row per
// thread, TMA-fed, or load-based with four rows per thread and 16-byte loads
enum : int { kInnerSdiaLoads = 0, kInnerSdiaTma = 1, kInnerSdiaRows4 = 2 };

enum TuneKind : int { kTuneInner = 1, kTuneStage31 = 31, kTuneStage32 = 32 };
struct TuneKey {
    int kind, dim, p, q;
};

// the recorded variant of the key, or -1
int tuneLookup(const TuneKey& k);
// record (or replace) the key's variant and its measured time in milliseconds
void tuneRecord(const TuneKey& k, int variant, double ms);
// the table as text lines "kind dim p q variant ms"; false on an I/O or format error
bool tuneSave(const char* path);
bool tuneLoad(const char* path);
void tuneClear();

}  // namespace gsgpu
