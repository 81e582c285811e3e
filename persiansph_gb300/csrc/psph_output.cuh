// Snapshot output (the reference's WriteXDMF, Source/Domain.cpp:1869-2064):
// device gather, copy to pinned host memory on a side stream, files written
// by a host thread (psph_output.cu).
#pragma once

#include <stdint.h>

#include <string>

#include "psph_device.cuh"

namespace psph {

struct OutputWriter;
OutputWriter* output_writer_create();
// Waits for every queued snapshot, then frees the writer.
void output_writer_destroy(OutputWriter* w);
// Enqueues on stream st the gather of instance rows [lo, hi) of the current
// sorted state (x, v, density, pressure of the persistent buffer; the step's
// accelerations) into the writer's staging buffer.
bool output_gather(OutputWriter* w, const DevView& v, int lo, int hi, cudaStream_t st, std::string* err);
// Copies the last gather to pinned host memory on the writer's own stream and
// queues <key>.bin / <key>.xmf for the writer thread. props (3 x m host values
// in output order, or null for zeros) are the UserOutput properties.
bool output_commit(OutputWriter* w, const char* key, const char* const names[3], const double* props, int64_t m,
                   std::string* err);
// Waits until every queued snapshot is on disk; false (with the message) if a
// write failed.
bool output_flush(OutputWriter* w, std::string* err);

}  // namespace psph
