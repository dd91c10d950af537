// batch.cuh -- recording the steps of many worlds into batched launches.
//
// Between alisgpu_batch_begin and alisgpu_batch_end, the half steps and
// phaser samples of the worlds a host thread steps are recorded instead
// of launched.  Consecutive records of one kind (E half steps, H half
// steps, phaser samples) of distinct worlds form a group, and a group
// runs as a few launches over all its worlds: one launch with a block per
// tile of every world's cells (the TFSF auxiliary columns and tiny worlds
// as one-block entries), then every world's source patches, then every
// world's ghost copies; or every phaser's ring flush, then every
// phaser's face gather.  A record of another kind, or a second record of
// a world already in the group, launches the group first, so the order
// of every world's own operations is that of the calls.
//
// A world's parameter structs change only when its objects, sources or
// boxes do: they live in device slots that are uploaded again only when
// their bytes differ.  What changes every step (source values, the
// phaser's ring slot) travels in one staging blob per group.
#pragma once
#include <vector>
#include "common.cuh"

// a device copy of a parameter struct, uploaded again when its bytes change
struct ParamSlot {
	void *dev = nullptr;
	std::vector<unsigned char> host;
};

enum { BATCH_NONE = 0, BATCH_E = 1, BATCH_H = 2, BATCH_PHASER = 3 };

// Is the calling thread recording?  With kind and world: join (or start)
// the group of that kind, launching the open group first when the kind
// differs or the world is in it already; returns 1 when the caller is to
// record instead of launching.
extern "C" int alisgpu__batch_enter(int kind, const void *world);
// the device address of src's bytes in slot s (uploaded when they changed)
extern "C" int alisgpu__slot_sync(ParamSlot *s, const void *src, size_t bytes, const void **dev);
extern "C" void alisgpu__slot_free(ParamSlot *s);
// staging of a group's tables: room for bytes, 256-byte aligned; returns
// the host address to fill and the device address it will have
extern "C" int alisgpu__blob_take(size_t bytes, void **host, const void **dev);
// upload the staged tables on the stream (before the group's launches)
extern "C" int alisgpu__blob_send(void);
// the group's launches are issued: the next group stages into another buffer
extern "C" int alisgpu__blob_done(void);
// launch the open group now (before work that is not recorded)
extern "C" int alisgpu__batch_flush(void);
// an entry point that reads or changes world data outside the recorded
// kinds launches the open group first
#define ALIS_BATCH_GUARD() do { int rc_ = alisgpu__batch_flush(); if (rc_) return rc_; } while (0)
// the phaser group: launch the recorded flushes and gathers (phaser.cu)
extern "C" int alisgpu__phaser_batch_launch(void);
extern "C" void alisgpu__phaser_batch_clear(void);
