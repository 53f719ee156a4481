/*
 * Arrow C Data Interface and C Device Data Interface structures.
 *
 * Written from the published Apache Arrow specifications ("The Arrow C data
 * interface" and "The Arrow C Device data interface"). The layouts are fixed by
 * those specifications, so these definitions are ABI-compatible with
 * arrow/c/abi.h; the include guards are the ones the specification asks for so
 * that a translation unit may include both headers.
 *
 * In the reference, operators exchange arrow::Table-backed TupleSets
 * (fpdb-tuple/include/fpdb/tuple/TupleSet.h:31-207). At the C-ABI boundary of
 * this library a TupleSet travels as one ArrowSchema of format "+s" (a struct
 * whose children are the columns) plus one ArrowDeviceArray whose struct array
 * holds one child per column: the standard C-interface form of a RecordBatch.
 */
#ifndef GFPDB_ARROW_H
#define GFPDB_ARROW_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef ARROW_C_DATA_INTERFACE
#define ARROW_C_DATA_INTERFACE

#define ARROW_FLAG_DICTIONARY_ORDERED 1
#define ARROW_FLAG_NULLABLE 2
#define ARROW_FLAG_MAP_KEYS_SORTED 4

struct ArrowSchema {
  const char* format;
  const char* name;
  const char* metadata;
  int64_t flags;
  int64_t n_children;
  struct ArrowSchema** children;
  struct ArrowSchema* dictionary;
  void (*release)(struct ArrowSchema*);
  void* private_data;
};

struct ArrowArray {
  int64_t length;
  int64_t null_count;
  int64_t offset;
  int64_t n_buffers;
  int64_t n_children;
  const void** buffers;
  struct ArrowArray** children;
  struct ArrowArray* dictionary;
  void (*release)(struct ArrowArray*);
  void* private_data;
};

#endif /* ARROW_C_DATA_INTERFACE */

#ifndef ARROW_C_DEVICE_DATA_INTERFACE
#define ARROW_C_DEVICE_DATA_INTERFACE

typedef int32_t ArrowDeviceType;

#define ARROW_DEVICE_CPU 1
#define ARROW_DEVICE_CUDA 2
#define ARROW_DEVICE_CUDA_HOST 3
#define ARROW_DEVICE_CUDA_MANAGED 13

struct ArrowDeviceArray {
  struct ArrowArray array;
  int64_t device_id;
  ArrowDeviceType device_type;
  void* sync_event;
  int64_t reserved[3];
};

#endif /* ARROW_C_DEVICE_DATA_INTERFACE */

#ifdef __cplusplus
}
#endif

#endif /* GFPDB_ARROW_H */
