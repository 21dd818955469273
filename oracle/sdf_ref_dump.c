/*
 * sdf_ref_dump.c -- TEST INFRASTRUCTURE: reads an SDF file with the
 * reference's own SDF C library (SDF/C/src, built by oracle/sdf_ref.py into
 * oracle/_ref/) and prints its header and every block, so that the tests can
 * check this package's dumps against the reader the reference ships.
 *
 * Output, one record per line:
 *   HEADER <step> <time> <nblocks> <restart_flag> <code_name>
 *   BLOCK <id>\t<name>\t<blocktype>\t<datatype>\t<ndims>\t<d0,d1,..>\t<stagger>\t<mesh_id>\t<units>
 *   CONST <value>                       (constant blocks, real8)
 *   DATA <n> v0 v1 ...                  (plain and point variables)
 *   GRID <k> <n> v0 v1 ...              (mesh axis k of plain and point meshes)
 * Reals are printed with %.17g (exact round trip), integer8 as integers.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#include <sdf.h>

static const char* s(const char* p) { return p ? p : ""; }

static void print_array(const void* data, int64_t n, int datatype) {
  if (datatype == SDF_DATATYPE_REAL8) {
    const double* d = (const double*)data;
    for (int64_t i = 0; i < n; ++i) printf(" %.17g", d[i]);
  } else if (datatype == SDF_DATATYPE_INTEGER8) {
    const int64_t* d = (const int64_t*)data;
    for (int64_t i = 0; i < n; ++i) printf(" %lld", (long long)d[i]);
  } else if (datatype == SDF_DATATYPE_REAL4) {
    const float* d = (const float*)data;
    for (int64_t i = 0; i < n; ++i) printf(" %.9g", (double)d[i]);
  } else if (datatype == SDF_DATATYPE_INTEGER4) {
    const int32_t* d = (const int32_t*)data;
    for (int64_t i = 0; i < n; ++i) printf(" %d", d[i]);
  }
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: sdf_ref_dump <file.sdf>\n");
    return 2;
  }
  sdf_file_t* h = sdf_open(argv[1], 0, SDF_READ, 0);
  if (!h) {
    fprintf(stderr, "cannot open %s\n", argv[1]);
    return 1;
  }
  if (sdf_read_blocklist(h) != 0) {
    fprintf(stderr, "cannot read the block list of %s\n", argv[1]);
    sdf_close(h);
    return 1;
  }
  printf("HEADER %d %.17g %d %d %s\n", h->step, h->time, h->nblocks, (int)h->restart_flag, s(h->code_name));
  for (sdf_block_t* b = h->blocklist; b; b = b->next) {
    printf("BLOCK %s\t%s\t%d\t%d\t%d\t", s(b->id), s(b->name), b->blocktype, b->datatype, b->ndims);
    for (int k = 0; k < b->ndims; ++k) printf(k ? ",%lld" : "%lld", (long long)b->dims[k]);
    printf("\t%d\t%s\t%s\n", b->stagger, s(b->mesh_id), s(b->units));
    h->current_block = b;
    if (b->blocktype == SDF_BLOCKTYPE_CONSTANT) {
      double v = 0.0;
      if (b->datatype == SDF_DATATYPE_REAL8) memcpy(&v, b->const_value, sizeof(v));
      printf("CONST %.17g\n", v);
      continue;
    }
    if (sdf_read_data(h) != 0) {
      printf("READ_ERROR\n");
      continue;
    }
    if (b->blocktype == SDF_BLOCKTYPE_PLAIN_VARIABLE || b->blocktype == SDF_BLOCKTYPE_POINT_VARIABLE) {
      printf("DATA %lld", (long long)b->nelements_local);
      print_array(b->data, b->nelements_local, b->datatype);
      printf("\n");
    } else if (b->blocktype == SDF_BLOCKTYPE_PLAIN_MESH || b->blocktype == SDF_BLOCKTYPE_POINT_MESH) {
      for (int k = 0; k < b->ndims && b->grids; ++k) {
        const int64_t n = b->blocktype == SDF_BLOCKTYPE_PLAIN_MESH ? b->local_dims[k] : b->nelements_local;
        printf("GRID %d %lld", k, (long long)n);
        print_array(b->grids[k], n, b->datatype);
        printf("\n");
      }
    }
  }
  sdf_close(h);
  return 0;
}
