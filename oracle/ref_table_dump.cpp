// Test infrastructure (oracle side). Not part of the shipped library.
//
// Compiles the reference's own generated tessellation table header
// (src/tessellation_table_nv_raw.hpp of vk_tessellated_clusters, the file that
// src/tessellation_table.cpp:19-22 includes) and dumps its three arrays in the
// binary container format used by vk_tessellated_clusters_gb300/data/tess_table_nv.bin:
//
//   u32 magic 'TCTB' (0x42544354), u32 version (1), u32 max_edge_segments,
//   u32 num_vertices, u32 num_triangles, u32 num_configs,
//   u32 vertices[num_vertices], u32 triangles[num_triangles], u16 configs[4*num_configs]
//
// All values little endian. The binary is built by oracle/Makefile into
// oracle/_ref/ and is only used to pin the committed table blob.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include TC_REF_TABLE_HEADER

static void put_u32(FILE* f, uint32_t v)
{
  unsigned char b[4] = {(unsigned char)(v & 0xFF), (unsigned char)((v >> 8) & 0xFF), (unsigned char)((v >> 16) & 0xFF),
                        (unsigned char)((v >> 24) & 0xFF)};
  fwrite(b, 1, 4, f);
}

static void put_u16(FILE* f, uint16_t v)
{
  unsigned char b[2] = {(unsigned char)(v & 0xFF), (unsigned char)((v >> 8) & 0xFF)};
  fwrite(b, 1, 2, f);
}

int main(int argc, char** argv)
{
  if(argc != 2)
  {
    fprintf(stderr, "usage: %s <out.bin>\n", argv[0]);
    return 2;
  }
  FILE* f = fopen(argv[1], "wb");
  if(!f)
  {
    fprintf(stderr, "cannot open %s\n", argv[1]);
    return 1;
  }
  namespace tt = tessellation_table;
  const uint32_t nv = tt::max_vertices;
  const uint32_t nt = tt::max_triangles;
  const uint32_t nc = tt::max_configs;
  // the arrays are sized by their initialisers; cross-check against the declared counts
  if(sizeof(tt::vertices) / sizeof(tt::vertices[0]) != nv || sizeof(tt::triangles) / sizeof(tt::triangles[0]) != nt
     || sizeof(tt::configs) / sizeof(tt::configs[0]) != 4u * nc)
  {
    fprintf(stderr, "table array sizes disagree with declared counts\n");
    return 1;
  }
  put_u32(f, 0x42544354u);
  put_u32(f, 1u);
  put_u32(f, tt::max_edge_segments);
  put_u32(f, nv);
  put_u32(f, nt);
  put_u32(f, nc);
  for(uint32_t i = 0; i < nv; i++)
    put_u32(f, tt::vertices[i]);
  for(uint32_t i = 0; i < nt; i++)
    put_u32(f, tt::triangles[i]);
  for(uint32_t i = 0; i < 4u * nc; i++)
    put_u16(f, tt::configs[i]);
  fclose(f);
  printf("max_edge_segments=%u vertices=%u triangles=%u configs=%u\n", tt::max_edge_segments, nv, nt, nc);
  return 0;
}
