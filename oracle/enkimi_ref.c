/* Reference decoder for the Minecraft import tests. TEST INFRASTRUCTURE:
 * oracle/build_ref.py compiles it with the reference's own region / NBT
 * reader (enkiMI and miniz, vendored in the reference's Dependencies/enkiMI)
 * into oracle/_ref/ when the reference sources are present. It drives that
 * reader the way Core/NBT/Importer.cpp ImportRegionFile (:111-166) does:
 * every chunk slot with data, every section with blocks, y-z-x order, a
 * voxel written only when its data value is 0, through the Minecraft-id
 * table, by WriteVoxel's placement (:91-108). */
#include <stdio.h>
#include <string.h>

#include "enkimi.h"

static void write_voxel(unsigned char* out, unsigned char voxel, int x, int y, int z, const int* origin) {
    x -= origin[0];
    y -= origin[1];
    z -= origin[2];
    x += 384 / 2;
    z += 384 / 2;
    if (y >= 128 || x >= 384 || z >= 384 || y < 0 || x < 0 || z < 0 || voxel == 0) return;
    out[(size_t)x + (size_t)y * 384 + (size_t)z * 384 * 128] = voxel;
}

/* Adds the voxels of one region file to out (384 x 128 x 384, x fastest);
 * returns the number of chunk slots with data, -1 if the file is missing. */
int ref_import_region(const char* path, const unsigned char* lut, const int* origin, unsigned char* out) {
    FILE* fp = fopen(path, "rb");
    if (!fp) return -1;
    enkiRegionFile rf = enkiRegionFileLoad(fp);
    int chunks = 0;
    for (int i = 0; i < ENKI_MI_REGION_CHUNKS_NUMBER; i++) {
        enkiNBTDataStream stream;
        enkiInitNBTDataStreamForChunk(rf, i, &stream);
        if (stream.dataLength) {
            enkiChunkBlockData chunk = enkiNBTReadChunk(&stream);
            chunks++;
            for (int section = 0; section < ENKI_MI_NUM_SECTIONS_PER_CHUNK; ++section) {
                if (!chunk.sections[section]) continue;
                enkiMICoordinate so = enkiGetChunkSectionOrigin(&chunk, section);
                enkiMICoordinate sp;
                for (sp.y = 0; sp.y < ENKI_MI_SIZE_SECTIONS; ++sp.y)
                    for (sp.z = 0; sp.z < ENKI_MI_SIZE_SECTIONS; ++sp.z)
                        for (sp.x = 0; sp.x < ENKI_MI_SIZE_SECTIONS; ++sp.x) {
                            enkiMIVoxelData v = enkiGetChunkSectionVoxelData(&chunk, section, sp);
                            if (v.dataValue == 0)
                                write_voxel(out, lut[v.blockID], so.x + sp.x, so.y + sp.y, so.z + sp.z, origin);
                        }
            }
            enkiNBTRewind(&stream);
        }
        enkiNBTFreeAllocations(&stream);
    }
    enkiRegionFileFreeAllocations(&rf);
    fclose(fp);
    return chunks;
}
