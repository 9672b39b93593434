/* c_caller.c -- a plain C99 caller of the library's C ABI (test support).
 *
 * Records the default dispatch schedule of an image with the reference's
 * entry point (nvproCmdPyramidDispatch) into a record-only command -- no
 * device memory is touched, so it runs without a GPU -- and prints one line
 * per recorded dispatch: isFast pushConstant groupsX isBlit configBits.
 * Also exercises the packed layout helpers and pipeline creation errors.
 * Usage: c_caller WIDTH HEIGHT [fastConfigBits generalConfigBits blit] */
#include <stdio.h>
#include <stdlib.h>

#include "nvpro_pyramid_cuda.h"

static int check(NvproPyramidResult r, const char* what) {
  if (r != NVPRO_PYRAMID_SUCCESS) {
    fprintf(stderr, "%s: %s (%s)\n", what, nvproPyramidResultString(r), nvproPyramidLastError());
    return 1;
  }
  return 0;
}

int main(int argc, char** argv) {
  uint32_t w, h, fastBits = 0, generalBits = 0, blit = 0, levels, i, n;
  uint64_t offsets[NVPRO_PYRAMID_MAX_LEVELS + 1];
  NvproPyramidPipeline fast = NULL, general = NULL, bad = NULL;
  NvproPyramidPipelines pipes;
  NvproPyramidCmd cmd = NULL;
  NvproPyramidImage image;
  NvproPyramidDispatchRecord records[64];
  if (argc < 3) return 2;
  w = (uint32_t)strtoul(argv[1], NULL, 10);
  h = (uint32_t)strtoul(argv[2], NULL, 10);
  if (argc >= 6) {
    fastBits = (uint32_t)strtoul(argv[3], NULL, 10);
    generalBits = (uint32_t)strtoul(argv[4], NULL, 10);
    blit = (uint32_t)strtoul(argv[5], NULL, 10);
  }
  levels = nvproPyramidFullLevelCount(w, h);
  if (check(nvproPyramidPackedLayout(w, h, levels, 4, offsets), "layout")) return 1;
  /* fake, aligned, never dereferenced level addresses */
  if (check(nvproPyramidImageInitPacked(&image, (void*)(uintptr_t)0x7F0000000000ull, w, h, levels, 4), "image"))
    return 1;
  if (nvproPyramidCreatePipelineEx(NVPRO_PYRAMID_PRESET_RGBA32F, 1, NVPRO_PYRAMID_CONFIG_SRGB_SHARED, &bad) !=
          NVPRO_PYRAMID_ERROR_UNSUPPORTED ||
      bad != NULL)
    return 3;
  if (check(nvproPyramidCreatePipelineEx(NVPRO_PYRAMID_PRESET_SRGBA8, 1, fastBits, &fast), "fast pipeline") ||
      check(nvproPyramidCreatePipelineEx(NVPRO_PYRAMID_PRESET_SRGBA8, 0, generalBits, &general), "general pipeline") ||
      check(nvproPyramidCreateCmd(NVPRO_PYRAMID_CMD_RECORD_ONLY, &cmd), "command"))
    return 1;
  pipes.generalPipeline = general;
  pipes.fastPipeline = fast;
  pipes.layout = NULL;
  pipes.pushConstantOffset = 0;
  if (check(nvproPyramidBeginCmd(cmd, NULL), "begin") || check(nvproPyramidCmdBindImage(cmd, &image), "bind"))
    return 1;
  if (blit) {
    if (check(nvproCmdPyramidDispatchEx(cmd, pipes, w, h, 0, nvproPyramidBlitGeneralDispatcher,
                                        nvproPyramidDefaultFastDispatcher),
              "dispatch"))
      return 1;
  } else if (check(nvproCmdPyramidDispatch(cmd, pipes, w, h, 0), "dispatch")) {
    return 1;
  }
  if (check(nvproPyramidEndCmd(cmd), "end")) return 1;
  n = nvproPyramidCmdRecordCount(cmd);
  if (n > 64 || check(nvproPyramidCmdGetRecords(cmd, records, n), "records")) return 1;
  printf("levels %u bytes %llu\n", levels, (unsigned long long)offsets[levels]);
  for (i = 0; i < n; ++i)
    printf("%u %u %u %u %u\n", records[i].isFastPipeline, records[i].pushConstant, records[i].groupCountX,
           records[i].isBlit, records[i].configBits);
  nvproPyramidDestroyCmd(cmd);
  nvproPyramidDestroyPipeline(fast);
  nvproPyramidDestroyPipeline(general);
  return 0;
}
