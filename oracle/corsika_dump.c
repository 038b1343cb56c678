/*
 * corsika_dump.c -- TEST INFRASTRUCTURE ONLY.  A small driver over the
 * reference's own eventio reader (src/bernlohr/{eventio,io_simtel,
 * fileopen,straux,warning}.c, compiled from where they lie by
 * oracle/build_ref.sh into oracle/_ref/corsika_dump).  It walks a CORSIKA
 * IACT file the way ACorsikaIACTFile::Open / ReadEvent do
 * (src/ACorsikaIACTFile.cxx:191-489) and prints, as text, everything the
 * GPU framework's own reader must reproduce: the run header, the input
 * card line count, the telescope positions, and per event the event
 * header, the array offsets and every photon bunch (telescope, array, x,
 * y, cx, cy, ctime, zem, photons, lambda).  Floats are printed with 9
 * significant digits, which round-trips float32 exactly.
 * tests/golden/make_fixtures.py turns the output into a golden fixture.
 */
#include <stdio.h>
#include <stdlib.h>

#include "initial.h"
#include "io_basic.h"
#include "mc_tel.h"
#include "fileopen.h"

#define MAX_TEL 1000
#define MAX_ARRAY 100
#define MAX_BUNCH 2000000

static void print_block(const char* tag, const float* v, int n) {
  int i;
  printf("%s %d", tag, n);
  for (i = 0; i < n; ++i) printf(" %.9g", v[i]);
  printf("\n");
}

int main(int argc, char** argv) {
  IO_BUFFER* iobuf;
  IO_ITEM_HEADER block;
  static double tx[MAX_TEL], ty[MAX_TEL], tz[MAX_TEL], tr[MAX_TEL];
  static struct bunch bunches[MAX_BUNCH];
  int ntel = 0;
  if (argc < 2) {
    fprintf(stderr, "usage: corsika_dump FILE\n");
    return 2;
  }
  iobuf = allocate_io_buffer(1000000);
  if (!iobuf) return 1;
  iobuf->max_length = 200000000;
  if ((iobuf->input_file = fileopen(argv[1], "r")) == NULL) {
    fprintf(stderr, "cannot open %s\n", argv[1]);
    return 1;
  }
  while (find_io_block(iobuf, &block) == 0) {
    if (read_io_block(iobuf, &block) != 0) break;
    switch (block.type) {
      case IO_TYPE_MC_RUNH:
      case IO_TYPE_MC_EVTH: {
        float h[273];
        if (read_tel_block(iobuf, block.type, h, 273) < 0) return 1;
        print_block(block.type == IO_TYPE_MC_RUNH ? "RUNH" : "EVTH", h, 273);
        break;
      }
      case IO_TYPE_MC_INPUTCFG: {
        struct linked_string lines = {NULL, NULL};
        const struct linked_string* xl;
        int n = 0;
        read_input_lines(iobuf, &lines);
        for (xl = &lines; xl != NULL && xl->text != NULL; xl = xl->next) ++n;
        printf("INPUT %d\n", n);
        break;
      }
      case IO_TYPE_MC_TELPOS: {
        int i;
        if (read_tel_pos(iobuf, MAX_TEL, &ntel, tx, ty, tz, tr) < 0) return 1;
        printf("TELPOS %d\n", ntel);
        for (i = 0; i < ntel; ++i) printf("TEL %.9g %.9g %.9g %.9g\n", tx[i], ty[i], tz[i], tr[i]);
        break;
      }
      case IO_TYPE_MC_TELOFF: {
        int narray = 0, i;
        double toff, xo[MAX_ARRAY], yo[MAX_ARRAY];
        if (read_tel_offset(iobuf, MAX_ARRAY, &narray, &toff, xo, yo) < 0) return 1;
        printf("TELOFF %d %.9g\n", narray, toff);
        for (i = 0; i < narray; ++i) printf("OFF %.9g %.9g\n", xo[i], yo[i]);
        break;
      }
      case IO_TYPE_MC_TELARRAY: {
        IO_ITEM_HEADER ih, sub;
        int array = 0, t;
        begin_read_tel_array(iobuf, &ih, &array);
        for (t = 0; t < ntel; ++t) {
          int arr, tel, nb = 0, j;
          double ph;
          sub.type = IO_TYPE_MC_PHOTONS;
          if (search_sub_item(iobuf, &ih, &sub) < 0) break;
          if (read_tel_photons(iobuf, MAX_BUNCH, &arr, &tel, &ph, bunches, &nb) < 0) continue;
          printf("PHOTONS %d %d %.9g %d\n", arr, tel, ph, nb);
          for (j = 0; j < nb; ++j)
            printf("B %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", bunches[j].x, bunches[j].y, bunches[j].cx,
                   bunches[j].cy, bunches[j].ctime, bunches[j].zem, bunches[j].photons, bunches[j].lambda);
        }
        end_read_tel_array(iobuf, &ih);
        break;
      }
      case IO_TYPE_MC_EVTE:
        printf("EVTE\n");
        break;
      case IO_TYPE_MC_RUNE:
        printf("RUNE\n");
        break;
      default:
        printf("BLOCK %ld\n", (long)block.type);
        break;
    }
  }
  return 0;
}
