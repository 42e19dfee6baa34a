/* Force-included before every reference source compiled for oracle/_ref.
 * Replaces the reference's src/globals.h switches: float build (the fp32
 * decode path), with the compact-table sizes of the code picked by REF_CODE
 * (1 = BG1, 2 = BG2, 3 = 802.11n 12x24). */
#ifndef REF_EMUL_PRELUDE_H
#define REF_EMUL_PRELUDE_H
#define GLOBALS
#define HALF_PRC 0
#define CHAR_PRC 0
#if REF_CODE == 1
#define BLK_ROW 46
#define BLK_COL 68
#define NON_EMPTY_ROW 19
#define NON_EMPTY_COL 30
#elif REF_CODE == 2
#define BLK_ROW 42
#define BLK_COL 52
#define NON_EMPTY_ROW 10
#define NON_EMPTY_COL 23
#elif REF_CODE == 3
#define BLK_ROW 12
#define BLK_COL 24
#define NON_EMPTY_ROW REF_WIFI_ROWDEG
#define NON_EMPTY_COL REF_WIFI_COLDEG
#else
#error "REF_CODE must be 1, 2 or 3"
#endif
#define H_COMPACT1_ROW BLK_ROW
#define H_COMPACT1_COL NON_EMPTY_ROW
#define H_COMPACT2_ROW NON_EMPTY_COL
#define H_COMPACT2_COL BLK_COL
#endif
