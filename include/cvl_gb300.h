/*
 * cvl_gb300.h -- C ABI of libcvl_gb300.so, the GB300 (sm_103a) CVL library.
 *
 * Drop-in for the C vector library that NESL's VCODE interpreter (vinterp)
 * and fused .fcode super-op libraries call: every prototype of
 * nesl/include/cvl.h of Nessie-Compiler/neslgpu, with the same name, C types
 * and argument meaning.  The comment after each prototype gives the line of
 * the cvl.h prototype it replaces.
 *
 * vec_p is the HAS_VOIDP form of cvl.h (cvl.h:50-53): a raw device pointer
 * into a heap allocated with alo_foz.  Sizes (alo_foz, siz_fo*, F_scratch)
 * count 8-byte units, as in the serial CVL (CVL_SIZE_UNIT = sizeof(MAXALIGN),
 * nesl/cvl/serial/facilt.c:92-93).  Every F has int F_scratch(...) (units of
 * caller-provided scratch; NULL scratch makes the library use its own
 * workspace) and unsigned F_inplace(void) (INPLACE_k bits, cvl.h:98-110).
 *
 * Calls are ordered on one library stream (gcvl_set_stream to change it).
 * Functions that return a scalar to the host, and the v2c/c2v transfers,
 * synchronise.  The ABI has no error returns: errors are recorded and read
 * with gcvl_last_error / gcvl_sync.
 */
#ifndef CVL_GB300_H
#define CVL_GB300_H

#include <stddef.h>
#include <time.h>

typedef void *vec_p;
typedef int cvl_bool;
typedef struct timespec cvl_timer_t;

#define CVL_SCRATCH_NULL ((vec_p)0)
#define INPLACE_NONE 0
#define INPLACE_1 0x001
#define INPLACE_2 0x002
#define INPLACE_3 0x004
#define INPLACE_4 0x008
#define INPLACE_5 0x010
#define INPLACE_6 0x020
#define INPLACE_7 0x040
#define INPLACE_8 0x080
#define INPLACE_9 0x100
#define INPLACE_10 0x200
#define INPLACE_11 0x400
#define INPLACE_12 0x800

#ifdef __cplusplus
extern "C" {
#endif

/* CVL_init (cvl.h:121-123, CUDA build): records the fused super-op library
 * named by vinterp's -l flag and brings the device up. */
void CVL_init(char*);                                                                                /* cvl.h:122 */

/* Elementwise maps (*_wu*): serial semantics nesl/cvl/serial/elwise.c:192-298; the
 * reference CUDA CVL maps are nesl/cvl/cuda/elementwise.gpu.cu:3-144. */
void max_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:124 */
int max_wuz_scratch(int len);                                                                        /* cvl.h:125 */
unsigned int max_wuz_inplace(void);                                                                  /* cvl.h:126 */
void max_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:127 */
int max_wud_scratch(int len);                                                                        /* cvl.h:128 */
unsigned int max_wud_inplace(void);                                                                  /* cvl.h:129 */
void min_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:130 */
int min_wuz_scratch(int len);                                                                        /* cvl.h:131 */
unsigned int min_wuz_inplace(void);                                                                  /* cvl.h:132 */
void min_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:133 */
int min_wud_scratch(int len);                                                                        /* cvl.h:134 */
unsigned int min_wud_inplace(void);                                                                  /* cvl.h:135 */
void add_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:136 */
int add_wuz_scratch(int len);                                                                        /* cvl.h:137 */
unsigned int add_wuz_inplace(void);                                                                  /* cvl.h:138 */
void add_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:139 */
int add_wud_scratch(int len);                                                                        /* cvl.h:140 */
unsigned int add_wud_inplace(void);                                                                  /* cvl.h:141 */
void sub_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:142 */
int sub_wuz_scratch(int len);                                                                        /* cvl.h:143 */
unsigned int sub_wuz_inplace(void);                                                                  /* cvl.h:144 */
void sub_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:145 */
int sub_wud_scratch(int len);                                                                        /* cvl.h:146 */
unsigned int sub_wud_inplace(void);                                                                  /* cvl.h:147 */
void mul_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:148 */
int mul_wuz_scratch(int len);                                                                        /* cvl.h:149 */
unsigned int mul_wuz_inplace(void);                                                                  /* cvl.h:150 */
void mul_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:151 */
int mul_wud_scratch(int len);                                                                        /* cvl.h:152 */
unsigned int mul_wud_inplace(void);                                                                  /* cvl.h:153 */
void div_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:154 */
int div_wuz_scratch(int len);                                                                        /* cvl.h:155 */
unsigned int div_wuz_inplace(void);                                                                  /* cvl.h:156 */
void div_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:157 */
int div_wud_scratch(int len);                                                                        /* cvl.h:158 */
unsigned int div_wud_inplace(void);                                                                  /* cvl.h:159 */
void grt_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:160 */
int grt_wuz_scratch(int len);                                                                        /* cvl.h:161 */
unsigned int grt_wuz_inplace(void);                                                                  /* cvl.h:162 */
void grt_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:163 */
int grt_wud_scratch(int len);                                                                        /* cvl.h:164 */
unsigned int grt_wud_inplace(void);                                                                  /* cvl.h:165 */
void les_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:166 */
int les_wuz_scratch(int len);                                                                        /* cvl.h:167 */
unsigned int les_wuz_inplace(void);                                                                  /* cvl.h:168 */
void les_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:169 */
int les_wud_scratch(int len);                                                                        /* cvl.h:170 */
unsigned int les_wud_inplace(void);                                                                  /* cvl.h:171 */
void geq_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:172 */
int geq_wuz_scratch(int len);                                                                        /* cvl.h:173 */
unsigned int geq_wuz_inplace(void);                                                                  /* cvl.h:174 */
void geq_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:175 */
int geq_wud_scratch(int len);                                                                        /* cvl.h:176 */
unsigned int geq_wud_inplace(void);                                                                  /* cvl.h:177 */
void leq_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:178 */
int leq_wuz_scratch(int len);                                                                        /* cvl.h:179 */
unsigned int leq_wuz_inplace(void);                                                                  /* cvl.h:180 */
void leq_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:181 */
int leq_wud_scratch(int len);                                                                        /* cvl.h:182 */
unsigned int leq_wud_inplace(void);                                                                  /* cvl.h:183 */
void lsh_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:184 */
int lsh_wuz_scratch(int len);                                                                        /* cvl.h:185 */
unsigned int lsh_wuz_inplace(void);                                                                  /* cvl.h:186 */
void rsh_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:187 */
int rsh_wuz_scratch(int len);                                                                        /* cvl.h:188 */
unsigned int rsh_wuz_inplace(void);                                                                  /* cvl.h:189 */
void mod_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:190 */
int mod_wuz_scratch(int len);                                                                        /* cvl.h:191 */
unsigned int mod_wuz_inplace(void);                                                                  /* cvl.h:192 */
void rnd_wuz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:193 */
int rnd_wuz_scratch(int len);                                                                        /* cvl.h:194 */
unsigned int rnd_wuz_inplace(void);                                                                  /* cvl.h:195 */
void eql_wub(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:196 */
int eql_wub_scratch(int len);                                                                        /* cvl.h:197 */
unsigned int eql_wub_inplace(void);                                                                  /* cvl.h:198 */
void eql_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:199 */
int eql_wuz_scratch(int len);                                                                        /* cvl.h:200 */
unsigned int eql_wuz_inplace(void);                                                                  /* cvl.h:201 */
void eql_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:202 */
int eql_wud_scratch(int len);                                                                        /* cvl.h:203 */
unsigned int eql_wud_inplace(void);                                                                  /* cvl.h:204 */
void neq_wub(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:205 */
int neq_wub_scratch(int len);                                                                        /* cvl.h:206 */
unsigned int neq_wub_inplace(void);                                                                  /* cvl.h:207 */
void neq_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:208 */
int neq_wuz_scratch(int len);                                                                        /* cvl.h:209 */
unsigned int neq_wuz_inplace(void);                                                                  /* cvl.h:210 */
void neq_wud(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:211 */
int neq_wud_scratch(int len);                                                                        /* cvl.h:212 */
unsigned int neq_wud_inplace(void);                                                                  /* cvl.h:213 */
void sel_wuz(vec_p d, vec_p s1, vec_p s2, vec_p s3, int len, vec_p scratch);                         /* cvl.h:214 */
int sel_wuz_scratch(int len);                                                                        /* cvl.h:215 */
unsigned int sel_wuz_inplace(void);                                                                  /* cvl.h:216 */
void sel_wub(vec_p d, vec_p s1, vec_p s2, vec_p s3, int len, vec_p scratch);                         /* cvl.h:217 */
int sel_wub_scratch(int len);                                                                        /* cvl.h:218 */
unsigned int sel_wub_inplace(void);                                                                  /* cvl.h:219 */
void sel_wud(vec_p d, vec_p s1, vec_p s2, vec_p s3, int len, vec_p scratch);                         /* cvl.h:220 */
int sel_wud_scratch(int len);                                                                        /* cvl.h:221 */
unsigned int sel_wud_inplace(void);                                                                  /* cvl.h:222 */
void not_wub(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:223 */
int not_wub_scratch(int len);                                                                        /* cvl.h:224 */
unsigned int not_wub_inplace(void);                                                                  /* cvl.h:225 */
void xor_wub(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:226 */
int xor_wub_scratch(int len);                                                                        /* cvl.h:227 */
unsigned int xor_wub_inplace(void);                                                                  /* cvl.h:228 */
void ior_wub(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:229 */
int ior_wub_scratch(int len);                                                                        /* cvl.h:230 */
unsigned int ior_wub_inplace(void);                                                                  /* cvl.h:231 */
void and_wub(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:232 */
int and_wub_scratch(int len);                                                                        /* cvl.h:233 */
unsigned int and_wub_inplace(void);                                                                  /* cvl.h:234 */
void ior_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:235 */
int ior_wuz_scratch(int len);                                                                        /* cvl.h:236 */
unsigned int ior_wuz_inplace(void);                                                                  /* cvl.h:237 */
void and_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:238 */
int and_wuz_scratch(int len);                                                                        /* cvl.h:239 */
unsigned int and_wuz_inplace(void);                                                                  /* cvl.h:240 */
void not_wuz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:241 */
int not_wuz_scratch(int len);                                                                        /* cvl.h:242 */
unsigned int not_wuz_inplace(void);                                                                  /* cvl.h:243 */
void xor_wuz(vec_p d, vec_p s1, vec_p s2, int len, vec_p scratch);                                   /* cvl.h:244 */
int xor_wuz_scratch(int len);                                                                        /* cvl.h:245 */
unsigned int xor_wuz_inplace(void);                                                                  /* cvl.h:246 */
void int_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:247 */
int int_wud_scratch(int len);                                                                        /* cvl.h:248 */
unsigned int int_wud_inplace(void);                                                                  /* cvl.h:249 */
void int_wub(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:250 */
int int_wub_scratch(int len);                                                                        /* cvl.h:251 */
unsigned int int_wub_inplace(void);                                                                  /* cvl.h:252 */
void dbl_wuz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:253 */
int dbl_wuz_scratch(int len);                                                                        /* cvl.h:254 */
unsigned int dbl_wuz_inplace(void);                                                                  /* cvl.h:255 */
void boo_wuz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:256 */
int boo_wuz_scratch(int len);                                                                        /* cvl.h:257 */
unsigned int boo_wuz_inplace(void);                                                                  /* cvl.h:258 */
void flr_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:259 */
int flr_wud_scratch(int len);                                                                        /* cvl.h:260 */
unsigned int flr_wud_inplace(void);                                                                  /* cvl.h:261 */
void cei_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:262 */
int cei_wud_scratch(int len);                                                                        /* cvl.h:263 */
unsigned int cei_wud_inplace(void);                                                                  /* cvl.h:264 */
void trn_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:265 */
int trn_wud_scratch(int len);                                                                        /* cvl.h:266 */
unsigned int trn_wud_inplace(void);                                                                  /* cvl.h:267 */
void rou_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:268 */
int rou_wud_scratch(int len);                                                                        /* cvl.h:269 */
unsigned int rou_wud_inplace(void);                                                                  /* cvl.h:270 */
void exp_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:271 */
int exp_wud_scratch(int len);                                                                        /* cvl.h:272 */
unsigned int exp_wud_inplace(void);                                                                  /* cvl.h:273 */
void log_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:274 */
int log_wud_scratch(int len);                                                                        /* cvl.h:275 */
unsigned int log_wud_inplace(void);                                                                  /* cvl.h:276 */
void sqt_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:277 */
int sqt_wud_scratch(int len);                                                                        /* cvl.h:278 */
unsigned int sqt_wud_inplace(void);                                                                  /* cvl.h:279 */
void sin_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:280 */
int sin_wud_scratch(int len);                                                                        /* cvl.h:281 */
unsigned int sin_wud_inplace(void);                                                                  /* cvl.h:282 */
void cos_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:283 */
int cos_wud_scratch(int len);                                                                        /* cvl.h:284 */
unsigned int cos_wud_inplace(void);                                                                  /* cvl.h:285 */
void tan_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:286 */
int tan_wud_scratch(int len);                                                                        /* cvl.h:287 */
unsigned int tan_wud_inplace(void);                                                                  /* cvl.h:288 */
void asn_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:289 */
int asn_wud_scratch(int len);                                                                        /* cvl.h:290 */
unsigned int asn_wud_inplace(void);                                                                  /* cvl.h:291 */
void acs_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:292 */
int acs_wud_scratch(int len);                                                                        /* cvl.h:293 */
unsigned int acs_wud_inplace(void);                                                                  /* cvl.h:294 */
void atn_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:295 */
int atn_wud_scratch(int len);                                                                        /* cvl.h:296 */
unsigned int atn_wud_inplace(void);                                                                  /* cvl.h:297 */
void snh_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:298 */
int snh_wud_scratch(int len);                                                                        /* cvl.h:299 */
unsigned int snh_wud_inplace(void);                                                                  /* cvl.h:300 */
void csh_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:301 */
int csh_wud_scratch(int len);                                                                        /* cvl.h:302 */
unsigned int csh_wud_inplace(void);                                                                  /* cvl.h:303 */
void tnh_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:304 */
int tnh_wud_scratch(int len);                                                                        /* cvl.h:305 */
unsigned int tnh_wud_inplace(void);                                                                  /* cvl.h:306 */
void cpy_wuz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:307 */
int cpy_wuz_scratch(int len);                                                                        /* cvl.h:308 */
unsigned int cpy_wuz_inplace(void);                                                                  /* cvl.h:309 */
void cpy_wub(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:310 */
int cpy_wub_scratch(int len);                                                                        /* cvl.h:311 */
unsigned int cpy_wub_inplace(void);                                                                  /* cvl.h:312 */
void cpy_wud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:313 */
int cpy_wud_scratch(int len);                                                                        /* cvl.h:314 */
unsigned int cpy_wud_inplace(void);                                                                  /* cvl.h:315 */
void cpy_wus(vec_p d, vec_p s, int n, int m, vec_p scratch);                                         /* cvl.h:316 */
int cpy_wus_scratch(int n, int m);                                                                   /* cvl.h:317 */
unsigned int cpy_wus_inplace(void);                                                                  /* cvl.h:318 */

/* Unsegmented exclusive scans (*_su*): nesl/cvl/serial/vprims.c:17-49; CUDA CVL
 * nesl/cvl/cuda/vprims.c:93-105 (thrust::exclusive_scan). */
void add_suz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:319 */
int add_suz_scratch(int len);                                                                        /* cvl.h:320 */
unsigned int add_suz_inplace(void);                                                                  /* cvl.h:321 */
void add_sud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:322 */
int add_sud_scratch(int len);                                                                        /* cvl.h:323 */
unsigned int add_sud_inplace(void);                                                                  /* cvl.h:324 */
void mul_suz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:325 */
int mul_suz_scratch(int len);                                                                        /* cvl.h:326 */
unsigned int mul_suz_inplace(void);                                                                  /* cvl.h:327 */
void mul_sud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:328 */
int mul_sud_scratch(int len);                                                                        /* cvl.h:329 */
unsigned int mul_sud_inplace(void);                                                                  /* cvl.h:330 */
void min_suz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:331 */
int min_suz_scratch(int len);                                                                        /* cvl.h:332 */
unsigned int min_suz_inplace(void);                                                                  /* cvl.h:333 */
void min_sud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:334 */
int min_sud_scratch(int len);                                                                        /* cvl.h:335 */
unsigned int min_sud_inplace(void);                                                                  /* cvl.h:336 */
void max_suz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:337 */
int max_suz_scratch(int len);                                                                        /* cvl.h:338 */
unsigned int max_suz_inplace(void);                                                                  /* cvl.h:339 */
void max_sud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:340 */
int max_sud_scratch(int len);                                                                        /* cvl.h:341 */
unsigned int max_sud_inplace(void);                                                                  /* cvl.h:342 */
void and_sub(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:343 */
int and_sub_scratch(int len);                                                                        /* cvl.h:344 */
unsigned int and_sub_inplace(void);                                                                  /* cvl.h:345 */
void and_suz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:346 */
int and_suz_scratch(int len);                                                                        /* cvl.h:347 */
unsigned int and_suz_inplace(void);                                                                  /* cvl.h:348 */
void ior_sub(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:349 */
int ior_sub_scratch(int len);                                                                        /* cvl.h:350 */
unsigned int ior_sub_inplace(void);                                                                  /* cvl.h:351 */
void ior_suz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:352 */
int ior_suz_scratch(int len);                                                                        /* cvl.h:353 */
unsigned int ior_suz_inplace(void);                                                                  /* cvl.h:354 */
void xor_sub(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:355 */
int xor_sub_scratch(int len);                                                                        /* cvl.h:356 */
unsigned int xor_sub_inplace(void);                                                                  /* cvl.h:357 */
void xor_suz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:358 */
int xor_suz_scratch(int len);                                                                        /* cvl.h:359 */
unsigned int xor_suz_inplace(void);                                                                  /* cvl.h:360 */

/* Segmented exclusive scans (*_se*): nesl/cvl/serial/vprims.c:62-109; CUDA CVL
 * nesl/cvl/cuda/vprims.c:118-134 (exclusive_scan_by_key).  Single-pass
 * decoupled look-back kernel; scratch = tile status (F_scratch units). */
void add_sez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:361 */
int add_sez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:362 */
unsigned int add_sez_inplace(void);                                                                  /* cvl.h:363 */
void add_sed(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:364 */
int add_sed_scratch(int vec_len, int seg_len);                                                       /* cvl.h:365 */
unsigned int add_sed_inplace(void);                                                                  /* cvl.h:366 */
void mul_sez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:367 */
int mul_sez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:368 */
unsigned int mul_sez_inplace(void);                                                                  /* cvl.h:369 */
void mul_sed(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:370 */
int mul_sed_scratch(int vec_len, int seg_len);                                                       /* cvl.h:371 */
unsigned int mul_sed_inplace(void);                                                                  /* cvl.h:372 */
void min_sez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:373 */
int min_sez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:374 */
unsigned int min_sez_inplace(void);                                                                  /* cvl.h:375 */
void min_sed(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:376 */
int min_sed_scratch(int vec_len, int seg_len);                                                       /* cvl.h:377 */
unsigned int min_sed_inplace(void);                                                                  /* cvl.h:378 */
void max_sez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:379 */
int max_sez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:380 */
unsigned int max_sez_inplace(void);                                                                  /* cvl.h:381 */
void max_sed(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:382 */
int max_sed_scratch(int vec_len, int seg_len);                                                       /* cvl.h:383 */
unsigned int max_sed_inplace(void);                                                                  /* cvl.h:384 */
void and_seb(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:385 */
int and_seb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:386 */
unsigned int and_seb_inplace(void);                                                                  /* cvl.h:387 */
void and_sez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:388 */
int and_sez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:389 */
unsigned int and_sez_inplace(void);                                                                  /* cvl.h:390 */
void ior_seb(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:391 */
int ior_seb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:392 */
unsigned int ior_seb_inplace(void);                                                                  /* cvl.h:393 */
void ior_sez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:394 */
int ior_sez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:395 */
unsigned int ior_sez_inplace(void);                                                                  /* cvl.h:396 */
void xor_seb(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:397 */
int xor_seb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:398 */
unsigned int xor_seb_inplace(void);                                                                  /* cvl.h:399 */
void xor_sez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:400 */
int xor_sez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:401 */
unsigned int xor_sez_inplace(void);                                                                  /* cvl.h:402 */

/* Unsegmented reductions (*_ru*, return to the host): nesl/cvl/serial/vprims.c:114-146;
 * CUDA CVL nesl/cvl/cuda/vprims.c:139-152. */
int add_ruz(vec_p s, int len, vec_p scratch);                                                        /* cvl.h:403 */
int add_ruz_scratch(int len);                                                                        /* cvl.h:404 */
unsigned int add_ruz_inplace(void);                                                                  /* cvl.h:405 */
double add_rud(vec_p s, int len, vec_p scratch);                                                     /* cvl.h:406 */
int add_rud_scratch(int len);                                                                        /* cvl.h:407 */
unsigned int add_rud_inplace(void);                                                                  /* cvl.h:408 */
int mul_ruz(vec_p s, int len, vec_p scratch);                                                        /* cvl.h:409 */
int mul_ruz_scratch(int len);                                                                        /* cvl.h:410 */
unsigned int mul_ruz_inplace(void);                                                                  /* cvl.h:411 */
double mul_rud(vec_p s, int len, vec_p scratch);                                                     /* cvl.h:412 */
int mul_rud_scratch(int len);                                                                        /* cvl.h:413 */
unsigned int mul_rud_inplace(void);                                                                  /* cvl.h:414 */
int min_ruz(vec_p s, int len, vec_p scratch);                                                        /* cvl.h:415 */
int min_ruz_scratch(int len);                                                                        /* cvl.h:416 */
unsigned int min_ruz_inplace(void);                                                                  /* cvl.h:417 */
double min_rud(vec_p s, int len, vec_p scratch);                                                     /* cvl.h:418 */
int min_rud_scratch(int len);                                                                        /* cvl.h:419 */
unsigned int min_rud_inplace(void);                                                                  /* cvl.h:420 */
int max_ruz(vec_p s, int len, vec_p scratch);                                                        /* cvl.h:421 */
int max_ruz_scratch(int len);                                                                        /* cvl.h:422 */
unsigned int max_ruz_inplace(void);                                                                  /* cvl.h:423 */
double max_rud(vec_p s, int len, vec_p scratch);                                                     /* cvl.h:424 */
int max_rud_scratch(int len);                                                                        /* cvl.h:425 */
unsigned int max_rud_inplace(void);                                                                  /* cvl.h:426 */
cvl_bool and_rub(vec_p s, int len, vec_p scratch);                                                   /* cvl.h:427 */
int and_rub_scratch(int len);                                                                        /* cvl.h:428 */
unsigned int and_rub_inplace(void);                                                                  /* cvl.h:429 */
int and_ruz(vec_p s, int len, vec_p scratch);                                                        /* cvl.h:430 */
int and_ruz_scratch(int len);                                                                        /* cvl.h:431 */
unsigned int and_ruz_inplace(void);                                                                  /* cvl.h:432 */
cvl_bool ior_rub(vec_p s, int len, vec_p scratch);                                                   /* cvl.h:433 */
int ior_rub_scratch(int len);                                                                        /* cvl.h:434 */
unsigned int ior_rub_inplace(void);                                                                  /* cvl.h:435 */
int ior_ruz(vec_p s, int len, vec_p scratch);                                                        /* cvl.h:436 */
int ior_ruz_scratch(int len);                                                                        /* cvl.h:437 */
unsigned int ior_ruz_inplace(void);                                                                  /* cvl.h:438 */
cvl_bool xor_rub(vec_p s, int len, vec_p scratch);                                                   /* cvl.h:439 */
int xor_rub_scratch(int len);                                                                        /* cvl.h:440 */
unsigned int xor_rub_inplace(void);                                                                  /* cvl.h:441 */
int xor_ruz(vec_p s, int len, vec_p scratch);                                                        /* cvl.h:442 */
int xor_ruz_scratch(int len);                                                                        /* cvl.h:443 */
unsigned int xor_ruz_inplace(void);                                                                  /* cvl.h:444 */

/* Segmented reductions (*_re*): nesl/cvl/serial/vprims.c:155-201; CUDA CVL
 * nesl/cvl/cuda/vprims.c:162-202.  Empty segments yield the initial value. */
void add_rez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:445 */
int add_rez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:446 */
unsigned int add_rez_inplace(void);                                                                  /* cvl.h:447 */
void add_red(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:448 */
int add_red_scratch(int vec_len, int seg_len);                                                       /* cvl.h:449 */
unsigned int add_red_inplace(void);                                                                  /* cvl.h:450 */
void mul_rez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:451 */
int mul_rez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:452 */
unsigned int mul_rez_inplace(void);                                                                  /* cvl.h:453 */
void mul_red(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:454 */
int mul_red_scratch(int vec_len, int seg_len);                                                       /* cvl.h:455 */
unsigned int mul_red_inplace(void);                                                                  /* cvl.h:456 */
void min_rez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:457 */
int min_rez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:458 */
unsigned int min_rez_inplace(void);                                                                  /* cvl.h:459 */
void min_red(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:460 */
int min_red_scratch(int vec_len, int seg_len);                                                       /* cvl.h:461 */
unsigned int min_red_inplace(void);                                                                  /* cvl.h:462 */
void max_rez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:463 */
int max_rez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:464 */
unsigned int max_rez_inplace(void);                                                                  /* cvl.h:465 */
void max_red(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:466 */
int max_red_scratch(int vec_len, int seg_len);                                                       /* cvl.h:467 */
unsigned int max_red_inplace(void);                                                                  /* cvl.h:468 */
void and_reb(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:469 */
int and_reb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:470 */
unsigned int and_reb_inplace(void);                                                                  /* cvl.h:471 */
void and_rez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:472 */
int and_rez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:473 */
unsigned int and_rez_inplace(void);                                                                  /* cvl.h:474 */
void ior_reb(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:475 */
int ior_reb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:476 */
unsigned int ior_reb_inplace(void);                                                                  /* cvl.h:477 */
void ior_rez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:478 */
int ior_rez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:479 */
unsigned int ior_rez_inplace(void);                                                                  /* cvl.h:480 */
void xor_reb(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:481 */
int xor_reb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:482 */
unsigned int xor_reb_inplace(void);                                                                  /* cvl.h:483 */
void xor_rez(vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:484 */
int xor_rez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:485 */
unsigned int xor_rez_inplace(void);                                                                  /* cvl.h:486 */

/* Extract / replace / distribute (ext_*, rep_*, dis_*): nesl/cvl/serial/vprims.c:207-344;
 * CUDA CVL nesl/cvl/cuda/vprims.c:208-316. */
int ext_vuz(vec_p V, int i, int len, vec_p scratch);                                                 /* cvl.h:487 */
int ext_vuz_scratch(int len);                                                                        /* cvl.h:488 */
unsigned int ext_vuz_inplace(void);                                                                  /* cvl.h:489 */
cvl_bool ext_vub(vec_p V, int i, int len, vec_p scratch);                                            /* cvl.h:490 */
int ext_vub_scratch(int len);                                                                        /* cvl.h:491 */
unsigned int ext_vub_inplace(void);                                                                  /* cvl.h:492 */
double ext_vud(vec_p V, int i, int len, vec_p scratch);                                              /* cvl.h:493 */
int ext_vud_scratch(int len);                                                                        /* cvl.h:494 */
unsigned int ext_vud_inplace(void);                                                                  /* cvl.h:495 */
void ext_vez(vec_p d, vec_p s, vec_p i, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:496 */
int ext_vez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:497 */
unsigned int ext_vez_inplace(void);                                                                  /* cvl.h:498 */
void ext_veb(vec_p d, vec_p s, vec_p i, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:499 */
int ext_veb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:500 */
unsigned int ext_veb_inplace(void);                                                                  /* cvl.h:501 */
void ext_ved(vec_p d, vec_p s, vec_p i, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:502 */
int ext_ved_scratch(int vec_len, int seg_len);                                                       /* cvl.h:503 */
unsigned int ext_ved_inplace(void);                                                                  /* cvl.h:504 */
void rep_vuz(vec_p V, int i, int val, int len, vec_p scratch);                                       /* cvl.h:505 */
int rep_vuz_scratch(int len);                                                                        /* cvl.h:506 */
unsigned int rep_vuz_inplace(void);                                                                  /* cvl.h:507 */
void rep_vub(vec_p V, int i, cvl_bool val, int len, vec_p scratch);                                  /* cvl.h:508 */
int rep_vub_scratch(int len);                                                                        /* cvl.h:509 */
unsigned int rep_vub_inplace(void);                                                                  /* cvl.h:510 */
void rep_vud(vec_p V, int i, double val, int len, vec_p scratch);                                    /* cvl.h:511 */
int rep_vud_scratch(int len);                                                                        /* cvl.h:512 */
unsigned int rep_vud_inplace(void);                                                                  /* cvl.h:513 */
void rep_vez(vec_p d, vec_p s, vec_p v, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:514 */
int rep_vez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:515 */
unsigned int rep_vez_inplace(void);                                                                  /* cvl.h:516 */
void rep_veb(vec_p d, vec_p s, vec_p v, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:517 */
int rep_veb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:518 */
unsigned int rep_veb_inplace(void);                                                                  /* cvl.h:519 */
void rep_ved(vec_p d, vec_p s, vec_p v, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:520 */
int rep_ved_scratch(int vec_len, int seg_len);                                                       /* cvl.h:521 */
unsigned int rep_ved_inplace(void);                                                                  /* cvl.h:522 */
void dis_vuz(vec_p d, int v, int len, vec_p scratch);                                                /* cvl.h:523 */
int dis_vuz_scratch(int len);                                                                        /* cvl.h:524 */
unsigned int dis_vuz_inplace(void);                                                                  /* cvl.h:525 */
void dis_vub(vec_p d, cvl_bool v, int len, vec_p scratch);                                           /* cvl.h:526 */
int dis_vub_scratch(int len);                                                                        /* cvl.h:527 */
unsigned int dis_vub_inplace(void);                                                                  /* cvl.h:528 */
void dis_vud(vec_p d, double v, int len, vec_p scratch);                                             /* cvl.h:529 */
int dis_vud_scratch(int len);                                                                        /* cvl.h:530 */
unsigned int dis_vud_inplace(void);                                                                  /* cvl.h:531 */
void dis_vez(vec_p d, vec_p v, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:532 */
int dis_vez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:533 */
unsigned int dis_vez_inplace(void);                                                                  /* cvl.h:534 */
void dis_veb(vec_p d, vec_p v, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:535 */
int dis_veb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:536 */
unsigned int dis_veb_inplace(void);                                                                  /* cvl.h:537 */
void dis_ved(vec_p d, vec_p v, vec_p sd, int n, int m, vec_p scratch);                               /* cvl.h:538 */
int dis_ved_scratch(int vec_len, int seg_len);                                                       /* cvl.h:539 */
unsigned int dis_ved_inplace(void);                                                                  /* cvl.h:540 */

/* Permute / back-permute (smp_*, bck_*): nesl/cvl/serial/vprims.c:356-467; CUDA CVL
 * nesl/cvl/cuda/vprims.c:327-411. */
void smp_puz(vec_p d, vec_p s, vec_p i, int len, vec_p scratch);                                     /* cvl.h:541 */
int smp_puz_scratch(int len);                                                                        /* cvl.h:542 */
unsigned int smp_puz_inplace(void);                                                                  /* cvl.h:543 */
void smp_pub(vec_p d, vec_p s, vec_p i, int len, vec_p scratch);                                     /* cvl.h:544 */
int smp_pub_scratch(int len);                                                                        /* cvl.h:545 */
unsigned int smp_pub_inplace(void);                                                                  /* cvl.h:546 */
void smp_pud(vec_p d, vec_p s, vec_p i, int len, vec_p scratch);                                     /* cvl.h:547 */
int smp_pud_scratch(int len);                                                                        /* cvl.h:548 */
unsigned int smp_pud_inplace(void);                                                                  /* cvl.h:549 */
void smp_pez(vec_p d, vec_p s, vec_p i, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:550 */
int smp_pez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:551 */
unsigned int smp_pez_inplace(void);                                                                  /* cvl.h:552 */
void smp_peb(vec_p d, vec_p s, vec_p i, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:553 */
int smp_peb_scratch(int vec_len, int seg_len);                                                       /* cvl.h:554 */
unsigned int smp_peb_inplace(void);                                                                  /* cvl.h:555 */
void smp_ped(vec_p d, vec_p s, vec_p i, vec_p sd, int n, int m, vec_p scratch);                      /* cvl.h:556 */
int smp_ped_scratch(int vec_len, int seg_len);                                                       /* cvl.h:557 */
unsigned int smp_ped_inplace(void);                                                                  /* cvl.h:558 */
void bck_puz(vec_p d, vec_p s, vec_p i, int s_len, int d_len, vec_p scratch);                        /* cvl.h:559 */
int bck_puz_scratch(int s_len, int d_len);                                                           /* cvl.h:560 */
unsigned int bck_puz_inplace(void);                                                                  /* cvl.h:561 */
void bck_pub(vec_p d, vec_p s, vec_p i, int s_len, int d_len, vec_p scratch);                        /* cvl.h:562 */
int bck_pub_scratch(int s_len, int d_len);                                                           /* cvl.h:563 */
unsigned int bck_pub_inplace(void);                                                                  /* cvl.h:564 */
void bck_pud(vec_p d, vec_p s, vec_p i, int s_len, int d_len, vec_p scratch);                        /* cvl.h:565 */
int bck_pud_scratch(int s_len, int d_len);                                                           /* cvl.h:566 */
unsigned int bck_pud_inplace(void);                                                                  /* cvl.h:567 */
void bck_pez(vec_p d, vec_p s, vec_p i, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:568 */
int bck_pez_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:569 */
unsigned int bck_pez_inplace(void);                                                                  /* cvl.h:570 */
void bck_peb(vec_p d, vec_p s, vec_p i, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:571 */
int bck_peb_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:572 */
unsigned int bck_peb_inplace(void);                                                                  /* cvl.h:573 */
void bck_ped(vec_p d, vec_p s, vec_p i, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:574 */
int bck_ped_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:575 */
unsigned int bck_ped_inplace(void);                                                                  /* cvl.h:576 */

/* Flag and default permutes (fpm_*, bfp_*, dpe_*, dfp_*): nesl/cvl/serial/vecops.c:22-286;
 * CUDA CVL nesl/cvl/cuda/vecops.c:15-182. */
void fpm_puz(vec_p d, vec_p s, vec_p i, vec_p f, int len_src, int len_dest, vec_p scratch);          /* cvl.h:577 */
int fpm_puz_scratch(int s_len, int d_len);                                                           /* cvl.h:578 */
unsigned int fpm_puz_inplace(void);                                                                  /* cvl.h:579 */
void fpm_pub(vec_p d, vec_p s, vec_p i, vec_p f, int len_src, int len_dest, vec_p scratch);          /* cvl.h:580 */
int fpm_pub_scratch(int s_len, int d_len);                                                           /* cvl.h:581 */
unsigned int fpm_pub_inplace(void);                                                                  /* cvl.h:582 */
void fpm_pud(vec_p d, vec_p s, vec_p i, vec_p f, int len_src, int len_dest, vec_p scratch);          /* cvl.h:583 */
int fpm_pud_scratch(int s_len, int d_len);                                                           /* cvl.h:584 */
unsigned int fpm_pud_inplace(void);                                                                  /* cvl.h:585 */
void fpm_pez(vec_p d, vec_p s, vec_p i, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:586 */
int fpm_pez_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:587 */
unsigned int fpm_pez_inplace(void);                                                                  /* cvl.h:588 */
void fpm_peb(vec_p d, vec_p s, vec_p i, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:589 */
int fpm_peb_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:590 */
unsigned int fpm_peb_inplace(void);                                                                  /* cvl.h:591 */
void fpm_ped(vec_p d, vec_p s, vec_p i, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:592 */
int fpm_ped_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:593 */
unsigned int fpm_ped_inplace(void);                                                                  /* cvl.h:594 */
void bfp_puz(vec_p d, vec_p s, vec_p i, vec_p f, int len_src, int len_dest, vec_p scratch);          /* cvl.h:595 */
int bfp_puz_scratch(int s_len, int d_len);                                                           /* cvl.h:596 */
unsigned int bfp_puz_inplace(void);                                                                  /* cvl.h:597 */
void bfp_pub(vec_p d, vec_p s, vec_p i, vec_p f, int len_src, int len_dest, vec_p scratch);          /* cvl.h:598 */
int bfp_pub_scratch(int s_len, int d_len);                                                           /* cvl.h:599 */
unsigned int bfp_pub_inplace(void);                                                                  /* cvl.h:600 */
void bfp_pud(vec_p d, vec_p s, vec_p i, vec_p f, int len_src, int len_dest, vec_p scratch);          /* cvl.h:601 */
int bfp_pud_scratch(int s_len, int d_len);                                                           /* cvl.h:602 */
unsigned int bfp_pud_inplace(void);                                                                  /* cvl.h:603 */
void bfp_pez(vec_p d, vec_p s, vec_p i, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:604 */
int bfp_pez_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:605 */
unsigned int bfp_pez_inplace(void);                                                                  /* cvl.h:606 */
void bfp_peb(vec_p d, vec_p s, vec_p i, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:607 */
int bfp_peb_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:608 */
unsigned int bfp_peb_inplace(void);                                                                  /* cvl.h:609 */
void bfp_ped(vec_p d, vec_p s, vec_p i, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:610 */
int bfp_ped_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:611 */
unsigned int bfp_ped_inplace(void);                                                                  /* cvl.h:612 */
void dpe_puz(vec_p d, vec_p s, vec_p i, vec_p v, int len_src, int len_dest, vec_p scratch);          /* cvl.h:613 */
unsigned int dpe_puz_inplace(void);                                                                  /* cvl.h:614 */
int dpe_puz_scratch(int s_len, int d_len);                                                           /* cvl.h:615 */
void dpe_pub(vec_p d, vec_p s, vec_p i, vec_p v, int len_src, int len_dest, vec_p scratch);          /* cvl.h:616 */
unsigned int dpe_pub_inplace(void);                                                                  /* cvl.h:617 */
int dpe_pub_scratch(int s_len, int d_len);                                                           /* cvl.h:618 */
void dpe_pud(vec_p d, vec_p s, vec_p i, vec_p v, int len_src, int len_dest, vec_p scratch);          /* cvl.h:619 */
unsigned int dpe_pud_inplace(void);                                                                  /* cvl.h:620 */
int dpe_pud_scratch(int s_len, int d_len);                                                           /* cvl.h:621 */
void dpe_pez(vec_p d, vec_p s, vec_p i, vec_p v, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:622 */
void dpe_peb(vec_p d, vec_p s, vec_p i, vec_p v, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:623 */
void dpe_ped(vec_p d, vec_p s, vec_p i, vec_p v, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:624 */
unsigned int dpe_pez_inplace(void);                                                                  /* cvl.h:625 */
int dpe_pez_scratch(int n_in, int m_in, int n_out, int m_out);                                       /* cvl.h:626 */
unsigned int dpe_peb_inplace(void);                                                                  /* cvl.h:627 */
int dpe_peb_scratch(int n_in, int m_in, int n_out, int m_out);                                       /* cvl.h:628 */
unsigned int dpe_ped_inplace(void);                                                                  /* cvl.h:629 */
int dpe_ped_scratch(int n_in, int m_in, int n_out, int m_out);                                       /* cvl.h:630 */
void dfp_puz(vec_p d, vec_p s, vec_p i, vec_p f, vec_p v, int len_src, int len_dest, vec_p scratch); /* cvl.h:631 */
void dfp_pub(vec_p d, vec_p s, vec_p i, vec_p f, vec_p v, int len_src, int len_dest, vec_p scratch); /* cvl.h:632 */
void dfp_pud(vec_p d, vec_p s, vec_p i, vec_p f, vec_p v, int len_src, int len_dest, vec_p scratch); /* cvl.h:633 */
unsigned int dfp_puz_inplace(void);                                                                  /* cvl.h:634 */
int dfp_puz_scratch(int s_len, int d_len);                                                           /* cvl.h:635 */
unsigned int dfp_pub_inplace(void);                                                                  /* cvl.h:636 */
int dfp_pub_scratch(int s_len, int d_len);                                                           /* cvl.h:637 */
unsigned int dfp_pud_inplace(void);                                                                  /* cvl.h:638 */
int dfp_pud_scratch(int s_len, int d_len);                                                           /* cvl.h:639 */
void dfp_pez(vec_p d, vec_p s, vec_p i, vec_p f, vec_p v, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:640 */
void dfp_peb(vec_p d, vec_p s, vec_p i, vec_p f, vec_p v, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:641 */
void dfp_ped(vec_p d, vec_p s, vec_p i, vec_p f, vec_p v, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:642 */
unsigned int dfp_pez_inplace(void);                                                                  /* cvl.h:643 */
int dfp_pez_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:644 */
unsigned int dfp_peb_inplace(void);                                                                  /* cvl.h:645 */
int dfp_peb_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:646 */
unsigned int dfp_ped_inplace(void);                                                                  /* cvl.h:647 */
int dfp_ped_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:648 */

/* Facilities: timers, sizes, segment descriptors, memory, transfers
 * (nesl/cvl/serial/facilt.c; CUDA CVL nesl/cvl/cuda/facilities.c).  vec_p is a
 * device pointer; sizes are in 8-byte units.  The segment descriptor holds
 * lengths, offsets and a granule table (siz_fos(n, m) units). */
void tgt_fos(cvl_timer_t *cvl_timer_p);                                                              /* cvl.h:649 */
double tdf_fos(cvl_timer_t *t1, cvl_timer_t *t2);                                                    /* cvl.h:650 */
int siz_fob(int length);                                                                             /* cvl.h:651 */
int siz_foz(int length);                                                                             /* cvl.h:652 */
int siz_fod(int length);                                                                             /* cvl.h:653 */
int siz_fos(int n, int m);                                                                           /* cvl.h:654 */
void mke_fov(vec_p sd, vec_p l, int n, int m, vec_p scratch);                                        /* cvl.h:655 */
unsigned int mke_fov_inplace(void);                                                                  /* cvl.h:656 */
int mke_fov_scratch(int n, int m);                                                                   /* cvl.h:657 */
void len_fos(vec_p l, vec_p sd, int n, int m, vec_p scratch);                                        /* cvl.h:658 */
int len_fos_scratch(int n, int m);                                                                   /* cvl.h:659 */
unsigned int len_fos_inplace(void);                                                                  /* cvl.h:660 */
vec_p alo_foz(int size);                                                                             /* cvl.h:661 */
void fre_fov(vec_p pointer);                                                                         /* cvl.h:662 */
void mov_fov(vec_p d, vec_p s, int size, vec_p scratch);                                             /* cvl.h:663 */
int mov_fov_scratch(int size);                                                                       /* cvl.h:664 */
vec_p add_fov(vec_p v, int a);                                                                       /* cvl.h:665 */
int sub_fov(vec_p v1, vec_p v2);                                                                     /* cvl.h:666 */
cvl_bool eql_fov(vec_p v1, vec_p v2);                                                                /* cvl.h:667 */
int cmp_fov(vec_p v1, vec_p v2);                                                                     /* cvl.h:668 */
void v2c_fuz(int *d, vec_p s, int len, vec_p scratch);                                               /* cvl.h:669 */
int v2c_fuz_scratch(int len);                                                                        /* cvl.h:670 */
unsigned int v2c_fuz_inplace(void);                                                                  /* cvl.h:671 */
void v2c_fub(cvl_bool *d, vec_p s, int len, vec_p scratch);                                          /* cvl.h:672 */
int v2c_fub_scratch(int len);                                                                        /* cvl.h:673 */
unsigned int v2c_fub_inplace(void);                                                                  /* cvl.h:674 */
void v2c_fud(double *d, vec_p s, int len, vec_p scratch);                                            /* cvl.h:675 */
int v2c_fud_scratch(int len);                                                                        /* cvl.h:676 */
unsigned int v2c_fud_inplace(void);                                                                  /* cvl.h:677 */
void c2v_fuz(vec_p d, int *s, int len, vec_p scratch);                                               /* cvl.h:678 */
int c2v_fuz_scratch(int len);                                                                        /* cvl.h:679 */
unsigned int c2v_fuz_inplace(void);                                                                  /* cvl.h:680 */
void c2v_fub(vec_p d, cvl_bool *s, int len, vec_p scratch);                                          /* cvl.h:681 */
int c2v_fub_scratch(int len);                                                                        /* cvl.h:682 */
unsigned int c2v_fub_inplace(void);                                                                  /* cvl.h:683 */
void c2v_fud(vec_p d, double *s, int len, vec_p scratch);                                            /* cvl.h:684 */
int c2v_fud_scratch(int len);                                                                        /* cvl.h:685 */
unsigned int c2v_fud_inplace(void);                                                                  /* cvl.h:686 */

/* Library functions: index, pack, rank (nesl/cvl/serial/library.c, rank.c; CUDA CVL
 * nesl/cvl/cuda/library.c:21-193, rank.c:23-100). */
void ind_luz(vec_p d, int init, int stride, int count, vec_p scratch);                               /* cvl.h:687 */
int ind_luz_scratch(int len);                                                                        /* cvl.h:688 */
unsigned int ind_luz_inplace(void);                                                                  /* cvl.h:689 */
void ind_lez(vec_p d, vec_p init, vec_p stride, vec_p dest_segd, int vec_len, int seg_count, vec_p scratch); /* cvl.h:690 */
int ind_lez_scratch(int vec_len, int seg_len);                                                       /* cvl.h:691 */
unsigned int ind_lez_inplace(void);                                                                  /* cvl.h:692 */
int pk1_luv(vec_p f, int len, vec_p scratch);                                                        /* cvl.h:693 */
int pk1_luv_scratch(int len);                                                                        /* cvl.h:694 */
unsigned int pk1_luv_inplace(void);                                                                  /* cvl.h:695 */
void pk2_luz(vec_p d, vec_p s, vec_p f, int src_len, int dest_len, vec_p scratch);                   /* cvl.h:696 */
int pk2_luz_scratch(int len);                                                                        /* cvl.h:697 */
unsigned int pk2_luz_inplace(void);                                                                  /* cvl.h:698 */
void pk2_lub(vec_p d, vec_p s, vec_p f, int src_len, int dest_len, vec_p scratch);                   /* cvl.h:699 */
int pk2_lub_scratch(int len);                                                                        /* cvl.h:700 */
unsigned int pk2_lub_inplace(void);                                                                  /* cvl.h:701 */
void pk2_lud(vec_p d, vec_p s, vec_p f, int src_len, int dest_len, vec_p scratch);                   /* cvl.h:702 */
int pk2_lud_scratch(int len);                                                                        /* cvl.h:703 */
unsigned int pk2_lud_inplace(void);                                                                  /* cvl.h:704 */
void pk1_lev(vec_p ds, vec_p f, vec_p sd, int n, int m, vec_p scratch);                              /* cvl.h:705 */
int pk1_lev_scratch(int vec_len, int seg_len);                                                       /* cvl.h:706 */
unsigned int pk1_lev_inplace(void);                                                                  /* cvl.h:707 */
void pk2_lez(vec_p d, vec_p s, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:708 */
int pk2_lez_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:709 */
unsigned int pk2_lez_inplace(void);                                                                  /* cvl.h:710 */
void pk2_leb(vec_p d, vec_p s, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:711 */
int pk2_leb_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:712 */
unsigned int pk2_leb_inplace(void);                                                                  /* cvl.h:713 */
void pk2_led(vec_p d, vec_p s, vec_p f, vec_p sd_s, int n_s, int m_s, vec_p sd_d, int n_d, int m_d, vec_p scratch); /* cvl.h:714 */
int pk2_led_scratch(int s_vec_len, int s_seg_len, int d_vec_len, int d_seg_len);                     /* cvl.h:715 */
unsigned int pk2_led_inplace(void);                                                                  /* cvl.h:716 */
void rku_luz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:717 */
int rku_luz_scratch(int len);                                                                        /* cvl.h:718 */
unsigned int rku_luz_inplace(void);                                                                  /* cvl.h:719 */
void rkd_luz(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:720 */
int rkd_luz_scratch(int len);                                                                        /* cvl.h:721 */
unsigned int rkd_luz_inplace(void);                                                                  /* cvl.h:722 */
void rku_lez(vec_p d, vec_p s, vec_p segd, int vec_len, int seg_count, vec_p scratch);               /* cvl.h:723 */
int rku_lez_scratch(int vec_len, int seg_count);                                                     /* cvl.h:724 */
unsigned int rku_lez_inplace(void);                                                                  /* cvl.h:725 */
void rkd_lez(vec_p d, vec_p s, vec_p segd, int vec_len, int seg_count, vec_p scratch);               /* cvl.h:726 */
int rkd_lez_scratch(int vec_len, int seg_count);                                                     /* cvl.h:727 */
unsigned int rkd_lez_inplace(void);                                                                  /* cvl.h:728 */
void rku_lud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:729 */
int rku_lud_scratch(int len);                                                                        /* cvl.h:730 */
unsigned int rku_lud_inplace(void);                                                                  /* cvl.h:731 */
void rkd_lud(vec_p d, vec_p s, int len, vec_p scratch);                                              /* cvl.h:732 */
int rkd_lud_scratch(int len);                                                                        /* cvl.h:733 */
unsigned int rkd_lud_inplace(void);                                                                  /* cvl.h:734 */
void rku_led(vec_p d, vec_p s, vec_p segd, int vec_len, int seg_count, vec_p scratch);               /* cvl.h:735 */
int rku_led_scratch(int vec_len, int seg_count);                                                     /* cvl.h:736 */
unsigned int rku_led_inplace(void);                                                                  /* cvl.h:737 */
void rkd_led(vec_p d, vec_p s, vec_p segd, int vec_len, int seg_count, vec_p scratch);               /* cvl.h:738 */
int rkd_led_scratch(int vec_len, int seg_count);                                                     /* cvl.h:739 */
unsigned int rkd_led_inplace(void);                                                                  /* cvl.h:740 */

/* RAND seed (nesl/cvl/serial/facilt.c:292-311). */
void rnd_foz(int seed);                                                                              /* cvl.h:741 */

/* ------------------------------------------------------------------------
 * Extensions (no counterpart in cvl.h).
 * ---------------------------------------------------------------------- */
/* Error state: the first error since the last clear (0 = none) and its text.
 * Replaces the reference CUDA CVL's abort-on-error cutilSafeCall
 * (nesl/cvl/cuda/facilities.c:10). */
int gcvl_last_error(void);
const char *gcvl_error_string(void);
void gcvl_clear_error(void);
/* Drain the library stream; fold the device status word (bounded waits that
 * gave up) into the error state; return the error code. */
int gcvl_sync(void);
/* The library stream (a cudaStream_t); set NULL to restore the library's own. */
void *gcvl_get_stream(void);
void gcvl_set_stream(void *stream);
/* A new non-blocking stream on the library's device (NULL on failure), and
 * its release.  No counterpart in the reference, whose CVL has one implicit
 * stream: two streams let transfers of one piece of a vector overlap the
 * kernels of another. */
void *gcvl_stream_create(void);
void gcvl_stream_destroy(void *stream);
int gcvl_sm_count(void);
int gcvl_device(void);
/* Iteration limit of every bounded device wait (failure-detection tests). */
void gcvl_set_spin_limit(int iters);
int gcvl_get_spin_limit(void);
/* A device wait on a flag nothing sets, bounded by `limit` iterations;
 * returns the resulting error code (3 = timeout detected). */
int gcvl_selftest_timeout(int limit);
/* CUDA events on the library stream, for timing. */
void *gcvl_event_create(void);
void gcvl_event_record(void *event);
float gcvl_event_elapsed_ms(void *start, void *stop);
void gcvl_event_destroy(void *event);
/* Make later work on the library stream wait for the event's last record
 * (on any stream).  No counterpart in the reference (one implicit stream). */
void gcvl_stream_wait_event(void *event);
/* Pinned host memory and asynchronous transfers on the library stream. */
void *gcvl_host_alloc(size_t bytes);
void gcvl_host_free(void *p);
void gcvl_h2d_async(vec_p d, const void *s, size_t bytes);
void gcvl_d2h_async(void *d, vec_p s, size_t bytes);
/* Kernels launched by this library so far (all entry points). */
unsigned long long gcvl_launch_count(void);
/* Seeded synthetic vector on the device (benchmark inputs); element i
 * depends only on (seed, i).  kind 0: int32 uniform over all values,
 * 1: float64 N(0,1), 2: cvl_bool Bernoulli(a), 3: int32 uniform in [0, b). */
void gcvl_fill_random(vec_p d, long n, int kind, unsigned long long seed, double a, int b);
/* CUDA graphs over library calls: calls issued between gcvl_graph_begin and
 * gcvl_graph_end are captured from the library stream into one executable
 * graph (returned) instead of running.  Captured calls must not synchronise
 * (no *_ru*, ext_vu*, rep_vu*, pk1_luv, c2v_fu*, v2c_fu*) and must be given
 * scratch.  gcvl_graph_launch replays it on the library stream.  A captured
 * rnd_wuz draws from the generator state at capture time on every replay. */
int gcvl_graph_begin(void);
void *gcvl_graph_end(void);
int gcvl_graph_launch(void *graph);
void gcvl_graph_destroy(void *graph);
/* add_ruz with the sum left in device memory at d[0] (no synchronisation),
 * for sequences captured in a graph. */
void gcvl_add_ruz_dev(vec_p d, vec_p s, int len, vec_p scratch);
int gcvl_add_ruz_dev_scratch(int len);
/* The per-vector CVL call sequence of the batched benchmark (one MAKE_SEGDES,
 * +_SCAN, DIST, >, PACK, DIST, RAND, BPERMUTE sequence per vector, with the
 * PACK length read back to the host each time, as vinterp does).  Returns 0
 * or a GCVL error code. */
int gcvl_pipeline_percall(int is_double, vec_p x, const int *seg_lens_host, const int *nseg_of,
                          const int *len_of, int nvec, vec_p y, vec_p f, vec_p p, vec_p newlens,
                          vec_p bnd, vec_p idx, vec_p g, vec_p zeros, vec_p lens_dev, vec_p sd,
                          vec_p sd2, vec_p work, unsigned seed);
/* Segmented exclusive +-scan of float64 (add_sed) that allocates nothing.
 * No counterpart in the reference.  For callers that may not allocate device
 * memory: embedders whose device memory all belongs to their own pool, and
 * runtimes that forbid allocation after start-up (an allocation can
 * synchronise the device or fail when the caller cannot handle it).  Same
 * arguments and results as add_sed minus the scratch vector: the look-back
 * scratch is a fixed array inside the library, sized for
 * n <= gcvl_add_sed_noalloc_max_n() (2^28 elements; 2,097,664 bytes = 2.0 MiB,
 * held on every GPU that loads the library until exit).  Larger n is
 * rejected with GCVL error 5 (range) and nothing runs.  The first call on a
 * device looks up the array's device address there (kept until exit, so no
 * call may follow a cudaDeviceReset); make that first call before any
 * stream capture.  The library's first-use set-up is not run; the call uses
 * the library stream if that exists, else the legacy default stream.  Calls
 * share the array: calls that overlap on the GPU race.  Returns 0, or a GCVL
 * error code when the call could not be issued; a bounded device wait that
 * gave up is reported by the next gcvl_sync (error 3), as for every other
 * call. */
int gcvl_add_sed_noalloc(vec_p d, vec_p s, vec_p sd, int n, int m);
long gcvl_add_sed_noalloc_max_n(void);
/* Kernel variants of the segmented scans, reductions and ranks (no
 * counterpart in the reference; they stand in for the entry points named by
 * `prim`: add_sez, add_sed, max_sez, max_sed, add_rez, add_red, max_rez,
 * max_red, rku_lez, rku_led, rkd_lez, rkd_led, with those functions'
 * arguments).  Variant 0 is the default tile kernel; 1 and 2 give each
 * segment to one CTA (2048- and 512-element chunks), 3 and 4 to one warp
 * (256- and 64-element chunks); 5 ranks each segment in one CTA's shared
 * memory and needs every segment to hold at most 2048 elements.  Integer,
 * min/max and rank results are identical for every variant; float64 sums
 * agree within the library's float64 tolerance.  gcvl_run_variant returns 0
 * or a GCVL error code (5: unknown primitive or variant). */
int gcvl_variant_count(void);
int gcvl_variant_valid(const char *prim, int variant, int max_segment_length);
int gcvl_variant_scratch(const char *prim, int n, int m);
int gcvl_run_variant(const char *prim, int variant, vec_p d, vec_p s, vec_p sd, int n, int m,
                     vec_p scratch);
/* The learned dispatcher (no counterpart in the reference).  A features row
 * is 16 floats describing a call (sizes, length statistics, a length
 * histogram, the kind of primitive and element type) followed by 8 floats,
 * 1 for each variant valid for it.  The model is an FP32 MLP (16 -> 64 ->
 * 64 -> 8, ReLU, softmax over the valid variants) of gcvl_mlp_param_count()
 * floats, trained by gcvl_mlp_train (Adam, soft targets T of N x 8 floats;
 * params, moments -- 2P floats, zero at first -- and X, T, loss on the
 * device) and evaluated by gcvl_mlp_infer (one class per row into cls_dev).
 * gcvl_dispatch_set_model installs a model (P floats of host memory, NULL to
 * remove it); gcvl_auto_run then runs the variant it picks for prim
 * (gcvl_dispatch_choice: synchronises once per new (prim, descriptor
 * address, n, m), then uses a cache).  Without a model the default kernel
 * runs.  Return 0 or a GCVL error code. */
int gcvl_mlp_param_count(void);
int gcvl_mlp_feature_stride(void);
int gcvl_mlp_classes(void);
int gcvl_seg_features(const char *prim, vec_p sd, int n, int m, float *out_dev);
int gcvl_mlp_train(float *params, float *moments, const float *X, const float *T, int N, int epochs, int batch,
                   float lr, unsigned seed, int step0, float *loss_dev);
int gcvl_mlp_infer(const float *params, const float *X, int N, int *cls_dev);
int gcvl_dispatch_set_model(const float *params_host);
int gcvl_dispatch_choice(const char *prim, vec_p sd, int n, int m);
int gcvl_auto_run(const char *prim, vec_p d, vec_p s, vec_p sd, int n, int m, vec_p scratch);
/* Sparse matrix-vector product in one pass (no counterpart in the
 * reference): y[r] = sum of vals[k] * x[cols[k]] over row r, rows given by
 * the segment descriptor sd (rows segments over nnz elements).  The same
 * products as BPERMUTE, * and +_REDUCE on FLOAT vectors compute, summed per
 * row (float64 sums within the library's tolerance); empty rows give 0.
 * Scratch: gcvl_spmv_csr_scratch(nnz, rows) units. */
void gcvl_spmv_csr(vec_p y, vec_p vals, vec_p cols, vec_p x, vec_p sd, int nnz, int rows, vec_p scratch);
int gcvl_spmv_csr_scratch(int nnz, int rows);
/* The 48-bit lrand48 state behind rnd_wuz. */
unsigned long long gcvl_rand_state(void);
void gcvl_set_rand_state(unsigned long long state);

#ifdef __cplusplus
}
#endif

#endif /* CVL_GB300_H */
