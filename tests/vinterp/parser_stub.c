/* parser_stub.c -- stands in for vinterp's yacc/lex-generated parser in the
 * link test (tests/test_vinterp_link.py).  No lex or yacc exists on this
 * machine, so the grammar (nesl/vcode/grammar.yy, tokens.ll) cannot be
 * generated; this file supplies the globals the generated parser would
 * define, and a yyparse that reports a parse failure.  It lets the
 * interpreter's other sources compile unchanged and link against
 * libcvl_gb300.so, which is what the test checks. */
#include <stdio.h>
#include <string.h>

#include "config.h"
#include "vcode.h"
#include "parse.h"

int parse_error = 0;
char main_fn[FN_NAME_MAX];
const_union constant;
FILE *yyin;
int yylineno;
/* glibc no longer exports sys_errlist, which main.c declares */
const char *const sys_errlist[] = {"unknown error"};

int yyparse(void) {
  parse_error = 1;
  return 1;
}
