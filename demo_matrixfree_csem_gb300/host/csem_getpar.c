/* key=value flag table with the semantics of the reference's CWP getpar
 * (cstd.c:936-1436), re-implemented for the GB300 host driver.
 *
 *  - argv[1..] tokens containing '=' are "name=value" parameters;
 *  - "par=file" (the last such token) names a parameter file whose whitespace-
 *    separated tokens (quotes suppress splitting) are tabulated BEFORE the command
 *    line, so the command line overrides the file (cstd.c:1254-1417);
 *  - a query returns the LAST occurrence of a name (cstd.c:1235-1252);
 *  - vectors are comma separated; the value count is commas+1 (cstd.c:1210-1227);
 *  - integers via strtol, floats via strtod rounded to float (cstd.c:1488-1516).
 */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../../include/csem_host.h"

typedef struct {
  char *name;
  char *value;
} csem_par_t;

static csem_par_t *g_tab = NULL;
static int g_ntab = 0;

static void tab_clear(void)
{
  for (int i = 0; i < g_ntab; i++) free(g_tab[i].name);
  free(g_tab);
  g_tab = NULL;
  g_ntab = 0;
}

static void tab_add(const char *tok)
{
  const char *eq = strchr(tok, '=');
  if (!eq) return;
  size_t len = strlen(tok);
  char *copy = (char *)malloc(len + 1);
  memcpy(copy, tok, len + 1);
  copy[eq - tok] = '\0';
  g_tab = (csem_par_t *)realloc(g_tab, sizeof(csem_par_t) * (size_t)(g_ntab + 1));
  g_tab[g_ntab].name = copy;
  g_tab[g_ntab].value = copy + (eq - tok) + 1;
  g_ntab++;
}

static void tab_parfile(const char *path)
{
  FILE *fp = fopen(path, "r");
  if (!fp) return;
  fseek(fp, 0, SEEK_END);
  long len = ftell(fp);
  rewind(fp);
  char *buf = (char *)malloc((size_t)len + 1);
  size_t nread = fread(buf, 1, (size_t)len, fp);
  fclose(fp);
  buf[nread] = '\0';
  int quoted = 0;
  size_t start = (size_t)-1;
  for (size_t i = 0; i <= nread; i++) {
    char c = (char)(buf[i] & 0x7F);
    buf[i] = c;
    int end = (i == nread);
    if (start == (size_t)-1) {
      if (!end && isgraph((unsigned char)c)) start = i;
    } else if (end || (!quoted && isspace((unsigned char)c))) {
      buf[i] = '\0';
      tab_add(buf + start);
      start = (size_t)-1;
    }
    if (!end && (c == '\'' || c == '"')) quoted = !quoted;
  }
  free(buf);
}

void csem_initargs(int argc, char **argv)
{
  tab_clear();
  const char *pf = NULL;
  for (int i = argc - 1; i > 0; i--) {
    if (!strncmp(argv[i], "par=", 4) && strlen(argv[i]) != 4) {
      pf = argv[i] + 4;
      break;
    }
  }
  if (pf) tab_parfile(pf);
  for (int i = 1; i < argc; i++) tab_add(argv[i]);
}

static const char *lookup(const char *name)
{
  for (int i = g_ntab - 1; i >= 0; i--)
    if (!strcmp(g_tab[i].name, name)) return g_tab[i].value;
  return NULL;
}

int csem_countparval(const char *name)
{
  const char *v = lookup(name);
  if (!v) return 0;
  int n = 1;
  for (; *v; v++)
    if (*v == ',') n++;
  return n;
}

/* advance past the next comma; returns NULL at the end of the string */
static const char *next_field(const char *s)
{
  while (*s && *s != ',') s++;
  return *s == ',' ? s + 1 : NULL;
}

int csem_getparint(const char *name, int *p)
{
  const char *v = lookup(name);
  if (!v) return 0;
  int n = 0;
  for (const char *s = v; s && *s; s = next_field(s)) p[n++] = (int)strtol(s, NULL, 10);
  return n;
}

int csem_getparfloat(const char *name, float *p)
{
  const char *v = lookup(name);
  if (!v) return 0;
  int n = 0;
  for (const char *s = v; s && *s; s = next_field(s)) {
    double d = strtod(s, NULL);
    p[n++] = (float)d;
  }
  return n;
}

int csem_getpardouble(const char *name, double *p)
{
  const char *v = lookup(name);
  if (!v) return 0;
  int n = 0;
  for (const char *s = v; s && *s; s = next_field(s)) p[n++] = strtod(s, NULL);
  return n;
}

int csem_getparstring(const char *name, char **p)
{
  const char *v = lookup(name);
  if (!v) return 0;
  *p = (char *)v;
  return 1;
}

int csem_getparstringarray(const char *name, char **p)
{
  const char *v = lookup(name);
  if (!v) return 0;
  int n = 0;
  for (const char *s = v; s && *s; s = next_field(s)) {
    size_t len = 0;
    while (s[len] && s[len] != ',') len++;
    char *f = (char *)malloc(len + 1);
    memcpy(f, s, len);
    f[len] = '\0';
    p[n++] = f;
  }
  return n;
}
