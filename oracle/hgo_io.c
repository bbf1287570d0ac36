/*
 * hgo_io.c — CPU oracle for table ingest: readCSV / loadCSV / getField /
 * loadItem (src/horseir/v3/backend/h_io.cc:50-188) and serializeV /
 * readSerializeV (h_io.cc:626-772).
 *
 * THIS IS TEST INFRASTRUCTURE, NOT THE PRODUCT (see hgo.h).  It restates the
 * reference's loaders with the same C library conversions (strtol, strtof,
 * strtod, sscanf) and returns an error where the reference's behaviour is
 * undefined:
 *   - a line whose loaded field count differs from numCols (the reference
 *     writes past its columns or leaves values unset): E_GENERAL;
 *   - a line of LINE_MAX_CHAR or more characters with its newline (fgets
 *     would split it into two rows): E_GENERAL;
 *   - a NUL byte in a line: E_GENERAL;
 *   - a date field that "%d-%d-%d" does not read completely: E_GENERAL;
 *   - hexadecimal floats and nan(...) payloads: E_NOT_IMPL.
 */
#include "hgo.h"
#include <ctype.h>

C LINE_SEP = '|';        /* h_io.cc:9 */
B LINE_HEADER = false;   /* h_io.cc:11 */
L LINE_MAX_CHAR = 1024;  /* h_io.cc:8 */

static int skip_set(char c) { R c == ' ' || c == '\r' || c == '\n'; }

/* trimLeft / trimRight (h_io.cc:190-206): ' ' on the left, ' ', '\r', '\n' on the right */
static void trim_span(const char *s, L *b, L *e) {
    while (*b < *e && s[*b] == ' ') (*b)++;
    while (*e > *b && skip_set(s[*e - 1])) (*e)--;
}

static int hexnan(const char *s) {  /* inputs whose strtod result the GPU reader does not accept */
    while (*s && isspace((unsigned char)*s)) s++;
    if (*s == '+' || *s == '-') s++;
    if (s[0] == '0' && (s[1] == 'x' || s[1] == 'X') &&
        (isxdigit((unsigned char)s[2]) || (s[2] == '.' && isxdigit((unsigned char)s[3])))) R 1;
    if ((s[0] == 'n' || s[0] == 'N') && (s[1] == 'a' || s[1] == 'A') && (s[2] == 'n' || s[2] == 'N') && s[3] == '(') R 1;
    R 0;
}

/* loadItem (h_io.cc:164-181) */
static I load_item(V x, L k, L typ, S s) {
    switch (typ) {
    case H_B: sB(x)[k] = atoi(s); break;
    case H_J: sJ(x)[k] = atoi(s); break;
    case H_H: sH(x)[k] = atoi(s); break;
    case H_I: sI(x)[k] = atoi(s); break;
    case H_L: sL(x)[k] = atol(s); break;
    case H_F: if (hexnan(s)) R E_NOT_IMPL; sF(x)[k] = strtof(s, NULL); break;
    case H_E: if (hexnan(s)) R E_NOT_IMPL; sE(x)[k] = atof(s); break;
    case H_C: sC(x)[k] = s[0]; break;
    case H_Q: sL(x)[k] = getSymbol(s); break;
    case H_S: { S t = hgo_alloc((L)strlen(s) + 1); strcpy(t, s); ((S *)vg(x))[k] = t; } break;
    case H_D: {
        int a, b, c;
        if (sscanf(s, "%d-%d-%d", &a, &b, &c) != 3) R E_GENERAL;
        sI(x)[k] = (I)((unsigned)a * 10000u + (unsigned)b * 100u + (unsigned)c);
    } break;
    default: R E_NOT_IMPL;
    }
    R 0;
}

/* readCSV (h_io.cc:50-71) with loadCSV / getField (:90-143) */
I hgoReadCSV(V z, S fileName, L numCols, L *types, Q *symList) {
    FILE *fp = fopen(fileName, "rb");
    if (!fp) R E_GENERAL;
    fseek(fp, 0, SEEK_END);
    L size = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    char *buf = (char *)malloc((size_t)size + 1);
    if ((L)fread(buf, 1, (size_t)size, fp) != size) { fclose(fp); free(buf); R E_GENERAL; }
    fclose(fp);
    /* lines as fgets returns them: up to and including each '\n' */
    L nlines = 0;
    for (L i = 0; i < size; i++) nlines += buf[i] == '\n';
    if (size > 0 && buf[size - 1] != '\n') nlines++;
    L *ls = (L *)malloc(sizeof(L) * (size_t)(nlines + 1)), *le = (L *)malloc(sizeof(L) * (size_t)(nlines + 1));
    L nl = 0, st = 0;
    for (L i = 0; i < size; i++)
        if (buf[i] == '\n') { ls[nl] = st; le[nl] = i; nl++; st = i + 1; }
    if (st < size) { ls[nl] = st; le[nl] = size; nl++; }
    L first = (LINE_HEADER && nl > 0) ? 1 : 0, rows = nl - first;
    V x = z;
    initV(x, H_A, 2);
    x->a = (A)hgo_alloc(sizeof(A0));
    x->a->row = rows; x->a->col = numCols; x->a->fkey = NULL;
    V keys = vV(x, 0), vals = vV(x, 1);
    initV(keys, H_Q, numCols);
    for (L j = 0; j < numCols; j++) sL(keys)[j] = symList[j];
    initV(vals, H_G, numCols);
    for (L j = 0; j < numCols; j++) {
        if (types[j] == H_S) initV(vV(vals, j), H_S, rows);
        else initV(vV(vals, j), (I)types[j], rows);
    }
    char *tmp = (char *)malloc((size_t)LINE_MAX_CHAR + 1);
    I rc = 0;
    for (L r = 0; r < rows && !rc; r++) {
        L li = r + first, b = ls[li], e = le[li];
        L with_nl = (li < nl - 1 || (size > 0 && buf[size - 1] == '\n')) ? 1 : 0;
        if (e - b + with_nl > LINE_MAX_CHAR - 1) { rc = E_GENERAL; break; }
        for (L i = b; i < e; i++) if (!buf[i]) { rc = E_GENERAL; break; }
        if (rc) break;
        trim_span(buf, &b, &e);
        L loaded = 0, fb = b;
        for (L i = b; i <= e && !rc; i++) {
            int at_sep = i < e && buf[i] == LINE_SEP;
            int remainder = i == e && LINE_SEP == ' ';
            if (!at_sep && !remainder) continue;
            if (loaded >= numCols) { rc = E_GENERAL; break; }
            L f0 = fb, f1 = i;
            trim_span(buf, &f0, &f1);
            memcpy(tmp, buf + f0, (size_t)(f1 - f0));
            tmp[f1 - f0] = 0;
            rc = load_item(vV(vals, loaded), r, types[loaded], tmp);
            loaded++;
            fb = i + 1;
        }
        if (!rc && loaded != numCols) rc = E_GENERAL;
    }
    free(tmp); free(ls); free(le); free(buf);
    R rc;
}

/* ------------------------------------------------------------ serialization */
static int raw_payload(I t) {
    R hgo_is_real(t) || t == H_C || t == H_X || (t >= H_M && t <= H_T);
}

/* serializeV (h_io.cc:672-697) */
I hgoWriteSerialized(V x, FILE *fp) {
    if (fwrite(x, sizeof(V0), 1, fp) != 1) R E_GENERAL;
    I t = vp(x);
    L n = vn(x);
    if (raw_payload(t)) {
        L nb = getTypeSize(t, n);
        if (t == H_C) {  /* the characters, then a NUL */
            if (n && fwrite(vg(x), 1, (size_t)n, fp) != (size_t)n) R E_GENERAL;
            if (fputc(0, fp) == EOF) R E_GENERAL;
            R 0;
        }
        R (nb && fwrite(vg(x), 1, (size_t)nb, fp) != (size_t)nb) ? E_GENERAL : 0;
    }
    switch (t) {
    case H_Q:
        for (L i = 0; i < n; i++) { L k = (L)strlen(getSymbolStr(sL(x)[i])); fwrite(&k, 8, 1, fp); }
        for (L i = 0; i < n; i++) { S s = getSymbolStr(sL(x)[i]); fwrite(s, 1, strlen(s) + 1, fp); }
        R 0;
    case H_S:
        for (L i = 0; i < n; i++) { L k = (L)strlen(((S *)vg(x))[i]); fwrite(&k, 8, 1, fp); }
        for (L i = 0; i < n; i++) { S s = ((S *)vg(x))[i]; fwrite(s, 1, strlen(s) + 1, fp); }
        R 0;
    case H_G:
        for (L i = 0; i < n; i++) CHECKE(hgoWriteSerialized(vV(x, i), fp));
        R 0;
    case H_A: {
        A0 a = {0, 0, NULL};
        if (x->a) a = *x->a;
        a.fkey = NULL;
        if (fwrite(&a, sizeof(A0), 1, fp) != 1) R E_GENERAL;
        CHECKE(hgoWriteSerialized(vV(x, 0), fp));
        R hgoWriteSerialized(vV(x, 1), fp);
    }
    default: R E_NOT_IMPL;
    }
}

/* readSerializeV (h_io.cc:748-772) */
I hgoReadSerialized(V x, FILE *fp) {
    V0 hdr;
    if (fread(&hdr, sizeof(V0), 1, fp) != 1) R E_GENERAL;
    I t = hdr.typ;
    L n = hdr.len;
    if (n < 0) R E_GENERAL;
    if (raw_payload(t)) {
        initV(x, t, n);
        if (n <= 1) x->i64 = hdr.i64;
        L nb = getTypeSize(t, n);
        R (nb && fread(vg(x), 1, (size_t)nb, fp) != (size_t)nb) ? E_GENERAL : 0;
    }
    switch (t) {
    case H_Q: {
        initV(x, H_Q, n);
        L *sz = (L *)malloc(sizeof(L) * (size_t)(n > 0 ? n : 1));
        if (n && fread(sz, 8, (size_t)n, fp) != (size_t)n) { free(sz); R E_GENERAL; }
        for (L i = 0; i < n; i++) {
            S tmp = (S)malloc((size_t)sz[i] + 1);
            if (fread(tmp, 1, (size_t)sz[i] + 1, fp) != (size_t)sz[i] + 1) { free(tmp); free(sz); R E_GENERAL; }
            sL(x)[i] = getSymbol(tmp);
            free(tmp);
        }
        free(sz);
        R 0;
    }
    case H_S: {
        initV(x, H_S, n);
        if (n <= 1) x->g = (G)&x->b;
        L *sz = (L *)malloc(sizeof(L) * (size_t)(n > 0 ? n : 1));
        if (n && fread(sz, 8, (size_t)n, fp) != (size_t)n) { free(sz); R E_GENERAL; }
        for (L i = 0; i < n; i++) {
            S s = hgo_alloc(sz[i] + 1);
            if (fread(s, 1, (size_t)sz[i] + 1, fp) != (size_t)sz[i] + 1) { free(sz); R E_GENERAL; }
            ((S *)vg(x))[i] = s;
        }
        free(sz);
        R 0;
    }
    case H_G:
        initV(x, H_G, n);
        for (L i = 0; i < n; i++) CHECKE(hgoReadSerialized(vV(x, i), fp));
        R 0;
    case H_A:
        if (n != 2) R E_GENERAL;
        initV(x, H_A, 2);
        x->a = (A)hgo_alloc(sizeof(A0));
        if (fread(x->a, sizeof(A0), 1, fp) != 1) R E_GENERAL;
        x->a->fkey = NULL;
        CHECKE(hgoReadSerialized(vV(x, 0), fp));
        R hgoReadSerialized(vV(x, 1), fp);
    default: R E_NOT_IMPL;
    }
}
