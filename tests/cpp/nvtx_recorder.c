/* NVTX injection library for the tracing test (tests/test_tracing.py): loaded
 * by the NVTX3 headers of the library under test when NVTX_INJECTION64_PATH
 * names it, it appends one line per domain created and per domain range
 * pushed or popped to the file named by NVTX_RECORD_FILE:
 *     domain <name> | push <domain> <message> | pop <domain>
 * Only the CORE2 (domain) callbacks are replaced; everything else stays a
 * no-op. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <nvtx3/nvToolsExt.h> /* brings the injection types (nvtxDetail/nvtxTypes.h) */

#define MAX_DOMAINS 64

static FILE *rec;
static char names[MAX_DOMAINS][64];
static int ndomains;

static const char *domain_name(nvtxDomainHandle_t d) {
    const intptr_t k = (intptr_t)d - 1;
    return (k >= 0 && k < ndomains) ? names[k] : "?";
}

static nvtxDomainHandle_t NVTX_API on_create(const char *name) {
    const int k = ndomains < MAX_DOMAINS ? ndomains++ : MAX_DOMAINS - 1;
    snprintf(names[k], sizeof names[k], "%s", name ? name : "");
    if (rec) fprintf(rec, "domain %s\n", names[k]), fflush(rec);
    return (nvtxDomainHandle_t)(intptr_t)(k + 1);
}

static int NVTX_API on_push(nvtxDomainHandle_t d, const nvtxEventAttributes_t *a) {
    const char *msg = (a && a->messageType == NVTX_MESSAGE_TYPE_ASCII && a->message.ascii) ? a->message.ascii : "";
    if (rec) fprintf(rec, "push %s %s\n", domain_name(d), msg), fflush(rec);
    return 0;
}

static int NVTX_API on_pop(nvtxDomainHandle_t d) {
    if (rec) fprintf(rec, "pop %s\n", domain_name(d)), fflush(rec);
    return 0;
}

int InitializeInjectionNvtx2(NvtxGetExportTableFunc_t get_table) {
    const NvtxExportTableCallbacks *cb = (const NvtxExportTableCallbacks *)get_table(NVTX_ETID_CALLBACKS);
    NvtxFunctionTable table = 0;
    unsigned int size = 0;
    if (!cb || !cb->GetModuleFunctionTable(NVTX_CB_MODULE_CORE2, &table, &size) || !table) return 0;
    if (size <= NVTX_CBID_CORE2_DomainCreateA) return 0;
    *table[NVTX_CBID_CORE2_DomainCreateA] = (NvtxFunctionPointer)on_create;
    *table[NVTX_CBID_CORE2_DomainRangePushEx] = (NvtxFunctionPointer)on_push;
    *table[NVTX_CBID_CORE2_DomainRangePop] = (NvtxFunctionPointer)on_pop;
    if (!rec) {
        const char *path = getenv("NVTX_RECORD_FILE");
        rec = path ? fopen(path, "a") : NULL;
    }
    return 1;
}
