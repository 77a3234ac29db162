// Test infrastructure only (the oracle side of the parity tests): a translation
// unit that compiles the reference codec (src/vc/vc.c, included by the build
// recipe oracle/Makefile from the reference checkout) together with a handful of
// exported entry points that reach its file-static per-atom kernels. Nothing in
// the product links or loads this file's output.
//
// Every exported function below is a thin call into the reference's own code:
//   refshim_tables      -> build_tables()            src/vc/vc.c:266-290
//   refshim_fdct        -> atom_dct_fwd()            src/vc/vc.c:212-218
//   refshim_idct        -> atom_dct_inv()            src/vc/vc.c:219-229
//   refshim_quantize    -> quantize()                src/vc/vc.c:293-306
//   refshim_dequantize  -> dequantize()/dq_build()   src/vc/vc.c:314-338
//   refshim_encode_atom -> encode_atom()             src/vc/vc.c:595-622
//   refshim_decode_atom -> decode_atom_payload()     src/vc/vc.c:625-633
//   refshim_enc_levels  -> enc_atom_coefs()+flush    src/vc/vc.c:528-544,399
//   refshim_dec_levels  -> dec_atom_coefs()          src/vc/vc.c:545-560
// The public vc_* API (writer, reader, test hooks) is exported unchanged.
#pragma GCC visibility push(default)
#include "vc.c"
#pragma GCC visibility pop

#define SHIM __attribute__((visibility("default")))

SHIM void refshim_tables(int32_t *cmat /*32*32*/, float *step /*32768*/,
                         uint16_t *scan /*32768*/) {
    build_tables();
    if (cmat) memcpy(cmat, CMATA, sizeof CMATA);
    if (step) memcpy(step, g_step, sizeof g_step);
    if (scan) memcpy(scan, g_scan, sizeof g_scan);
}

SHIM void refshim_fdct(const uint8_t *vox, int32_t dc, int32_t *coef) {
    build_tables();
    atom_dct_fwd(vox, dc, coef);
}

SHIM void refshim_idct(const int32_t *coef, int32_t dc, uint8_t *vox) {
    build_tables();
    atom_dct_inv(coef, dc, vox);
}

SHIM void refshim_quantize(const int32_t *coef, float base_q, int16_t *q) {
    build_tables();
    quantize(coef, base_q, q);
}

SHIM void refshim_dequantize(const int16_t *q, float base_q, int32_t *coef) {
    build_tables();
    dequantize(q, base_q, coef);
}

SHIM void refshim_dq_tables(float base_q, int32_t *dq_step, int32_t *dq_bias) {
    build_tables();
    dq_build(base_q);
    memcpy(dq_step, g_dq_step, sizeof g_dq_step);
    memcpy(dq_bias, g_dq_bias, sizeof g_dq_bias);
}

// Returns the payload length ([dc][rc bytes]); 0 for an all-zero atom.
SHIM uint32_t refshim_encode_atom(const uint8_t *vox, float base_q, uint8_t *out,
                                  uint32_t cap, int *is_zero, uint8_t *dc) {
    build_tables();
    bbuf b = {0};
    uint32_t len = encode_atom(vox, base_q, &b, is_zero, dc);
    if (len > cap) len = 0;
    else if (len) memcpy(out, b.p, len);
    free(b.p);
    return len;
}

SHIM void refshim_decode_atom(const uint8_t *pay, uint32_t len, float base_q, uint8_t *vox) {
    build_tables();
    decode_atom_payload(pay, len, base_q, vox);
}

// Range-code raster-order levels exactly as encode_atom does after quantize.
SHIM uint32_t refshim_enc_levels(const int16_t *q, uint8_t *out, uint32_t cap) {
    build_tables();
    static _Thread_local uint8_t scratch[A3 * 4 + 64];
    rc_enc e; enc_init(&e, scratch, sizeof scratch);
    enc_atom_coefs(&e, q);
    enc_flush(&e);
    if (e.len > cap) return 0;
    memcpy(out, scratch, e.len);
    return (uint32_t)e.len;
}

SHIM void refshim_dec_levels(const uint8_t *buf, uint32_t len, int16_t *q) {
    build_tables();
    rc_dec d; dec_init(&d, buf, len);
    dec_atom_coefs(&d, q);
}
