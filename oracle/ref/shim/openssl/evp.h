/* Stand-in for <openssl/evp.h>: declares the two opaque types the
 * reference's CryptoDigest.h names.  The oracle harness never hashes.
 * ORACLE / TEST INFRASTRUCTURE ONLY. */
#pragma once
typedef struct qhg_oracle_evp_md_ctx EVP_MD_CTX;
typedef struct qhg_oracle_evp_md EVP_MD;
