/* empty stand-in: the oracle harness never hashes (ORACLE / TEST INFRASTRUCTURE ONLY) */
#pragma once
