/*
 * No-op definitions for the QDF (HDF5) attribute helpers and the md5 digest
 * that the reference's hot-path sources reference but the oracle harness
 * never calls.  Each returns failure.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY (linked into oracle/_ref/ programs).
 */
#include <string>
#include <hdf5.h>
#include "types.h"

class CryptoDigest {
public:
    static unsigned char *md5sum_string(std::string sData, unsigned int *piDigestLen);
};

unsigned char *CryptoDigest::md5sum_string(std::string sData, unsigned int *piDigestLen) {
    (void)sData;
    if (piDigestLen != NULL) {
        *piDigestLen = 0;
    }
    return NULL;
}

int qdf_insertAttribute(hid_t hLoc, const std::string sName, const uint iNum, void *vValue, const hid_t hType) {
    (void)hLoc; (void)sName; (void)iNum; (void)vValue; (void)hType;
    return -1;
}

int qdf_extractAttribute(hid_t hLoc, const std::string sName, const uint iNum, void *vValue, const hid_t hType) {
    (void)hLoc; (void)sName; (void)iNum; (void)vValue; (void)hType;
    return -1;
}

class PolyLine;

hid_t qdf_openGroup(hid_t hGroup, const std::string sGroupName, bool bForceCheck) {
    (void)hGroup; (void)sGroupName; (void)bForceCheck;
    return -1;
}
hid_t qdf_opencreateGroup(hid_t hGroup, const std::string sGroupName, bool bForceCheck) {
    (void)hGroup; (void)sGroupName; (void)bForceCheck;
    return -1;
}
void qdf_closeGroup(hid_t hGroup) { (void)hGroup; }
void qdf_closeDataSpace(hid_t hDataSpace) { (void)hDataSpace; }
void qdf_closeDataType(hid_t hDataType) { (void)hDataType; }
void qdf_closeAttribute(hid_t hAttribute) { (void)hAttribute; }
bool qdf_link_exists(hid_t hGroup, const std::string sName) { (void)hGroup; (void)sName; return false; }
int qdf_insertSAttribute(hid_t hLoc, const std::string sName, const std::string sValue) {
    (void)hLoc; (void)sName; (void)sValue;
    return -1;
}
int qdf_insertSAttribute(hid_t hLoc, const std::string sName, const char *pValue) {
    (void)hLoc; (void)sName; (void)pValue;
    return -1;
}
int qdf_extractSAttribute(hid_t hLoc, const std::string sName, std::string &sValue) {
    (void)hLoc; (void)sName; (void)sValue;
    return -1;
}
PolyLine *qdf_createPolyLine(hid_t hSpeciesGroup, const std::string sPLParName) {
    (void)hSpeciesGroup; (void)sPLParName;
    return NULL;
}
int qdf_writePolyLine(hid_t hSpeciesGroup, PolyLine *pPL, const std::string sPLParName) {
    (void)hSpeciesGroup; (void)pPL; (void)sPLParName;
    return -1;
}
int qdf_compareDataTypes(hid_t t1, hid_t t2) { (void)t1; (void)t2; return -1; }
void qdf_closeDataSet(hid_t hDataSet) { (void)hDataSet; }
int qdf_readArray(hid_t hGroup, const std::string sName, const uint iNum, void *vData, const hid_t hType) {
    (void)hGroup; (void)sName; (void)iNum; (void)vData; (void)hType;
    return -1;
}
int qdf_writeArray(hid_t hGroup, const std::string sName, const uint iNum, void *vData, const hid_t hType) {
    (void)hGroup; (void)sName; (void)iNum; (void)vData; (void)hType;
    return -1;
}

#ifdef QHG_PHILOX_TEST_BUILD
/* the Philox test build has no WELL state to manage; these two helpers of
 * utils/WELLUtils.cpp are only reached from dump code and from Genetics
 * objects that own their generators (the harness creates neither) */
namespace WELLUtils {
    void destroyWELLs(WELL512 **pWELLs, int iNum) {
        if (pWELLs != NULL) {
            for (int i = 0; i < iNum; i++) {
                delete pWELLs[i];
            }
            delete[] pWELLs;
        }
    }
    void showStates(WELL512 **pWELL, int iNum, bool bFull) { (void)pWELL; (void)iNum; (void)bFull; }
}
#endif
