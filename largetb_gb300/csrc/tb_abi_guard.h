// tb_abi_guard.h -- exception guard for the C-ABI entry points.
#pragma once

#include <new>

// No C++ exception may cross the C-ABI: every int-returning extern "C" entry
// point runs its body inside TB_ABI_TRY ... TB_ABI_CATCH, which turns a host
// allocation failure into TB_ERR_OUT_OF_MEMORY and any other exception into
// TB_ERR_INVALID_ARG.
#define TB_ABI_TRY try {
#define TB_ABI_CATCH                          \
    }                                         \
    catch (const std::bad_alloc &)            \
    {                                         \
        return TB_ERR_OUT_OF_MEMORY;          \
    }                                         \
    catch (...)                               \
    {                                         \
        return TB_ERR_INVALID_ARG;            \
    }
