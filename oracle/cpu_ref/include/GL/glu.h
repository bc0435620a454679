// Empty: the reference names this header but calls nothing from it.
#pragma once
