/* stand-in for the termcolor submodule, which the programs do not use (TEST INFRASTRUCTURE) */
#pragma once
