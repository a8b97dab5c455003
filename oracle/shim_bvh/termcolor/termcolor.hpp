/* stand-in for the termcolor submodule, which the builder does not use (TEST INFRASTRUCTURE) */
#pragma once
