// No optional G+Smo modules are enabled for the parity oracle build.
#pragma once
