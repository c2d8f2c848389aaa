// Stand-in header (oracle pin, test infrastructure): the reference's filter
// sources include it but use nothing from it.
#pragma once
