set output "hist_group1_MOTIF00004.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-76.2107:19.6035]
set yrange [0:161564]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00004.dat" using 1:2 title 'MOTIF00004 (group1)' with boxes
