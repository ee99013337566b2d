set output "hist_group2_MOTIF00008.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-33.4829:10.5355]
set yrange [0:130375]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00008.dat" using 1:2 title 'MOTIF00008 (group2)' with boxes
